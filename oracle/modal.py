"""Oracle of the modal (reduced) linear Newmark path -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this
module; the product path (opendeformer_gb300, od_modal_*) never does.

The reference's path (intergrator/linearNewmark.cpp):
  * K: HookeMaterial::generateStiffnessMatrix (material/hooke.cpp:18-60) and
    M: MechMaterial::generateMassMatrix, both scalar CSC lower triangles from
    the reference's own assembler -- taken here from the compiled reference
    (oracle/_ref, ``RefScene.linear_csc``);
  * the n_modes eigenpairs nearest zero of K phi = lambda M phi:
    EigenSolver::getEigenValVectors (core/eigensolver.cpp:8-13) calls
    ARPACK++'s ARluSymGenEig in shift-invert mode at 0 (ARPACK's implicitly
    restarted Lanczos on (K - 0 M)^-1 M with a SuperLU factorisation).  The
    reference links ARPACK, ARPACK++ 1.2 and SuperLU as Win32 binaries that
    cannot be used here; the same published algorithm is available as
    scipy.sparse.linalg.eigsh (ARPACK's dsaupd/dseupd in mode 3 with
    sigma = 0, the factorisation by SuperLU), which this module calls.  The
    eigenvectors are M-orthonormal, as ARPACK returns them.
  * the time step restated from linearNewmark.cpp:27-30 and 57-79 (every
    mode independently, the reference's operation order), the external
    forces projected as Forcer::getVirtualWorks does (forcer.cpp:80-96) and
    the accelerations set to them (linearNewmark.cpp:52-55), and the full
    order displacement sum_i d_i phi_i (getFullOrderProperties, :81-92).
"""
from __future__ import annotations

import numpy as np


def sym_from_lower_csc(pcol, rows, vals, n):
    """The full symmetric scipy matrix of a lower-triangle CSC."""
    import scipy.sparse as sp
    L = sp.csc_matrix((np.asarray(vals, np.float64), np.asarray(rows), np.asarray(pcol)), shape=(n, n))
    return (L + L.T - sp.diags(L.diagonal())).tocsc()


def reference_matrices(ref_scene, youngs, poisson):
    """K (Hooke) and M (consistent mass) of a compiled-reference scene."""
    n = ref_scene.dofs
    K = sym_from_lower_csc(*ref_scene.linear_csc("K", youngs, poisson), n)
    M = sym_from_lower_csc(*ref_scene.linear_csc("M", youngs, poisson), n)
    return K, M


def modes(K, M, n_modes, tol=0.0):
    """ARPACK shift-invert at 0 (the reference's EigenSolver call): the
    n_modes smallest eigenvalues ascending and their M-orthonormal modes as
    columns."""
    from scipy.sparse.linalg import eigsh
    lam, phi = eigsh(K, k=n_modes, M=M, sigma=0.0, which="LM", tol=tol)
    order = np.argsort(lam)
    return lam[order], phi[:, order]


class LinearNewmarkOracle:
    """LinearNewmark's reduced state and step (linearNewmark.cpp:8-79)."""

    def __init__(self, lam, phi, beta, gamma, mass_damp, stiff_damp, dt):
        self.lam = np.asarray(lam, np.float64)
        self.phi = np.asarray(phi, np.float64)           # dofs x n_modes
        r = self.lam.size
        self.d = np.zeros(r)
        self.v = np.zeros(r)
        self.a = np.zeros(r)
        self.f = np.zeros(r)
        self.h = dt
        self.alpha_m, self.beta_k = mass_damp, stiff_damp
        self.betaDeltaT2 = beta * dt * dt
        self.gammaDeltaT = gamma * dt
        self.minusBetaDeltaT2 = dt * dt * 0.5 - self.betaDeltaT2
        self.minusGammaDeltaT = dt - self.gammaDeltaT

    def set_external(self, f_ext):
        # vws[i] = sum over the forcer's entries (ascending DOF) of f * basis_i
        f = np.asarray(f_ext, np.float64)
        self.f = np.array([float(np.sum(f * self.phi[:, i])) for i in range(self.lam.size)])
        self.a = self.f.copy()

    def step(self, n=1):
        d, v, a = self.d, self.v, self.a
        for _ in range(n):
            d_pre, v_pre, a_pre = d, v, a
            d_predict = d_pre + self.h * v_pre + self.minusBetaDeltaT2 * a_pre
            v_predict = v_pre + self.minusGammaDeltaT * a_pre
            xi = self.alpha_m + self.beta_k * self.lam
            righthand = self.f - xi * v_predict - self.lam * d_predict
            lefthand = 1.0 + self.gammaDeltaT * xi + self.betaDeltaT2 * self.lam
            a = righthand / lefthand
            v = v_predict + self.gammaDeltaT * a
            d = d_predict + self.betaDeltaT2 * a
        self.d, self.v, self.a = d, v, a

    def full_order(self, c=None):
        """sum_i c_i phi_i (c defaults to the displacement d), compacted DOFs."""
        c = self.d if c is None else c
        out = np.zeros(self.phi.shape[0])
        for i in range(c.size):
            out += c[i] * self.phi[:, i]
        return out


def to_nodes(red, n_nodes, cdofs, base=None):
    """Compacted DOF values in the node layout (constrained entries: base or 0)."""
    out = np.zeros(3 * n_nodes) if base is None else np.array(base, np.float64).reshape(-1).copy()
    free = np.setdiff1d(np.arange(3 * n_nodes), np.asarray(cdofs, np.int64))
    out[free] = red
    return out.reshape(n_nodes, 3)
