"""The modal-path oracle (oracle/modal.py) pinned against the golden fixtures.

* The compiled reference (oracle/_ref, when present) reproduces the fixtures'
  Hooke stiffness and consistent mass bit for bit (HookeMaterial and the
  scalar mass assembler, material/hooke.cpp:18-60).
* The eigenpairs: ARPACK's shift-invert mode (scipy's eigsh, the algorithm
  the reference links) and, independently, a dense generalized symmetric
  eigensolve (LAPACK) of the fixtures' K and M agree with the fixtures'
  eigenvalues to 1e-9 and span the same modes.
* The restated LinearNewmark steps reproduce the fixtures' reduced state and
  displacements bit for bit from the fixtures' eigenpairs and loads.
"""
import numpy as np
import pytest

from oracle import modal as MO
from oracle import reforacle as R

CASES = ["full", "partial", "grid"]


def matrices(z):
    n = z["fext"].size
    K = MO.sym_from_lower_csc(z["K_pcol"], z["K_rows"], z["K_vals"], n)
    M = MO.sym_from_lower_csc(z["M_pcol"], z["M_rows"], z["M_vals"], n)
    return K, M


@pytest.mark.parametrize("case", CASES)
def test_reference_matrices_match_golden(golden, case):
    if not R.available():
        pytest.skip("compiled reference not available (oracle/build_ref.py)")
    z = golden(f"modal_{case}")
    rho, E, nu = z["material"]
    s = R.RefScene(z["X"], z["tets"], z["facets"], z["cdofs"], "corotational", rho, E, nu, 0.1)
    for which in ("K", "M"):
        pcol, rows, vals = s.linear_csc(which, E, nu)
        assert np.array_equal(pcol, z[f"{which}_pcol"])
        assert np.array_equal(rows, z[f"{which}_rows"])
        assert np.array_equal(vals, z[f"{which}_vals"])


@pytest.mark.parametrize("case", CASES)
def test_eigenpairs_two_ways(golden, case):
    import scipy.linalg as sl
    z = golden(f"modal_{case}")
    K, M = matrices(z)
    r = int(z["n_modes"])
    lam, phi = MO.modes(K, M, r)
    assert np.allclose(lam, z["lam"], rtol=1e-9, atol=0)
    # same modes up to sign: |phi_i^T M phi_ref_i| = 1
    overlap = np.abs(np.einsum("ij,ij->j", phi, M @ z["phi"]))
    assert np.allclose(overlap, 1.0, atol=1e-8)
    w = sl.eigh(K.toarray(), M.toarray(), eigvals_only=True, subset_by_index=[0, r - 1])
    assert np.allclose(w, z["lam"], rtol=1e-9, atol=0)
    # M-orthonormal, and K phi = lambda M phi
    assert np.abs(z["phi"].T @ (M @ z["phi"]) - np.eye(r)).max() < 1e-12
    res = K @ z["phi"] - (M @ z["phi"]) * z["lam"]
    assert np.abs(res).max() <= 1e-8 * np.abs(K @ z["phi"]).max()


@pytest.mark.parametrize("case", CASES)
def test_restated_steps_bit_exact(golden, case):
    z = golden(f"modal_{case}")
    beta, gamma, am, bk, dt = z["step_params"]
    o = MO.LinearNewmarkOracle(z["lam"], z["phi"], beta, gamma, am, bk, dt)
    o.set_external(z["fext"])
    assert np.array_equal(o.f, z["f_modal"])
    assert np.array_equal(o.a, z["f_modal"])
    o.step(int(z["steps"]))
    assert np.array_equal(o.d, z["d"]) and np.array_equal(o.v, z["v"]) and np.array_equal(o.a, z["a"])
    n_nodes = z["X"].shape[0]
    assert np.array_equal(MO.to_nodes(o.full_order(), n_nodes, z["cdofs"]), z["u"])
    assert np.array_equal(MO.to_nodes(o.full_order(o.v), n_nodes, z["cdofs"]), z["vel"])
    assert np.abs(z["u"]).max() > 1e-4   # the load moves the mesh
