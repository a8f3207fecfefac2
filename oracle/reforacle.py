"""ctypes binding of the compiled reference oracle (``oracle/_ref/libodref.so``).

Test infrastructure only: used by ``tests/``, the golden-fixture generator and
the CPU baseline leg of ``bench.py``.  Every call runs the reference's own
C++ code (see ``oracle/ref_harness.cpp``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libodref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError(f"reference oracle not built: {LIB_PATH} (run oracle/build_ref.py)")
        L = C.CDLL(LIB_PATH)
        L.odref_scene_create.restype = C.c_void_p
        L.odref_scene_create.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip,
                                         C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        L.odref_scene_destroy.argtypes = [C.c_void_p]
        L.odref_dofs.argtypes = [C.c_void_p]
        L.odref_pattern_sizes.argtypes = [C.c_void_p, _ip]
        L.odref_pattern.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip]
        L.odref_set_displacements.argtypes = [C.c_void_p, _dp]
        L.odref_get_displacements.argtypes = [C.c_void_p, _dp]
        L.odref_element_values.argtypes = [C.c_void_p, _dp, _dp]
        L.odref_assemble.argtypes = [C.c_void_p, _dp, _dp]
        L.odref_mass.argtypes = [C.c_void_p, _dp]
        L.odref_spmdv.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.odref_cg.restype = C.c_int
        L.odref_cg.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double]
        L.odref_loads_clear.argtypes = [C.c_void_p]
        L.odref_loads_body.argtypes = [C.c_void_p, _dp]
        L.odref_loads_surface.argtypes = [C.c_void_p, _dp, C.c_int, _ip]
        L.odref_loads_get.argtypes = [C.c_void_p, _dp]
        L.odref_be_setup.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                     C.c_int, C.c_double, C.c_double]
        L.odref_be_apply_loads.argtypes = [C.c_void_p]
        L.odref_be_step.restype = C.c_int
        L.odref_be_step.argtypes = [C.c_void_p, C.c_int]
        L.odref_be_velocity.argtypes = [C.c_void_p, _dp]
        L.odref_nm_setup.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double]
        L.odref_nm_apply_loads.argtypes = [C.c_void_p]
        L.odref_nm_step.restype = C.c_int
        L.odref_nm_step.argtypes = [C.c_void_p, C.c_int]
        L.odref_nm_state.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.odref_polar.argtypes = [_dp, _dp, _dp]
        L.odref_qr.argtypes = [_dp, _dp, _dp]
        L.odref_eigsym.argtypes = [_dp, _dp, _dp]
        L.odref_plastic_params.argtypes = [C.c_double, C.c_double, C.c_double]
        L.odref_plastic_state.argtypes = [C.c_void_p, _dp]
        L.odref_ldlt_factor.restype = C.c_int
        L.odref_ldlt_factor.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double]
        L.odref_ldlt_get.argtypes = [C.c_void_p, _dp, _ip, _ip, _dp]
        L.odref_ldlt_apply.argtypes = [C.c_void_p, _dp, _dp]
        L.odref_ic_factor.restype = C.c_int
        L.odref_ic_factor.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double]
        L.odref_ic_get.argtypes = [C.c_void_p, _dp, _ip, _ip]
        L.odref_ic_apply.argtypes = [C.c_void_p, _dp, _dp]
        L.odref_relabel.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip]
        L.odref_plane_damping.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_double, C.c_int, _ip, _dp]
        L.odref_be_plane_damping.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double, C.c_int, _ip]
        L.odref_linear_csc.restype = C.c_int
        L.odref_linear_csc.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, _ip, _ip, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


PRECOND = {"none": 0, "jacobi": 1, "ic": 2, "ldlt": 3}
MATERIAL = {"corotational": 0, "neohookean": 1, "stvk": 2, "corotational_plastic": 3}


class RefScene:
    """One reference scene: mesh, constraints, material, pattern and state."""

    def __init__(self, X, tets, facets, cdofs, material="corotational", density=1000.0,
                 youngs=1e5, poisson=0.45, threshold=0.1, plastic=(1e-3, 0.5, 0.05)):
        """plastic: (yieldCriterion, creepRatio, maxPlasticStrain) of the
        corotational plastic material."""
        L = lib()
        L.odref_plastic_params(*[float(v) for v in plastic])
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32)
        self.facets = np.ascontiguousarray(facets, dtype=np.int32).reshape(-1, 3)
        self.cdofs = np.ascontiguousarray(np.sort(cdofs), dtype=np.int32)
        self.n_nodes = self.X.shape[0]
        self.n_tets = self.tets.shape[0]
        self.h = L.odref_scene_create(self.n_nodes, _d(self.X), self.n_tets, _i(self.tets),
                                      self.facets.shape[0], _i(self.facets),
                                      self.cdofs.size, _i(self.cdofs), MATERIAL[material],
                                      density, youngs, poisson, threshold)
        self.dofs = L.odref_dofs(self.h)
        s = np.zeros(5, dtype=np.int32)
        L.odref_pattern_sizes(self.h, _i(s))
        self.sizes = s

    def close(self):
        if self.h:
            lib().odref_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_values(self) -> int:
        return int(self.sizes[4])

    def pattern(self):
        nc = int(self.sizes[1] + self.sizes[2])
        pcol = np.zeros(nc + 1, np.int32)
        rows = np.zeros(int(self.sizes[3]), np.int32)
        oris = np.zeros(nc + 1, np.int32)
        emap = np.full((self.n_tets, 78), -1, np.int32)
        lib().odref_pattern(self.h, _i(pcol), _i(rows), _i(oris), _i(emap))
        return pcol, rows, oris, emap

    def set_displacements(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 3)
        lib().odref_set_displacements(self.h, _d(u))

    def displacements(self):
        u = np.zeros((self.n_nodes, 3))
        lib().odref_get_displacements(self.h, _d(u))
        return u

    def element_values(self):
        K = np.zeros((self.n_tets, 78))
        f = np.zeros((self.n_tets, 12))
        lib().odref_element_values(self.h, _d(K), _d(f))
        return K, f

    def plastic_state(self):
        """Plastic strain, 9 per element (row-major), of a corotational plastic scene."""
        out = np.zeros((self.n_tets, 9))
        lib().odref_plastic_state(self.h, _d(out))
        return out

    def assemble(self):
        v = np.zeros(self.n_values)
        f = np.zeros(self.dofs)
        lib().odref_assemble(self.h, _d(v), _d(f))
        return v, f

    def mass(self):
        v = np.zeros(self.n_values)
        lib().odref_mass(self.h, _d(v))
        return v

    def linear_csc(self, which, youngs, poisson):
        """The modal path's Hooke stiffness (which="K") or consistent mass
        (which="M") from the reference's scalar assembler: (pcol, rows,
        values) of the lower triangle by columns."""
        w = {"K": 0, "M": 1}[which]
        nnz = lib().odref_linear_csc(self.h, w, youngs, poisson, None, None, None)
        pcol = np.zeros(self.dofs + 1, np.int32)
        rows = np.zeros(nnz, np.int32)
        vals = np.zeros(nnz)
        lib().odref_linear_csc(self.h, w, youngs, poisson, _i(pcol), _i(rows), _d(vals))
        return pcol, rows, vals

    def spmdv(self, values, x, y=None):
        values = np.ascontiguousarray(values, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.dofs) if y is None else np.array(y, dtype=np.float64)
        lib().odref_spmdv(self.h, _d(values), _d(x), _d(y))
        return y

    def cg(self, values, b, x0=None, tol=1e-8, maxit=1000, precond="jacobi", eps=1e-3, relax=0.0):
        values = np.ascontiguousarray(values, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.dofs) if x0 is None else np.array(x0, dtype=np.float64)
        it = lib().odref_cg(self.h, _d(values), _d(b), _d(x), tol, maxit, PRECOND[precond], eps, relax)
        return x, it

    def ldlt(self, values, sainv_eps, ldlt_eps):
        """InLDLTPreconditioner::Preprocess on A = values: returns (L values,
        L rows, pcol, inverted diagonal) in the reference's storage."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        nnz = lib().odref_ldlt_factor(self.h, _d(values), sainv_eps, ldlt_eps)
        lv = np.zeros(max(nnz, 1))
        lr = np.zeros(max(nnz, 1), dtype=np.int32)
        pc = np.zeros(max(self.dofs, 1), dtype=np.int32)
        dinv = np.zeros(self.dofs)
        lib().odref_ldlt_get(self.h, _d(lv), _i(lr), _i(pc), _d(dinv))
        return lv[:nnz], lr[:nnz], pc, dinv

    def ic(self, values, eps, relax):
        """InCholeskyPreconditioner::Preprocess on A = values: returns (L
        values, L rows, pcol) in the reference's storage (diagonal first in
        every column)."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        nnz = lib().odref_ic_factor(self.h, _d(values), eps, relax)
        lv = np.zeros(max(nnz, 1))
        lr = np.zeros(max(nnz, 1), dtype=np.int32)
        pc = np.zeros(self.dofs + 1, dtype=np.int32)
        lib().odref_ic_get(self.h, _d(lv), _i(lr), _i(pc))
        return lv[:nnz], lr[:nnz], pc

    def ic_apply(self, rhs):
        """(L L^T)^-1 rhs with the factor of the last ic() call."""
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        out = np.zeros(self.dofs)
        lib().odref_ic_apply(self.h, _d(rhs), _d(out))
        return out

    def ldlt_apply(self, rhs):
        """(L D L^T)^-1 rhs with the factor of the last ldlt() call."""
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        out = np.zeros(self.dofs)
        lib().odref_ldlt_apply(self.h, _d(rhs), _d(out))
        return out

    def plane_damping(self, vel, normal, constant, coeff, elems):
        """MeshPlaneCollisionDampingForcer values for elems against the plane
        normal.x + constant = 0 with node velocities vel (n_nodes x 3)."""
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        nrm = np.ascontiguousarray(normal, dtype=np.float64)
        el = np.ascontiguousarray(elems, dtype=np.int32)
        out = np.zeros(self.n_values)
        lib().odref_plane_damping(self.h, _d(vel), _d(nrm), float(constant), float(coeff), el.size, _i(el), _d(out))
        return out

    def be_plane_damping(self, normal, constant, coeff, elems):
        """Backward Euler: replace the damping matrix by the plane forcer's,
        with the integrator's current node velocities."""
        nrm = np.ascontiguousarray(normal, dtype=np.float64)
        el = np.ascontiguousarray(elems, dtype=np.int32)
        lib().odref_be_plane_damping(self.h, _d(nrm), float(constant), float(coeff), el.size, _i(el))

    def loads(self, body=None, tractions=()):
        """Rebuild the load set: body force density then (traction, facets) pairs."""
        L = lib()
        L.odref_loads_clear(self.h)
        if body is not None:
            b = np.asarray(body, dtype=np.float64)
            L.odref_loads_body(self.h, _d(b))
        for t, fac in tractions:
            t = np.asarray(t, dtype=np.float64)
            fac = np.ascontiguousarray(fac, dtype=np.int32)
            L.odref_loads_surface(self.h, _d(t), fac.size, _i(fac))
        f = np.zeros(self.dofs)
        L.odref_loads_get(self.h, _d(f))
        return f

    def be_setup(self, dt, alpha_m, beta_k, tol=1e-8, maxit=1000, precond="jacobi", eps=1e-3, relax=0.0):
        lib().odref_be_setup(self.h, alpha_m, beta_k, dt, tol, maxit, PRECOND[precond], eps, relax)

    def be_apply_loads(self):
        lib().odref_be_apply_loads(self.h)

    def be_step(self, n=1) -> int:
        return lib().odref_be_step(self.h, n)

    def be_velocity(self):
        v = np.zeros(self.dofs)
        lib().odref_be_velocity(self.h, _d(v))
        return v

    def nm_setup(self, dt, alpha_m, beta_k, beta=0.25, gamma=0.5, newton=1, tol=1e-8, maxit=1000,
                 precond="jacobi", eps=1e-3, relax=0.0):
        lib().odref_nm_setup(self.h, beta, gamma, alpha_m, beta_k, dt, newton, tol, maxit,
                             PRECOND[precond], eps, relax)

    def nm_apply_loads(self):
        lib().odref_nm_apply_loads(self.h)

    def nm_step(self, n=1) -> int:
        return lib().odref_nm_step(self.h, n)

    def nm_state(self):
        d, v, a = np.zeros(self.dofs), np.zeros(self.dofs), np.zeros(self.dofs)
        lib().odref_nm_state(self.h, _d(d), _d(v), _d(a))
        return d, v, a


def relabel(n_nodes, elems):
    """MeshRelabeler::getNewLables: (new label of every node, elements with
    the new labels in the reference's new order)."""
    e = np.ascontiguousarray(elems, dtype=np.int32).copy()
    labels = np.zeros(n_nodes, dtype=np.int32)
    lib().odref_relabel(int(n_nodes), e.shape[0], e.shape[1], _i(e), _i(labels))
    return labels, e


def polar(F):
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
    R, S = np.zeros(9), np.zeros(9)
    lib().odref_polar(_d(F), _d(R), _d(S))
    return R.reshape(3, 3), S.reshape(3, 3)


def qr(F):
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
    Q, R = np.zeros(9), np.zeros(9)
    lib().odref_qr(_d(F), _d(Q), _d(R))
    return Q.reshape(3, 3), R.reshape(3, 3)


def eigsym(tri6):
    t = np.ascontiguousarray(tri6, dtype=np.float64).reshape(6)
    vals, vecs = np.zeros(3), np.zeros(9)
    lib().odref_eigsym(_d(t), _d(vals), _d(vecs))
    return vals, vecs.reshape(3, 3)
