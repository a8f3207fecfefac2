"""ctypes binding of the oracle restatement (``oracle/_build/libodoracle.so``).

Test infrastructure only: used by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libodoracle.so")
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None

PRECOND = {"none": 0, "jacobi": 1, "block_jacobi": 2, "ic0": 3, "ldlt": 4, "ic": 5}
MATERIAL = {"corotational": 0, "neohookean": 1, "stvk": 2, "corotational_plastic": 3}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build_oracle
            build_oracle.build()
        L = C.CDLL(LIB_PATH)
        L.odo_scene_create.restype = C.c_void_p
        L.odo_scene_create.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip,
                                       C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        L.odo_scene_destroy.argtypes = [C.c_void_p]
        L.odo_dofs.argtypes = [C.c_void_p]
        L.odo_pattern_sizes.argtypes = [C.c_void_p, _ip]
        L.odo_pattern.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip]
        L.odo_set_displacements.argtypes = [C.c_void_p, _dp]
        L.odo_set_plastic.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.odo_plastic_state.argtypes = [C.c_void_p, _dp]
        L.odo_get_displacements.argtypes = [C.c_void_p, _dp]
        L.odo_element_values.argtypes = [C.c_void_p, _dp, _dp]
        L.odo_assemble.argtypes = [C.c_void_p, _dp, _dp]
        L.odo_mass.argtypes = [C.c_void_p, _dp]
        L.odo_spmdv.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.odo_set_ic0_natural.argtypes = [C.c_void_p, C.c_int]
        L.odo_pcg.restype = C.c_int
        L.odo_pcg.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int]
        L.odo_loads.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _ip, _ip, _dp]
        L.odo_integrator_setup.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_int, C.c_double, C.c_int, C.c_int]
        L.odo_set_fext.argtypes = [C.c_void_p, _dp]
        L.odo_be_step.restype = C.c_int
        L.odo_be_step.argtypes = [C.c_void_p, C.c_int]
        L.odo_nm_step.restype = C.c_int
        L.odo_nm_step.argtypes = [C.c_void_p, C.c_int]
        L.odo_state.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.odo_polar.argtypes = [_dp, _dp, _dp]
        L.odo_qr.argtypes = [_dp, _dp, _dp]
        L.odo_eigsym.argtypes = [_dp, _dp, _dp]
        L.odo_set_ldlt.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.odo_ldlt_factor.restype = C.c_int
        L.odo_ldlt_factor.argtypes = [C.c_void_p, _dp]
        L.odo_ldlt_get.argtypes = [C.c_void_p, _dp, _ip, _ip, _dp]
        L.odo_ldlt_apply.argtypes = [C.c_void_p, _dp, _dp]
        L.odo_set_ic.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.odo_ic_factor.restype = C.c_int
        L.odo_ic_factor.argtypes = [C.c_void_p, _dp]
        L.odo_ic_get.argtypes = [C.c_void_p, _dp, _ip, _ip]
        L.odo_ic_apply.argtypes = [C.c_void_p, _dp, _dp]
        L.odo_plane_damping.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_double, C.c_int, _ip, _dp]
        L.odo_clear_damping.argtypes = [C.c_void_p]
        L.odo_integrator_plane_damping.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double, C.c_int, _ip]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class OracleScene:
    """Restated scene with the same surface as ``reforacle.RefScene``."""

    def __init__(self, X, tets, facets, cdofs, material="corotational", density=1000.0,
                 youngs=1e5, poisson=0.45, threshold=0.1, plastic=(1e-3, 0.5, 0.05)):
        """plastic: (yieldCriterion, creepRatio, maxPlasticStrain) of the
        corotational plastic material."""
        L = lib()
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32)
        self.facets = np.ascontiguousarray(facets, dtype=np.int32).reshape(-1, 3)
        self.cdofs = np.ascontiguousarray(np.sort(cdofs), dtype=np.int32)
        self.n_nodes = self.X.shape[0]
        self.n_tets = self.tets.shape[0]
        self.h = L.odo_scene_create(self.n_nodes, _d(self.X), self.n_tets, _i(self.tets),
                                    self.facets.shape[0], _i(self.facets), self.cdofs.size,
                                    _i(self.cdofs), MATERIAL[material], density, youngs, poisson,
                                    threshold)
        self.dofs = L.odo_dofs(self.h)
        if material == "corotational_plastic":
            L.odo_set_plastic(self.h, *[float(v) for v in plastic])
        s = np.zeros(5, np.int32)
        L.odo_pattern_sizes(self.h, _i(s))
        self.sizes = s

    def close(self):
        if self.h:
            lib().odo_scene_destroy(self.h)
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
        lib().odo_pattern(self.h, _i(pcol), _i(rows), _i(oris), _i(emap))
        return pcol, rows, oris, emap

    def set_displacements(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 3)
        lib().odo_set_displacements(self.h, _d(u))

    def displacements(self):
        u = np.zeros((self.n_nodes, 3))
        lib().odo_get_displacements(self.h, _d(u))
        return u

    def element_values(self):
        K = np.zeros((self.n_tets, 78))
        f = np.zeros((self.n_tets, 12))
        lib().odo_element_values(self.h, _d(K), _d(f))
        return K, f

    def plastic_state(self):
        """Plastic strain, 9 per element (row-major), of a corotational plastic scene."""
        out = np.zeros((self.n_tets, 9))
        lib().odo_plastic_state(self.h, _d(out))
        return out

    def assemble(self):
        v = np.zeros(self.n_values)
        f = np.zeros(self.dofs)
        lib().odo_assemble(self.h, _d(v), _d(f))
        return v, f

    def mass(self):
        v = np.zeros(self.n_values)
        lib().odo_mass(self.h, _d(v))
        return v

    def spmdv(self, values, x, y=None):
        values = np.ascontiguousarray(values, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.dofs) if y is None else np.array(y, dtype=np.float64)
        lib().odo_spmdv(self.h, _d(values), _d(x), _d(y))
        return y

    def pcg(self, values, b, x0=None, tol=1e-8, maxit=1000, precond="jacobi"):
        values = np.ascontiguousarray(values, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.dofs) if x0 is None else np.array(x0, dtype=np.float64)
        it = lib().odo_pcg(self.h, _d(values), _d(b), _d(x), tol, maxit, PRECOND[precond])
        return x, it

    def set_ldlt(self, sainv_eps=0.1, ldlt_eps=0.01):
        """Drop bounds of the incomplete LDL^T (precond "ldlt")."""
        lib().odo_set_ldlt(self.h, float(sainv_eps), float(ldlt_eps))

    def ldlt(self, values):
        """Incomplete LDL^T of A = values with the bounds of set_ldlt: (L
        values, L rows, pcol, inverted diagonal) in the reference's storage."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        nnz = lib().odo_ldlt_factor(self.h, _d(values))
        lv = np.zeros(max(nnz, 1))
        lr = np.zeros(max(nnz, 1), np.int32)
        pc = np.zeros(max(self.dofs, 1), np.int32)
        dinv = np.zeros(max(self.dofs, 1))
        lib().odo_ldlt_get(self.h, _d(lv), _i(lr), _i(pc), _d(dinv))
        return lv[:nnz], lr[:nnz], pc[: self.dofs], dinv[: self.dofs]

    def set_ic0_natural(self, natural=True):
        """IC(0) (precond "ic0") in the DOF order instead of by block colours."""
        lib().odo_set_ic0_natural(self.h, int(bool(natural)))

    def set_ic(self, eps=1e-3, relax=0.0):
        """(epsilon, relaxedScale) of the threshold incomplete Cholesky (precond "ic")."""
        lib().odo_set_ic(self.h, float(eps), float(relax))

    def ic(self, values):
        """Threshold incomplete Cholesky of A = values: (L values, L rows,
        pcol) in the reference's storage."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        nnz = lib().odo_ic_factor(self.h, _d(values))
        lv = np.zeros(max(nnz, 1))
        lr = np.zeros(max(nnz, 1), np.int32)
        pc = np.zeros(self.dofs + 1, np.int32)
        lib().odo_ic_get(self.h, _d(lv), _i(lr), _i(pc))
        return lv[:nnz], lr[:nnz], pc

    def ic_apply(self, rhs):
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        out = np.zeros(self.dofs)
        lib().odo_ic_apply(self.h, _d(rhs), _d(out))
        return out

    def ldlt_apply(self, rhs):
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        out = np.zeros(self.dofs)
        lib().odo_ldlt_apply(self.h, _d(rhs), _d(out))
        return out

    def plane_damping(self, vel, normal, constant, coeff, elems):
        """Plane collision damping values (reference layout) for elems."""
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        nrm = np.ascontiguousarray(normal, dtype=np.float64)
        el = np.ascontiguousarray(elems, dtype=np.int32)
        out = np.zeros(self.n_values)
        lib().odo_plane_damping(self.h, _d(vel), _d(nrm), float(constant), float(coeff), el.size, _i(el), _d(out))
        return out

    def clear_damping(self):
        lib().odo_clear_damping(self.h)

    def integrator_plane_damping(self, normal, constant, coeff, elems):
        """Replace the integrators' damping matrix by the plane forcer's, with
        the integrator's current node velocities."""
        nrm = np.ascontiguousarray(normal, dtype=np.float64)
        el = np.ascontiguousarray(elems, dtype=np.int32)
        lib().odo_integrator_plane_damping(self.h, _d(nrm), float(constant), float(coeff), el.size, _i(el))

    def loads(self, body=None, tractions=()):
        t = np.zeros((max(len(tractions), 1), 3))
        sizes = np.zeros(max(len(tractions), 1), np.int32)
        ids = [np.zeros(0, np.int32)]
        for k, (tr, fac) in enumerate(tractions):
            t[k] = tr
            fac = np.asarray(fac, dtype=np.int32)
            sizes[k] = fac.size
            ids.append(fac)
        ids = np.ascontiguousarray(np.concatenate(ids), dtype=np.int32)
        if ids.size == 0:
            ids = np.zeros(1, np.int32)
        f = np.zeros(self.dofs)
        b = None if body is None else np.ascontiguousarray(body, dtype=np.float64)
        lib().odo_loads(self.h, None if b is None else _d(b), len(tractions), _d(t), _i(sizes),
                        _i(ids), _d(f))
        return f

    def integrator_setup(self, dt, alpha_m, beta_k, beta=0.25, gamma=0.5, newton=1, tol=1e-8,
                         maxit=1000, precond="jacobi"):
        lib().odo_integrator_setup(self.h, dt, alpha_m, beta_k, beta, gamma, newton, tol, maxit,
                                   PRECOND[precond])

    def set_fext(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        lib().odo_set_fext(self.h, _d(f))

    def be_step(self, n=1) -> int:
        return lib().odo_be_step(self.h, n)

    def nm_step(self, n=1) -> int:
        return lib().odo_nm_step(self.h, n)

    def state(self):
        d, v, a = np.zeros(self.dofs), np.zeros(self.dofs), np.zeros(self.dofs)
        lib().odo_state(self.h, _d(d), _d(v), _d(a))
        return d, v, a


def polar(F):
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
    R, S = np.zeros(9), np.zeros(9)
    lib().odo_polar(_d(F), _d(R), _d(S))
    return R.reshape(3, 3), S.reshape(3, 3)


def qr(F):
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
    Q, R = np.zeros(9), np.zeros(9)
    lib().odo_qr(_d(F), _d(Q), _d(R))
    return Q.reshape(3, 3), R.reshape(3, 3)


def eigsym(tri6):
    t = np.ascontiguousarray(tri6, dtype=np.float64).reshape(6)
    vals, vecs = np.zeros(3), np.zeros(9)
    lib().odo_eigsym(_d(t), _d(vals), _d(vecs))
    return vals, vecs.reshape(3, 3)
