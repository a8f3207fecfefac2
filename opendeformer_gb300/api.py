"""Python host side of the GB300 implicit FEM step, over the C ABI.

Mirrors the reference's plugin seams so that code written against the
reference reads the same:

* materials: ``CorotationalHyperelasticMaterial(rho, youngs, poisson,
  threshold)`` (material/corotationalHyperelastic.h:13),
  ``InvertibleNeoHookeanMaterial`` / ``InvertibleStVKMaterial(rho, youngs,
  poisson, inversionThreshold)`` (material/invertibleNeoHookean.h,
  material/invertibleStVK.h);
* preconditioners / solver: ``JacobiPreconditioner()``,
  ``BlockJacobiPreconditioner()``, ``IC0Preconditioner()``,
  ``InLDLTPreconditioner(sainvEpsilon, ldltEpsilon)``,
  ``InCholeskyPreconditioner(epsilon, relaxedScale)`` and
  ``CGSolver(tol, maxIter, preconditioner)`` (solver/cgSolver.h:16-17);
* integrators: ``NonlinearImplicitBackwardEuler(massDamp, stiffDamp, ts,
  solver)`` (intergrator/nonlinearImplicitBackwardEuler.h:48-73) and
  ``NewmarkIntegrator(beta, gamma, massDamp, stiffDamp, ts, solver,
  newton_iters)``;
* ``Simulator(scene, integrator)`` with ``runTimeSteps`` /
  ``getVertexPositions`` (core/simulator.h:12-28).

Everything computes on the GPU through ``libodgpu.so``; there is no CPU
fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import atexit
import ctypes as C
import dataclasses
import os
import weakref

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libodgpu.so")

OD_OK = 0
STATUS = {0: "OD_OK", 1: "OD_ERR_INVALID_ARG", 2: "OD_ERR_OUT_OF_MEMORY", 3: "OD_ERR_NOT_CONVERGED",
          4: "OD_ERR_NAN", 5: "OD_ERR_DEVICE_TIMEOUT", 6: "OD_ERR_CUDA", 7: "OD_ERR_UNSUPPORTED",
          8: "OD_ERR_INTERNAL"}

MATERIAL_KIND = {"corotational": 0, "neohookean": 1, "stvk": 2, "corotational_plastic": 3}
PRECOND_KIND = {"none": 0, "jacobi": 1, "block_jacobi": 2, "ic0": 3, "ldlt": 4, "ic": 5}
PRECISION = {"fp64": 0, "mixed": 1}


class ODError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class od_material(C.Structure):
    _fields_ = [("kind", C.c_int), ("density", C.c_double), ("youngs", C.c_double),
                ("poisson", C.c_double), ("threshold", C.c_double), ("yield_criterion", C.c_double),
                ("creep_ratio", C.c_double), ("max_plastic_strain", C.c_double)]


class od_solver_params(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("precond", C.c_int), ("precision", C.c_int),
                ("replace_every", C.c_int), ("inner_tol", C.c_double), ("max_refine", C.c_int),
                ("sainv_eps", C.c_double), ("ldlt_eps", C.c_double), ("ic_eps", C.c_double),
                ("ic_relax", C.c_double)]


class od_solve_stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("refinements", C.c_int), ("rel_residual", C.c_double),
                ("ic_shift", C.c_double), ("status", C.c_int)]


class od_integrator_params(C.Structure):
    _fields_ = [("kind", C.c_int), ("dt", C.c_double), ("alpha_m", C.c_double), ("beta_k", C.c_double),
                ("nm_beta", C.c_double), ("nm_gamma", C.c_double), ("newton_iters", C.c_int),
                ("solver", od_solver_params)]


class od_step_stats(C.Structure):
    _fields_ = [("steps", C.c_int), ("pcg_iterations", C.c_int), ("solves", C.c_int),
                ("max_rel_residual", C.c_double), ("status", C.c_int), ("device_ms", C.c_double)]


class od_counters(C.Structure):
    _fields_ = [("kernel_launches", C.c_longlong), ("host_syncs", C.c_longlong),
                ("spmv_launches", C.c_longlong), ("spmv_ms", C.c_double),
                ("pcg_launches", C.c_longlong), ("pcg_iterations", C.c_longlong), ("pcg_ms", C.c_double),
                ("mix_iterations", C.c_longlong), ("mix_spmv_ms", C.c_double), ("mix_spmv_bytes", C.c_double),
                ("mix_spmv_work_ms", C.c_double), ("mix_fallbacks", C.c_longlong),
                ("sweep_factors", C.c_longlong), ("sweep_factor_ms", C.c_double), ("sweep_nnz", C.c_longlong),
                ("sweep_applies", C.c_longlong), ("sweep_apply_ms", C.c_double), ("sweep_apply_bytes", C.c_double),
                ("sweep_levels", C.c_longlong), ("pcg_phase_ms", C.c_double * 6),
                ("pcg_phase_iterations", C.c_longlong), ("pcg_work_max_ms", C.c_double * 3),
                ("pcg_work_mean_ms", C.c_double * 3), ("mix_fallback_ms", C.c_double)]


class od_scene_info(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_tets", C.c_int), ("n_facets", C.c_int), ("dofs", C.c_int),
                ("num_block_columns", C.c_int), ("num_remained_columns", C.c_int),
                ("num_row_indices", C.c_int), ("num_values", C.c_int), ("num_full_blocks", C.c_int),
                ("num_colors", C.c_int), ("device_bytes", C.c_longlong), ("pcg_smem_bytes", C.c_int)]


class od_mixed_tuning(C.Structure):
    _fields_ = [("piece_steps", C.c_int), ("consumer_warps", C.c_int), ("slice_cost", C.c_double)]


class od_tune_report(C.Structure):
    _fields_ = [("candidates", C.c_int), ("best", od_mixed_tuning), ("default_ms", C.c_double),
                ("best_ms", C.c_double), ("default_iters", C.c_int), ("best_iters", C.c_int)]


class od_server_config(C.Structure):
    _fields_ = [("budget_bytes", C.c_longlong), ("reserve_bytes", C.c_longlong), ("max_batch", C.c_int),
                ("batched", C.c_int), ("admission_thread", C.c_int)]


class od_scene_spec(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("X", C.POINTER(C.c_double)), ("n_tets", C.c_int),
                ("tets", C.POINTER(C.c_int)), ("n_facets", C.c_int), ("facets", C.POINTER(C.c_int)),
                ("n_cdofs", C.c_int), ("cdofs", C.POINTER(C.c_int)), ("n_load_facets", C.c_int),
                ("load_facets", C.POINTER(C.c_int)), ("material", od_material),
                ("integrator", od_integrator_params)]


class od_step_request(C.Structure):
    _fields_ = [("scene", C.c_int), ("dt", C.c_double), ("body", C.c_double * 3), ("traction", C.c_double * 3),
                ("arrival", C.c_double)]


class od_step_result(C.Structure):
    _fields_ = [("ticket", C.c_longlong), ("scene", C.c_int), ("status", C.c_int), ("pcg_iterations", C.c_int),
                ("arrival", C.c_double), ("done", C.c_double)]


class od_server_stats(C.Structure):
    _fields_ = [("ticks", C.c_longlong), ("steps", C.c_longlong), ("admissions", C.c_longlong),
                ("restores", C.c_longlong), ("evictions", C.c_longlong), ("deferred", C.c_longlong),
                ("s_admit", C.c_double), ("s_loads", C.c_double), ("s_step", C.c_double), ("s_worker", C.c_double),
                ("resident", C.c_longlong), ("resident_bytes", C.c_longlong), ("budget_bytes", C.c_longlong),
                ("s_build", C.c_double), ("s_device", C.c_double)]


class od_modal_params(C.Structure):
    _fields_ = [("n_modes", C.c_int), ("beta", C.c_double), ("gamma", C.c_double), ("alpha_m", C.c_double),
                ("beta_k", C.c_double), ("dt", C.c_double), ("youngs", C.c_double), ("poisson", C.c_double),
                ("tol", C.c_double), ("krylov", C.c_int), ("inner_tol", C.c_double), ("inner_max_iter", C.c_int),
                ("max_restarts", C.c_int)]


class od_modal_info(C.Structure):
    _fields_ = [("n_modes", C.c_int), ("dofs", C.c_int), ("krylov", C.c_int), ("lanczos_steps", C.c_int),
                ("restarts", C.c_int), ("pcg_iterations", C.c_longlong), ("max_residual", C.c_double),
                ("setup_ms", C.c_double)]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
_lib = None

# Live handles, released in a safe order (scenes before contexts) when the
# interpreter exits, before the CUDA runtime itself is torn down.
_live_batches: "weakref.WeakSet" = weakref.WeakSet()
_live_modals: "weakref.WeakSet" = weakref.WeakSet()
_live_scenes: "weakref.WeakSet" = weakref.WeakSet()
_live_ctxs: "weakref.WeakSet" = weakref.WeakSet()
_shutting_down = False


@atexit.register
def _release_all():
    global _shutting_down
    for md in list(_live_modals):
        try:
            md.close()
        except Exception:
            pass
    for bt in list(_live_batches):
        try:
            bt.close()
        except Exception:
            pass
    for sc in list(_live_scenes):
        try:
            sc.close()
        except Exception:
            pass
    for cx in list(_live_ctxs):
        try:
            cx.close()
        except Exception:
            pass
    _shutting_down = True

# name -> (restype, argtypes); every entry point of include/od_gb300.h
SIGNATURES = {
    "od_status_string": (C.c_char_p, [C.c_int]),
    "od_last_error": (C.c_char_p, []),
    "od_abi_version": (C.c_int, []),
    "od_selftest_bounded_waits": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "od_measure_fma_rate": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "od_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "od_ctx_destroy": (C.c_int, [_vp]),
    "od_ctx_synchronize": (C.c_int, [_vp]),
    "od_ctx_set_profiling": (C.c_int, [_vp, C.c_int]),
    "od_ctx_get_counters": (C.c_int, [_vp, C.POINTER(od_counters)]),
    "od_ctx_reset_counters": (C.c_int, [_vp]),
    "od_scene_create": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip,
                                  C.POINTER(od_material), C.POINTER(_vp)]),
    "od_scene_destroy": (C.c_int, [_vp]),
    "od_scene_get_info": (C.c_int, [_vp, C.POINTER(od_scene_info)]),
    "od_scene_pattern": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "od_scene_set_displacements": (C.c_int, [_vp, _dp]),
    "od_scene_get_displacements": (C.c_int, [_vp, _dp]),
    "od_scene_get_positions": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "od_scene_evaluate": (C.c_int, [_vp, _dp, _dp]),
    "od_scene_element_values": (C.c_int, [_vp, _dp, _dp]),
    "od_scene_mass": (C.c_int, [_vp, _dp]),
    "od_scene_spmdv": (C.c_int, [_vp, _dp, _dp, _dp]),
    "od_scene_pcg": (C.c_int, [_vp, _dp, _dp, _dp, C.POINTER(od_solver_params), C.POINTER(od_solve_stats)]),
    "od_scene_ldlt_factor": (C.c_int, [_vp, _dp, C.c_double, C.c_double, C.POINTER(C.c_longlong)]),
    "od_scene_ldlt_get": (C.c_int, [_vp, _dp, _ip, _ip, _dp]),
    "od_scene_ldlt_apply": (C.c_int, [_vp, _dp, _dp]),
    "od_scene_ic_factor": (C.c_int, [_vp, _dp, C.c_double, C.c_double, C.POINTER(C.c_longlong)]),
    "od_scene_ic_get": (C.c_int, [_vp, _dp, _ip, _ip]),
    "od_scene_ic_apply": (C.c_int, [_vp, _dp, _dp]),
    "od_scene_add_plane_damping": (C.c_int, [_vp, _dp, C.c_double, C.c_double, C.c_int, _ip, _dp]),
    "od_scene_clear_damping": (C.c_int, [_vp]),
    "od_scene_get_damping": (C.c_int, [_vp, _dp]),
    "od_scene_set_loads": (C.c_int, [_vp, _dp, C.c_int, _dp, _ip, _ip]),
    "od_scene_update_loads": (C.c_int, [_vp, C.c_double]),
    "od_scene_set_traction_schedule": (C.c_int, [_vp, C.c_double, C.c_double]),
    "od_scene_set_external_forces": (C.c_int, [_vp, _dp]),
    "od_scene_get_external_forces": (C.c_int, [_vp, _dp]),
    "od_integrator_setup": (C.c_int, [_vp, C.POINTER(od_integrator_params)]),
    "od_step": (C.c_int, [_vp, C.c_int, C.POINTER(od_step_stats)]),
    "od_get_state": (C.c_int, [_vp, _dp, _dp, _dp]),
    "od_set_state": (C.c_int, [_vp, _dp, _dp, _dp]),
    "od_integrator_update": (C.c_int, [_vp, C.POINTER(od_integrator_params)]),
    "od_scene_get_plastic_strain": (C.c_int, [_vp, _dp]),
    "od_scene_set_plastic_strain": (C.c_int, [_vp, _dp]),
    "od_batch_create": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), C.POINTER(_vp)]),
    "od_batch_step": (C.c_int, [_vp, C.c_int, C.POINTER(od_step_stats)]),
    "od_batch_destroy": (C.c_int, [_vp]),
    "od_batch_get_tuning": (C.c_int, [_vp, C.POINTER(od_mixed_tuning)]),
    "od_batch_set_tuning": (C.c_int, [_vp, C.POINTER(od_mixed_tuning)]),
    "od_batch_autotune": (C.c_int, [_vp, C.c_int, C.POINTER(od_tune_report)]),
    "od_bsr_pcg_noalloc": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, C.POINTER(od_solver_params), _vp,
                                     C.POINTER(od_solve_stats)]),
    "od_mesh_relabel": (C.c_int, [C.c_int, C.c_int, C.c_int, _ip, _ip]),
    "od_server_create": (C.c_int, [_vp, C.POINTER(od_server_config), C.POINTER(_vp)]),
    "od_server_destroy": (C.c_int, [_vp]),
    "od_server_add_scene": (C.c_int, [_vp, C.POINTER(od_scene_spec), C.POINTER(C.c_int)]),
    "od_server_now": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "od_server_submit": (C.c_int, [_vp, C.POINTER(od_step_request), C.POINTER(C.c_longlong)]),
    "od_server_tick": (C.c_int, [_vp, C.c_int, C.POINTER(od_step_result), C.POINTER(C.c_int)]),
    "od_server_pending": (C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    "od_server_warm": (C.c_int, [_vp, C.c_int, _ip, C.POINTER(C.c_int)]),
    "od_server_get_scene": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "od_server_get_stats": (C.c_int, [_vp, C.POINTER(od_server_stats)]),
    "od_modal_create": (C.c_int, [_vp, C.POINTER(od_modal_params), C.POINTER(_vp)]),
    "od_modal_destroy": (C.c_int, [_vp]),
    "od_modal_set_external_forces": (C.c_int, [_vp, _dp]),
    "od_modal_step": (C.c_int, [_vp, C.c_int]),
    "od_modal_get_displacements": (C.c_int, [_vp, _dp]),
    "od_modal_get_velocities": (C.c_int, [_vp, _dp]),
    "od_modal_get_modes": (C.c_int, [_vp, _dp, _dp]),
    "od_modal_get_state": (C.c_int, [_vp, _dp, _dp, _dp]),
    "od_modal_get_stiffness": (C.c_int, [_vp, _dp]),
    "od_modal_get_info": (C.c_int, [_vp, C.POINTER(od_modal_info)]),
    "od_scene_save": (C.c_int, [_vp, _vp, C.POINTER(C.c_size_t)]),
    "od_scene_load": (C.c_int, [_vp, _vp, C.c_size_t]),
}


def load_library(path: str | None = None):
    """Load libodgpu.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"GB300 library not built: {path} (run opendeformer_gb300/build.py)")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(status, what=""):
    if status != OD_OK:
        msg = load_library().od_last_error().decode(errors="replace")
        raise ODError(status, f"{what}: {msg}")


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


# ----------------------------------------------------------------- values
@dataclasses.dataclass
class Material:
    kind: str
    density: float
    youngs: float
    poisson: float
    threshold: float
    yield_criterion: float = 0.0      # corotational plastic only
    creep_ratio: float = 0.0
    max_plastic_strain: float = 0.0

    def to_c(self):
        return od_material(MATERIAL_KIND[self.kind], self.density, self.youngs, self.poisson, self.threshold,
                           self.yield_criterion, self.creep_ratio, self.max_plastic_strain)


def CorotationalHyperelasticMaterial(rho, youngs, poisson, compressingThreshold):
    return Material("corotational", rho, youngs, poisson, compressingThreshold)


def InvertibleNeoHookeanMaterial(rho, youngs, poisson, inversionThreshold):
    return Material("neohookean", rho, youngs, poisson, inversionThreshold)


def InvertibleStVKMaterial(rho, youngs, poisson, inversionThreshold):
    return Material("stvk", rho, youngs, poisson, inversionThreshold)


def CorotationalPlasticMaterial(rho, youngs, poisson, yieldCriterion, creepRatio, maxPlasticStrain,
                                compressingThreshold):
    """CorotationalPlasticMaterial (material/corotationalPlastic.h:11-30), same argument order."""
    return Material("corotational_plastic", rho, youngs, poisson, compressingThreshold, yieldCriterion, creepRatio,
                    maxPlasticStrain)


@dataclasses.dataclass
class Preconditioner:
    kind: str = "none"
    sainvEpsilon: float = 0.0   # LDL^T drop bounds (0: 0.1 and 0.01)
    ldltEpsilon: float = 0.0
    epsilon: float = 0.0        # IC: (epsilon, relaxedScale); epsilon 0: 1e-3
    relaxedScale: float = 0.0


def JacobiPreconditioner():
    return Preconditioner("jacobi")


def BlockJacobiPreconditioner():
    return Preconditioner("block_jacobi")


def IC0Preconditioner():
    return Preconditioner("ic0")


def InLDLTPreconditioner(sainvEpsilon=0.1, ldltEpsilon=0.01):
    """InLDLTPreconditioner(sainvEpsilon, ldltEpsilon) (solver/inLDLTPreconditioner.h:14-15)."""
    return Preconditioner("ldlt", float(sainvEpsilon), float(ldltEpsilon))


def InCholeskyPreconditioner(epsilon=1e-3, relaxedScale=0.0):
    """InCholeskyPreconditioner(epsilon, relaxedScale) (solver/inCholeskyPreconditioner.h):
    threshold incomplete Cholesky with fill."""
    return Preconditioner("ic", epsilon=float(epsilon), relaxedScale=float(relaxedScale))


@dataclasses.dataclass
class CGSolver:
    tol: float = 1e-8
    maxIter: int = 1000
    preconditioner: Preconditioner = dataclasses.field(default_factory=Preconditioner)
    precision: str = "fp64"
    replace_every: int = 0
    inner_tol: float = 0.0
    max_refine: int = 0

    def to_c(self):
        return od_solver_params(self.tol, self.maxIter, PRECOND_KIND[self.preconditioner.kind],
                                PRECISION[self.precision], self.replace_every, self.inner_tol,
                                self.max_refine, self.preconditioner.sainvEpsilon,
                                self.preconditioner.ldltEpsilon, self.preconditioner.epsilon,
                                self.preconditioner.relaxedScale)


@dataclasses.dataclass
class NonlinearImplicitBackwardEuler:
    massDamp: float
    stiffDamp: float
    ts: float
    solver: CGSolver

    def to_c(self):
        return od_integrator_params(0, self.ts, self.massDamp, self.stiffDamp, 0.25, 0.5, 1, self.solver.to_c())


@dataclasses.dataclass
class NewmarkIntegrator:
    beta: float
    gamma: float
    massDamp: float
    stiffDamp: float
    ts: float
    solver: CGSolver
    newton_iters: int = 1

    def to_c(self):
        return od_integrator_params(1, self.ts, self.massDamp, self.stiffDamp, self.beta, self.gamma,
                                    self.newton_iters, self.solver.to_c())


def mesh_relabel(n_nodes, elements):
    """MeshRelabeler::getNewLables (core/meshRelabler.cpp): Gibbs-Poole-
    Stockmeyer node relabeling.  Returns (new label of every node, elements
    rewritten with the new labels, reordered by the sum of their labels)."""
    e = np.ascontiguousarray(elements, dtype=np.int32).copy()
    labels = np.zeros(int(n_nodes), dtype=np.int32)
    _check(load_library().od_mesh_relabel(int(n_nodes), e.shape[0], e.shape[1], _i(e), _i(labels)), "mesh_relabel")
    return labels, e


def relabel_mesh(X, tets, facets, constrained_dofs):
    """A whole mesh under mesh_relabel: positions, elements, facets and the
    constrained DOFs in the new node order (plus the labels)."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    labels, t2 = mesh_relabel(X.shape[0], tets)
    X2 = np.empty_like(X)
    X2[labels] = X
    f2 = labels[np.asarray(facets, dtype=np.int64)].astype(np.int32)
    cd = np.asarray(constrained_dofs, dtype=np.int64)
    cd2 = np.sort(3 * labels[cd // 3] + cd % 3).astype(np.int32)
    return X2, t2, f2, cd2, labels


# ----------------------------------------------------------------- handles
class Context:
    """One CUDA device and stream (od_ctx)."""

    def __init__(self, device: int = 0):
        L = load_library()
        h = _vp()
        _check(L.od_ctx_create(device, C.byref(h)), "od_ctx_create")
        self.h = h
        self.device = device
        _live_ctxs.add(self)

    def synchronize(self):
        _check(load_library().od_ctx_synchronize(self.h), "od_ctx_synchronize")

    def set_profiling(self, enable):
        """False / 0 off; True / 1 CUDA events around PCG launches; 2 also the
        one-launch PCG's per-iteration phase timers (they slow each iteration)."""
        _check(load_library().od_ctx_set_profiling(self.h, int(enable)), "od_ctx_set_profiling")

    def selftest_bounded_waits(self):
        """od_selftest_bounded_waits: runs the grid-barrier and triangular-sweep
        waits against conditions that never clear; returns (barrier wait ran
        out, sweep wait ran out).  Takes a few seconds."""
        b, v = C.c_int(0), C.c_int(0)
        _check(load_library().od_selftest_bounded_waits(self.h, C.byref(b), C.byref(v)), "selftest_bounded_waits")
        return bool(b.value), bool(v.value)

    def measure_fma_rate(self, fp64: bool = True, iters: int = 1 << 14):
        """od_measure_fma_rate: (multiply-adds per second, launch ms) of
        independent FP64 (or FP32) multiply-add chains on every SM."""
        r, ms = C.c_double(0.0), C.c_double(0.0)
        _check(load_library().od_measure_fma_rate(self.h, int(bool(fp64)), int(iters), C.byref(r), C.byref(ms)),
               "od_measure_fma_rate")
        return r.value, ms.value

    def counters(self):
        c = od_counters()
        _check(load_library().od_ctx_get_counters(self.h, C.byref(c)), "od_ctx_get_counters")
        return c

    def reset_counters(self):
        _check(load_library().od_ctx_reset_counters(self.h), "od_ctx_reset_counters")

    def close(self):
        if getattr(self, "h", None) and not _shutting_down:
            load_library().od_ctx_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """Mesh + constraints + material on the device (od_scene)."""

    def __init__(self, ctx: Context, X, tets, facets, cdofs, material: Material):
        L = load_library()
        self.ctx = ctx
        self.X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1, 4)
        self.facets = np.ascontiguousarray(facets, dtype=np.int32).reshape(-1, 3)
        self.cdofs = np.ascontiguousarray(np.unique(np.asarray(cdofs, dtype=np.int64)), dtype=np.int32)
        self.material = material
        h = _vp()
        m = material.to_c()
        _check(L.od_scene_create(ctx.h, self.X.shape[0], _d(self.X), self.tets.shape[0], _i(self.tets),
                                 self.facets.shape[0], _i(self.facets), self.cdofs.size, _i(self.cdofs),
                                 C.byref(m), C.byref(h)), "od_scene_create")
        self.h = h
        _live_scenes.add(self)
        self.info = od_scene_info()
        _check(L.od_scene_get_info(self.h, C.byref(self.info)), "od_scene_get_info")
        self.dofs = self.info.dofs
        self.n_nodes = self.info.n_nodes
        self.n_tets = self.info.n_tets

    def close(self):
        if getattr(self, "h", None) and not _shutting_down:
            load_library().od_scene_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_values(self) -> int:
        return self.info.num_values

    def pattern(self):
        i = self.info
        nc = i.num_block_columns + i.num_remained_columns
        pcol = np.zeros(nc + 1, np.int32)
        rows = np.zeros(i.num_row_indices, np.int32)
        oris = np.zeros(nc + 1, np.int32)
        emap = np.zeros((self.n_tets, 78), np.int32)
        _check(load_library().od_scene_pattern(self.h, _i(pcol), _i(rows), _i(oris), _i(emap)), "pattern")
        return pcol, rows, oris, emap

    def set_displacements(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 3)
        _check(load_library().od_scene_set_displacements(self.h, _d(u)), "set_displacements")

    def plastic_strain(self):
        """Plastic strain of a corotational plastic scene, (n_tets, 9) row-major."""
        out = np.zeros((self.n_tets, 9))
        _check(load_library().od_scene_get_plastic_strain(self.h, _d(out)), "get_plastic_strain")
        return out

    def set_plastic_strain(self, plastic):
        p = np.ascontiguousarray(plastic, dtype=np.float64).reshape(self.n_tets, 9)
        _check(load_library().od_scene_set_plastic_strain(self.h, _d(p)), "set_plastic_strain")

    def info_now(self):
        """od_scene_get_info now (device_bytes grows with the first mixed solve)."""
        info = od_scene_info()
        _check(load_library().od_scene_get_info(self.h, C.byref(info)), "od_scene_get_info")
        return info

    def displacements(self):
        u = np.zeros((self.n_nodes, 3))
        _check(load_library().od_scene_get_displacements(self.h, _d(u)), "get_displacements")
        return u

    def getVertexPositions(self):
        xyz = np.zeros((self.n_nodes, 3), np.float32)
        _check(load_library().od_scene_get_positions(self.h, xyz.ctypes.data_as(C.POINTER(C.c_float))),
               "get_positions")
        return xyz

    def evaluate(self):
        """generateMatrixAndVirtualWorks: (tangent values, internal forces)."""
        v = np.zeros(self.n_values)
        f = np.zeros(self.dofs)
        _check(load_library().od_scene_evaluate(self.h, _d(v), _d(f)), "evaluate")
        return v, f

    def element_values(self):
        K = np.zeros((self.n_tets, 78))
        f = np.zeros((self.n_tets, 12))
        _check(load_library().od_scene_element_values(self.h, _d(K), _d(f)), "element_values")
        return K, f

    def mass(self):
        v = np.zeros(self.n_values)
        _check(load_library().od_scene_mass(self.h, _d(v)), "mass")
        return v

    def spmdv(self, values, x, y=None):
        values = np.ascontiguousarray(values, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.dofs) if y is None else np.array(y, dtype=np.float64)
        _check(load_library().od_scene_spmdv(self.h, _d(values), _d(x), _d(y)), "spmdv")
        return y

    def pcg(self, values, b, x0=None, solver: CGSolver | None = None):
        solver = solver or CGSolver()
        values = np.ascontiguousarray(values, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.dofs) if x0 is None else np.array(x0, dtype=np.float64)
        p = solver.to_c()
        st = od_solve_stats()
        _check(load_library().od_scene_pcg(self.h, _d(values), _d(b), _d(x), C.byref(p), C.byref(st)), "pcg")
        return x, st

    def ldlt_factor(self, values, sainv_eps=0.1, ldlt_eps=0.01):
        """InLDLTPreconditioner::Preprocess on A = values (reference layout);
        returns the factor in the reference's storage: (L values, L rows,
        pcol (dofs entries), inverted diagonal).  The factor stays with the
        scene for ldlt_apply."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        nnz = C.c_longlong(0)
        L = load_library()
        _check(L.od_scene_ldlt_factor(self.h, _d(values), float(sainv_eps), float(ldlt_eps), C.byref(nnz)),
               "ldlt_factor")
        n = nnz.value
        lv = np.zeros(max(n, 1))
        lr = np.zeros(max(n, 1), np.int32)
        pc = np.zeros(max(self.dofs, 1), np.int32)
        dinv = np.zeros(max(self.dofs, 1))
        _check(L.od_scene_ldlt_get(self.h, _d(lv), _i(lr), _i(pc), _d(dinv)), "ldlt_get")
        return lv[:n], lr[:n], pc[: self.dofs], dinv[: self.dofs]

    def ic_factor(self, values, eps=1e-3, relax=0.0):
        """InCholeskyPreconditioner::Preprocess on A = values (reference
        layout); returns (L values, L rows, pcol (dofs + 1)) in the
        reference's storage.  The factor stays with the scene for ic_apply."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        nnz = C.c_longlong(0)
        L = load_library()
        _check(L.od_scene_ic_factor(self.h, _d(values), float(eps), float(relax), C.byref(nnz)), "ic_factor")
        n = nnz.value
        lv = np.zeros(max(n, 1))
        lr = np.zeros(max(n, 1), np.int32)
        pc = np.zeros(self.dofs + 1, np.int32)
        _check(L.od_scene_ic_get(self.h, _d(lv), _i(lr), _i(pc)), "ic_get")
        return lv[:n], lr[:n], pc

    def ic_apply(self, rhs):
        """(L L^T)^-1 rhs on the device with the last ic_factor."""
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        out = np.zeros(self.dofs)
        _check(load_library().od_scene_ic_apply(self.h, _d(rhs), _d(out)), "ic_apply")
        return out

    def ldlt_apply(self, rhs):
        """(L D L^T)^-1 rhs on the device with the last ldlt_factor."""
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        out = np.zeros(self.dofs)
        _check(load_library().od_scene_ldlt_apply(self.h, _d(rhs), _d(out)), "ldlt_apply")
        return out

    def add_plane_damping(self, normal, constant, dampingCoefficient, elements, node_velocities=None):
        """MeshPlaneCollisionDampingForcer for each element against the plane
        normal.x + constant = 0, added to the external damping matrix
        (addExternalDampingForceMatrix); velocities: the integrator's unless
        given (n_nodes x 3)."""
        nrm = np.ascontiguousarray(normal, dtype=np.float64)
        el = np.ascontiguousarray(elements, dtype=np.int32)
        vel = None
        if node_velocities is not None:
            vel = np.ascontiguousarray(node_velocities, dtype=np.float64).reshape(-1)
        _check(load_library().od_scene_add_plane_damping(self.h, _d(nrm), float(constant), float(dampingCoefficient),
                                                          el.size, _i(el), _d(vel) if vel is not None else None),
               "add_plane_damping")

    def clear_damping(self):
        """clearExternalDampingForceMatrix."""
        _check(load_library().od_scene_clear_damping(self.h), "clear_damping")

    def damping_values(self):
        """The external damping matrix values (reference layout)."""
        v = np.zeros(self.n_values)
        _check(load_library().od_scene_get_damping(self.h, _d(v)), "damping_values")
        return v

    def set_loads(self, body=None, tractions=()):
        """Forcer: body force density (N/m^3) then (traction Pa, facet ids) groups."""
        ng = len(tractions)
        tv = np.zeros((max(ng, 1), 3))
        sizes = np.zeros(max(ng, 1), np.int32)
        ids = [np.zeros(0, np.int32)]
        for k, (t, fac) in enumerate(tractions):
            tv[k] = t
            fac = np.asarray(fac, dtype=np.int32)
            sizes[k] = fac.size
            ids.append(fac)
        ids = np.ascontiguousarray(np.concatenate(ids), dtype=np.int32)
        if ids.size == 0:
            ids = np.zeros(1, np.int32)
        b = None if body is None else np.ascontiguousarray(body, dtype=np.float64)
        _check(load_library().od_scene_set_loads(self.h, None if b is None else _d(b), ng, _d(tv), _i(sizes),
                                                 _i(ids)), "set_loads")

    def update_loads(self, traction_scale: float):
        """Re-evaluate the stored loads on the device with scaled tractions."""
        _check(load_library().od_scene_update_loads(self.h, float(traction_scale)), "update_loads")

    def set_traction_schedule(self, frequency_hz: float, phase: float = 0.0):
        """Scale tractions by sin(2 pi f t + phase) at the start of every step."""
        _check(load_library().od_scene_set_traction_schedule(self.h, float(frequency_hz), float(phase)),
               "set_traction_schedule")

    def set_external_forces(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        _check(load_library().od_scene_set_external_forces(self.h, _d(f)), "set_external_forces")

    def external_forces(self):
        f = np.zeros(self.dofs)
        _check(load_library().od_scene_get_external_forces(self.h, _d(f)), "get_external_forces")
        return f

    def setup_integrator(self, integrator):
        p = integrator.to_c()
        _check(load_library().od_integrator_setup(self.h, C.byref(p)), "integrator_setup")

    def update_integrator(self, integrator):
        """New integrator parameters (same kind), state kept."""
        p = integrator.to_c()
        _check(load_library().od_integrator_update(self.h, C.byref(p)), "integrator_update")

    def step(self, n: int = 1):
        st = od_step_stats()
        _check(load_library().od_step(self.h, n, C.byref(st)), "step")
        return st

    def state(self):
        d, v, a = np.zeros(self.dofs), np.zeros(self.dofs), np.zeros(self.dofs)
        _check(load_library().od_get_state(self.h, _d(d), _d(v), _d(a)), "get_state")
        return d, v, a

    def set_state(self, d=None, v=None, a=None):
        keep = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None for x in (d, v, a)]
        args = [None if k is None else _d(k) for k in keep]
        _check(load_library().od_set_state(self.h, *args), "set_state")

    def save(self) -> bytes:
        L = load_library()
        n = C.c_size_t(0)
        _check(L.od_scene_save(self.h, None, C.byref(n)), "save")
        buf = (C.c_char * n.value)()
        _check(L.od_scene_save(self.h, C.cast(buf, _vp), C.byref(n)), "save")
        return bytes(buf)

    def load(self, blob: bytes):
        buf = C.create_string_buffer(blob, len(blob))
        _check(load_library().od_scene_load(self.h, C.cast(buf, _vp), len(blob)), "load")


class LinearNewmark:
    """Modal (reduced) linear Newmark on a scene's mesh and constraints
    (intergrator/linearNewmark.{h,cpp}; od_modal_*): the n_modes lowest
    eigenpairs of the Hooke stiffness against the scene's consistent mass,
    then the reference's per-mode Newmark update.  The scene's density is
    the mass density; youngs and poisson are HookeMaterial's."""

    def __init__(self, scene: "Scene", n_modes: int, beta=0.25, gamma=0.5, massDamp=0.0, stiffDamp=0.0,
                 ts=1.0 / 60, youngs=None, poisson=None, tol=0.0, krylov=0, inner_tol=0.0,
                 inner_max_iter=0, max_restarts=0):
        L = load_library()
        self.scene = scene
        m = scene.material
        p = od_modal_params(int(n_modes), float(beta), float(gamma), float(massDamp), float(stiffDamp), float(ts),
                            float(m.youngs if youngs is None else youngs),
                            float(m.poisson if poisson is None else poisson), float(tol), int(krylov),
                            float(inner_tol), int(inner_max_iter), int(max_restarts))
        h = _vp()
        _check(L.od_modal_create(scene.h, C.byref(p), C.byref(h)), "od_modal_create")
        self.h = h
        self.n_modes = int(n_modes)
        _live_modals.add(self)

    def close(self):
        if getattr(self, "h", None) and not _shutting_down:
            load_library().od_modal_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setExternalVirtualWork(self, f_ext=None):
        """Modal forces of a compacted DOF vector, or of the scene's loads (None)."""
        f = None if f_ext is None else np.ascontiguousarray(f_ext, dtype=np.float64)
        if f is not None and f.size != self.scene.dofs:
            raise ValueError(f"f_ext must have {self.scene.dofs} entries")
        _check(load_library().od_modal_set_external_forces(self.h, _d(f) if f is not None else None),
               "od_modal_set_external_forces")

    def runOneTimeStep(self, steps: int = 1):
        _check(load_library().od_modal_step(self.h, int(steps)), "od_modal_step")

    def displacements(self):
        u = np.zeros((self.scene.n_nodes, 3))
        _check(load_library().od_modal_get_displacements(self.h, _d(u)), "od_modal_get_displacements")
        return u

    def velocities(self):
        v = np.zeros((self.scene.n_nodes, 3))
        _check(load_library().od_modal_get_velocities(self.h, _d(v)), "od_modal_get_velocities")
        return v

    def modes(self, basis=True):
        """(eigenvalues ascending, modes as rows of the compacted DOFs or None)."""
        lam = np.zeros(self.n_modes)
        ph = np.zeros((self.n_modes, self.scene.dofs)) if basis else None
        _check(load_library().od_modal_get_modes(self.h, _d(lam), _d(ph) if basis else None), "od_modal_get_modes")
        return lam, ph

    def state(self):
        d, v, a = (np.zeros(self.n_modes) for _ in range(3))
        _check(load_library().od_modal_get_state(self.h, _d(d), _d(v), _d(a)), "od_modal_get_state")
        return d, v, a

    def stiffness(self):
        """The assembled Hooke stiffness in the reference value layout."""
        k = np.zeros(self.scene.n_values)
        _check(load_library().od_modal_get_stiffness(self.h, _d(k)), "od_modal_get_stiffness")
        return k

    @property
    def info(self):
        i = od_modal_info()
        _check(load_library().od_modal_get_info(self.h, C.byref(i)), "od_modal_get_info")
        return i


class Batch:
    """Many scenes stepped together (od_batch_*): each scene advances exactly as
    Scene.step would, with one set of kernel launches and one mixed-precision
    solve per Newton iteration for the whole batch.  Scenes need a Newmark
    integrator with CGSolver(precision="mixed"), the same Newton count and the
    same preconditioner kind."""

    def __init__(self, ctx: Context, scenes):
        self.ctx = ctx
        self.scenes = list(scenes)
        arr = (_vp * len(self.scenes))(*[sc.h for sc in self.scenes])
        h = _vp()
        _check(load_library().od_batch_create(ctx.h, len(self.scenes), arr, C.byref(h)), "od_batch_create")
        self.h = h
        _live_batches.add(self)

    def step(self, n: int = 1):
        """Advance every scene n steps; returns one od_step_stats per scene."""
        st = (od_step_stats * len(self.scenes))()
        _check(load_library().od_batch_step(self.h, n, st), "od_batch_step")
        return list(st)

    def tuning(self) -> dict:
        t = od_mixed_tuning()
        _check(load_library().od_batch_get_tuning(self.h, C.byref(t)), "od_batch_get_tuning")
        return {"piece_steps": t.piece_steps, "consumer_warps": t.consumer_warps, "slice_cost": t.slice_cost}

    def set_tuning(self, piece_steps: int, slice_cost: float, consumer_warps: int = 12):
        t = od_mixed_tuning(int(piece_steps), int(consumer_warps), float(slice_cost))
        _check(load_library().od_batch_set_tuning(self.h, C.byref(t)), "od_batch_set_tuning")

    def tuning_key(self) -> str:
        """Device and mesh class of the batch: SM count, scene count and the
        scenes' total block rows and stored blocks, each rounded to two
        significant digits."""
        import math

        def r2(v):
            if v <= 0:
                return 0
            e = int(math.floor(math.log10(v))) - 1
            return int(round(v / 10 ** e) * 10 ** e)
        try:
            import torch
            sms = torch.cuda.get_device_properties(self.ctx.device).multi_processor_count
        except Exception:
            sms = f"dev{self.ctx.device}"
        nb = sum((sc.info.dofs + 2) // 3 for sc in self.scenes)
        nnzb = sum(sc.info.num_full_blocks for sc in self.scenes)
        return f"sm{sms}-scenes{r2(len(self.scenes))}-rows{r2(nb)}-blocks{r2(nnzb)}"

    def autotune(self, repeats: int = 1, cache: str | None = None) -> dict:
        """od_batch_autotune: picks the inner solve's tile shapes (ring-kernel
        piece size and consumer warps, partition slice cost) by timing the batch's last Newton
        system with every candidate; the batch must have been stepped once.
        With a cache file (JSON; default $OD_GB300_TUNE_CACHE when set) a
        choice made before for the same device and mesh class is reused."""
        import json
        cache = cache or os.environ.get("OD_GB300_TUNE_CACHE")
        key = self.tuning_key()
        table = {}
        if cache and os.path.exists(cache):
            with open(cache) as f:
                table = json.load(f)
        if key in table:
            self.set_tuning(table[key]["piece_steps"], table[key]["slice_cost"], table[key]["consumer_warps"])
            return {"key": key, "cached": True, **table[key]}
        rep = od_tune_report()
        _check(load_library().od_batch_autotune(self.h, int(repeats), C.byref(rep)), "od_batch_autotune")
        out = {"piece_steps": rep.best.piece_steps, "consumer_warps": rep.best.consumer_warps,
               "slice_cost": rep.best.slice_cost,
               "candidates": rep.candidates, "default_ms": rep.default_ms, "best_ms": rep.best_ms,
               "default_iters": rep.default_iters, "best_iters": rep.best_iters}
        if cache:
            table[key] = out
            os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
            with open(cache, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
        return {"key": key, "cached": False, **out}

    def close(self):
        if getattr(self, "h", None) and not _shutting_down:
            load_library().od_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulator:
    """Simulator(mesh, indexer, integrator) (core/simulator.h:15-16)."""

    def __init__(self, scene: Scene, integrator):
        self.scene = scene
        scene.setup_integrator(integrator)

    def runTimeSteps(self, stepCount: int):
        return self.scene.step(stepCount)

    def getVertexPositions(self):
        return self.scene.getVertexPositions()
