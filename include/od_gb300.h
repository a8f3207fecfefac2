/*
 * od_gb300.h -- C ABI of the GB300-native implicit FEM time step.
 *
 * Plain C types only (no CUDA or torch types).  Host pointers in, device-
 * resident state inside.  Every call returns an od_status; od_last_error()
 * gives a message for the calling thread.  One context per host thread;
 * scenes are not shared across threads without external locking (the
 * reference is single-threaded and not re-entrant either).
 *
 * Reference interfaces replaced (paths inside OpenDeformer/):
 *   FullOrderNonlinearMaterial<SpMatrix>   material/fullOrderNonlinear.h:36-44
 *   MechMaterial::generateMassMatrix       core/mechMaterial.h:31-32
 *   BlockedSymSparseMatrix + SpMDV         core/sparseMatrix.h:183-274, core/numerMethod.h:134-262
 *   LinearSolver / CGSolver                core/linearSolver.h:12-20, solver/cgSolver.h:16-17
 *   Preconditioner (+ Jacobi, IC)          core/preconditioner.h:12-22
 *   InLDLTPreconditioner                   solver/inLDLTPreconditioner.h:12-44
 *   InCholeskyPreconditioner               solver/inCholeskyPreconditioner.h
 *   Forcer                                 core/forcer.h:13-22
 *   MeshPlaneCollisionDampingForcer        collision/penaltyDampingForcer.h:25-35
 *   MeshRelabeler                          core/meshRelabeler.h:103-135
 *   Intergrator / NonlinearImplicitBackwardEuler
 *                                          core/intergrator.h:13-35,
 *                                          intergrator/nonlinearImplicitBackwardEuler.h:48-128
 *   Simulator::runTimeSteps / getVertexPositions  core/simulator.h:21-22
 */
#ifndef OD_GB300_H
#define OD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OD_ABI_VERSION 6

typedef enum od_status {
  OD_OK = 0,
  OD_ERR_INVALID_ARG = 1,
  OD_ERR_OUT_OF_MEMORY = 2,
  OD_ERR_NOT_CONVERGED = 3, /* PCG hit max_iter (the reference exits silently) */
  OD_ERR_NAN = 4,           /* non-finite residual or state */
  OD_ERR_DEVICE_TIMEOUT = 5,/* a bounded device wait ran out */
  OD_ERR_CUDA = 6,
  OD_ERR_UNSUPPORTED = 7,
  OD_ERR_INTERNAL = 8
} od_status;

typedef enum od_material_kind {
  OD_MATERIAL_COROTATIONAL = 0, /* material/corotationalHyperelastic.h:11-21 */
  OD_MATERIAL_NEOHOOKEAN = 1,   /* material/invertibleNeoHookean.h */
  OD_MATERIAL_STVK = 2,         /* material/invertibleStVK.h */
  OD_MATERIAL_COROTATIONAL_PLASTIC = 3  /* material/corotationalPlastic.h:11-30 */
} od_material_kind;

typedef enum od_precond_kind {
  OD_PRECOND_NONE = 0,         /* Preconditioner (identity), core/preconditioner.h:14-16 */
  OD_PRECOND_JACOBI = 1,       /* solver/jacobiPreconditioner.cpp:12-26 */
  OD_PRECOND_BLOCK_JACOBI = 2, /* 3x3 diagonal blocks (no reference counterpart) */
  OD_PRECOND_IC0 = 3,          /* shifted IC(0), level-scheduled (no reference counterpart;
                                  the reference's fill-in IC is inCholeskyPreconditioner.cpp) */
  OD_PRECOND_LDLT = 4,         /* incomplete LDL^T, solver/inLDLTPreconditioner.cpp:34-184:
                                  factor on the host (bit-identical to the reference's),
                                  triangular sweeps on the device */
  OD_PRECOND_IC = 5            /* threshold incomplete Cholesky with fill,
                                  solver/inCholeskyPreconditioner.cpp:18-162: factor on the host
                                  (bit-identical to the reference's), sweeps on the device */
} od_precond_kind;

typedef enum od_precision {
  OD_PRECISION_FP64 = 0,  /* plain FP64 everywhere */
  OD_PRECISION_MIXED = 1  /* FP32 matrix/SpMV/preconditioner apply; FP64 dots, residual
                             replacement and outer iterative refinement */
} od_precision;

typedef enum od_integrator_kind {
  OD_INTEGRATOR_BACKWARD_EULER = 0, /* nonlinearImplicitBackwardEuler.h:82-116 */
  OD_INTEGRATOR_NEWMARK = 1         /* full-order Newmark + Newton (formulas of
                                       intergrator/linearNewmark.cpp:27-30,57-79) */
} od_integrator_kind;

typedef struct od_material {
  int kind;          /* od_material_kind */
  double density;    /* rho, kg/m^3 */
  double youngs;     /* E, Pa */
  double poisson;    /* nu */
  double threshold;  /* corotational compressing threshold / invertible inversion threshold */
  /* corotational plastic only (CorotationalPlasticMaterial ctor,
     corotationalPlastic.cpp:8-22): */
  double yield_criterion;     /* elastic-strain norm above which plastic strain grows */
  double creep_ratio;         /* share of the excess strain moved to plastic strain per evaluation */
  double max_plastic_strain;  /* cap on the plastic-strain norm */
} od_material;

typedef struct od_solver_params {
  double tol;         /* stop when ||r||^2 <= tol^2 ||b||^2 (cgSolver.cpp:42-46) */
  int max_iter;
  int precond;        /* od_precond_kind */
  int precision;      /* od_precision */
  int replace_every;  /* mixed: true-residual recompute period (0 = 25) */
  double inner_tol;   /* mixed: inner FP32 solve tolerance (0 = 1e-4) */
  int max_refine;     /* mixed: max outer refinement sweeps (0 = 20) */
  double sainv_eps;   /* LDL^T: sainvEpsilon, drop bound of the inverse factor's
                         entries (0 = 0.1; InLDLTPreconditioner(sainvEpsilon, ldltEpsilon)) */
  double ldlt_eps;    /* LDL^T: ldltEpsilon, drop bound of L's entries (0 = 0.01) */
  double ic_eps;      /* IC: epsilon of InCholeskyPreconditioner(epsilon, relaxedScale) (0 = 1e-3) */
  double ic_relax;    /* IC: relaxedScale, taken as given (0: dropped entries are not compensated) */
} od_solver_params;

typedef struct od_solve_stats {
  int iterations;       /* total inner iterations */
  int refinements;      /* mixed: outer sweeps */
  double rel_residual;  /* ||b - A x|| / ||b|| at exit (FP64) */
  double ic_shift;      /* IC(0) diagonal shift used */
  int status;           /* od_status of the solve */
} od_solve_stats;

typedef struct od_integrator_params {
  int kind;              /* od_integrator_kind */
  double dt;             /* time step h */
  double alpha_m;        /* Rayleigh mass damping */
  double beta_k;         /* Rayleigh stiffness damping */
  double nm_beta;        /* Newmark beta (0.25) */
  double nm_gamma;       /* Newmark gamma (0.5) */
  int newton_iters;      /* Newmark Newton iterations per step (>= 1) */
  od_solver_params solver;
} od_integrator_params;

typedef struct od_step_stats {
  int steps;
  int pcg_iterations;    /* summed over solves */
  int solves;
  double max_rel_residual;
  int status;
  double device_ms;      /* CUDA-event time on the context stream, first launch to last */
} od_step_stats;

/* Launch and timing counters of a context (no reference counterpart). */
typedef struct od_counters {
  long long kernel_launches;  /* every kernel this library launched */
  long long host_syncs;       /* stream synchronisations inside library calls */
  long long spmv_launches;    /* PCG SpMV launches timed while profiling is on */
  double spmv_ms;             /* their summed CUDA-event durations */
  long long pcg_launches;     /* persistent (one-launch) PCG solves timed while profiling */
  long long pcg_iterations;   /* their iterations */
  double pcg_ms;              /* their summed CUDA-event durations */
  long long mix_iterations;   /* inner FP32 PCG loop iterations of mixed solves (profiling on) */
  double mix_spmv_ms;         /* their SpMV + p.q phase, start to end of the grid-wide sum */
  double mix_spmv_bytes;      /* algorithmic bytes of those phases: stored blocks x 40 B
                                 (FP32 values + column index) + 24 B per block row (own p
                                 read, q written), for the scenes active in each iteration */
  double mix_spmv_work_ms;    /* the same phases up to the moment the last CTA finished its
                                 SpMV work (without the grid-wide sum that follows) */
  long long mix_fallbacks;    /* mixed solves whose refinement stalled and that the FP64 PCG
                                 finished (counted whether profiling is on or not) */
  /* preconditioners applied by triangular sweeps (LDL^T, IC): */
  long long sweep_factors;    /* host factorisations (always counted) */
  double sweep_factor_ms;     /* their host time: rebuild of A in the reference layout, the
                                 factorisation and the upload of the sweep arrays */
  long long sweep_nnz;        /* strictly lower entries of the last factor */
  long long sweep_applies;    /* applies timed while profiling is on */
  double sweep_apply_ms;      /* their summed CUDA-event durations */
  double sweep_apply_bytes;   /* their algorithmic bytes: 2 x (nnz x 12 B) + 7 x 8 B per row */
  long long sweep_levels;     /* dependency levels of the last factor's two sweeps (the apply's
                                 critical path, in rows) */
  /* persistent PCG iterations timed phase by phase while profiling (the clock of
     CTA 0, whose share of the rows equals every CTA's): [0] SpMV and p.q, [1] the
     grid-wide sum of p.q (the wait for the slowest CTA included), [2] x, r, z
     updates with r.z and r.r, [3] their sum, [4] p = z + beta p, [5] the barrier
     before the next SpMV */
  double pcg_phase_ms[6];
  long long pcg_phase_iterations;
  /* the same solves, each CTA's own SpMV, update and direction work (its warps'
     time, without the waits): per solve the slowest CTA's and the mean over CTAs */
  double pcg_work_max_ms[3];
  double pcg_work_mean_ms[3];
  double mix_fallback_ms;     /* host wall time of the FP64 solves that finished stalled mixed
                                 solves (counted whether profiling is on or not) */
} od_counters;

typedef struct od_scene_info {
  int n_nodes, n_tets, n_facets;
  int dofs;                  /* compacted DOF count (NodeIndexer::getMatrixOrder) */
  int num_block_columns;     /* reference numBlockColumn */
  int num_remained_columns;  /* reference numRemainedColumn */
  int num_row_indices;       /* reference blockPcol[last] */
  int num_values;            /* reference blockColumnOris[last] */
  int num_full_blocks;       /* device full-BSR block count (both triangles) */
  int num_colors;            /* element colours used by the atomic-free scatter */
  long long device_bytes;    /* device memory held by the scene */
  int pcg_smem_bytes;        /* shared memory per CTA of the one-launch PCG when it keeps the
                                matrix rows on chip (0: it reads them from L2 / HBM) */
} od_scene_info;

typedef struct od_ctx od_ctx;
typedef struct od_scene od_scene;

const char* od_status_string(od_status s);
const char* od_last_error(void);
int od_abi_version(void);

/* Context: one CUDA device and stream.  Replaces nothing in the reference
 * (it has no device); owns the stream every call of its scenes runs on. */
od_status od_ctx_create(int device, od_ctx** out);
od_status od_ctx_destroy(od_ctx* ctx);
od_status od_ctx_synchronize(od_ctx* ctx);
/* Failure detection, tested without a GPU fault: runs the bounded device
 * waits against conditions that never clear -- the two grid barriers (the
 * generation barrier and the one-launch PCG's counting barrier) with a CTA
 * that never reaches them, a triangular-sweep wait on a value nobody
 * writes -- and reports
 * whether each ran out and raised its timeout flag (the flag the calls
 * above turn into OD_ERR_DEVICE_TIMEOUT).  Takes a few seconds; the context
 * stays usable. */
od_status od_selftest_bounded_waits(od_ctx* ctx, int* barrier_timed_out, int* value_wait_timed_out);
/* Multiply-add throughput of the context's device (no reference
 * counterpart): fixed chains of independent multiply-adds on every SM at full
 * occupancy, iters per chain, timed with CUDA events on the context stream
 * (best of three launches after one warm-up).  fp64 = 1 measures FP64, 0
 * FP32; *fma_per_s receives multiply-adds per second (2 operations each),
 * *ms the launch time.  The roofline of the FP64 kernels. */
od_status od_measure_fma_rate(od_ctx* ctx, int fp64, int iters, double* fma_per_s, double* ms);
/* Counters (no reference counterpart).  enable = 1: every PCG launch is
 * bracketed by CUDA events on the context stream (and the mixed solve's
 * kernel records its phase times); 2: also the one-launch FP64 PCG's
 * per-iteration phase timers (pcg_phase_ms, pcg_work_*), which add clock
 * reads and a CTA barrier to every iteration; 0: off. */
od_status od_ctx_set_profiling(od_ctx* ctx, int enable);
od_status od_ctx_get_counters(od_ctx* ctx, od_counters* out);
od_status od_ctx_reset_counters(od_ctx* ctx);

/* Scene = TetMesh + Constrainer/NodeIndexer + material + pattern + caches.
 * Replaces TetMesh(numN, numE, numS) + setVertex/setElement/setFacet
 * (mesh/tetmesh.h:12, core/mesh.cpp:7-40), NodeIndexer(constrainer)
 * (core/nodeIndexer.cpp:8-10), material ctor + getPrecomputes +
 * getMatrixStructure + getMatrixIndicesPerElement + generateMassMatrix
 * (material/fullOrderNonlinear.h:36-110, core/mechMaterial.cpp:69-98).
 *   X: n_nodes*3 rest positions; tets: n_tets*4; facets: n_facets*3;
 *   cdofs: sorted constrained DOFs 3*node+axis (Constrainer output). */
od_status od_scene_create(od_ctx* ctx, int n_nodes, const double* X, int n_tets, const int* tets,
                          int n_facets, const int* facets, int n_cdofs, const int* cdofs,
                          const od_material* material, od_scene** out);
od_status od_scene_destroy(od_scene* scene);
od_status od_scene_get_info(od_scene* scene, od_scene_info* info);

/* Pattern export, bit-identical to BlockedSymSparseMatrix's blockPcol /
 * blockRows / blockColumnOris (core/sparseMatrix.h:186-274) and to the
 * element->value map of getMatrixIndicesPerElement (fullOrderNonlinear.h:73-110,
 * 78 ints per tet, -1 for constrained).  Any output may be NULL. */
od_status od_scene_pattern(od_scene* scene, int* block_pcol, int* block_rows,
                           int* block_column_oris, int* elem_map);

/* Mesh displacement (Mesh::getVertexDisplacement, core/mesh.h:38-39), n_nodes*3.
 * Constrained DOFs keep what is written here (prescribed displacements). */
od_status od_scene_set_displacements(od_scene* scene, const double* u);
od_status od_scene_get_displacements(od_scene* scene, double* u);
/* Simulator::getVertexPositions (core/simulator.cpp:24-33): X + u as float. */
od_status od_scene_get_positions(od_scene* scene, float* xyz);

/* FullOrderNonlinearMaterial::generateMatrixAndVirtualWorks
 * (corotationalHyperelastic.cpp:43-102, invertibleHyperelastic.cpp:34-114):
 * tangent values in the reference value layout and internal forces (dofs),
 * at the current mesh displacement.  Outputs may be NULL (device only). */
od_status od_scene_evaluate(od_scene* scene, double* values, double* f_int);
/* Per-element 78 packed stiffness values and 12 nodal forces (element order). */
od_status od_scene_element_values(od_scene* scene, double* k78, double* f12);
/* MechMaterial::generateMassMatrix values (mechMaterial.cpp:69-98). */
od_status od_scene_mass(od_scene* scene, double* values);

/* SpMDV (numerMethod.h:134-262): y += A x, A given by reference-layout values. */
od_status od_scene_spmdv(od_scene* scene, const double* values, const double* x, double* y);
/* CGSolver::solveLinearSystem (cgSolver.cpp:13-57) on A (reference-layout
 * values); x is the warm start and the result. */
od_status od_scene_pcg(od_scene* scene, const double* values, const double* b, double* x,
                       const od_solver_params* params, od_solve_stats* stats);

/* InLDLTPreconditioner (solver/inLDLTPreconditioner.cpp) as a stand-alone
 * preconditioner.  od_scene_ldlt_factor is Preprocess (:27-149) on A given by
 * reference-layout values, with InLDLTPreconditioner(sainv_eps, ldlt_eps)'s
 * drop bounds taken as given (>= 0); *nnz receives the stored L entries.
 * od_scene_ldlt_get copies the factor out in the reference's storage:
 * values[nnz], rows[nnz], pcol[dofs] (L columns 0..dofs-2), inv_diag[dofs].
 * od_scene_ldlt_apply is solvePreconditionerSystem (:151-184) on the device
 * with the last factor: result = (L D L^T)^-1 rhs (dofs entries each). */
od_status od_scene_ldlt_factor(od_scene* scene, const double* values, double sainv_eps, double ldlt_eps,
                               long long* nnz);
od_status od_scene_ldlt_get(od_scene* scene, double* values, int* rows, int* pcol, double* inv_diag);
od_status od_scene_ldlt_apply(od_scene* scene, const double* rhs, double* result);
/* InCholeskyPreconditioner (solver/inCholeskyPreconditioner.cpp) the same
 * way: od_scene_ic_factor is Preprocess (:76-130) with
 * InCholeskyPreconditioner(eps, relax) (both >= 0; dofs >= 2); *nnz receives
 * the stored entries, diagonals included.  od_scene_ic_get copies the factor
 * out in the reference's storage: values[nnz], rows[nnz] (column c holds its
 * diagonal, then its rows below ascending), pcol[dofs + 1].
 * od_scene_ic_apply is solvePreconditionerSystem (:132-162) on the device:
 * result = (L L^T)^-1 rhs. */
od_status od_scene_ic_factor(od_scene* scene, const double* values, double eps, double relax, long long* nnz);
od_status od_scene_ic_get(od_scene* scene, double* values, int* rows, int* pcol);
od_status od_scene_ic_apply(od_scene* scene, const double* rhs, double* result);

/* Collision damping (collision/penaltyDampingForcer.cpp:8-61,
 * intergrator/nonlinearImplicitBackwardEuler.h:122-128).
 * od_scene_add_plane_damping is MeshPlaneCollisionDampingForcer: for every
 * element of elems (original element ids; an id listed twice is added
 * twice) against the plane normal.x + constant = 0 it adds the forcer's
 * damping block to the scene's external damping matrix, at the current
 * displacements, with node velocities node_velocities (n_nodes x 3) or,
 * when NULL, the integrator's current velocities (constrained DOFs 0, as
 * getMeshVerticesVelocities gives them) -- addExternalDampingForceMatrix.
 * od_scene_clear_damping is clearExternalDampingForceMatrix.  Both
 * integrators use the matrix (backward Euler as the reference does; the
 * Newmark step in C = alpha_M M + beta_K K + D). */
od_status od_scene_add_plane_damping(od_scene* scene, const double* normal, double constant, double damping,
                                     int n_elems, const int* elems, const double* node_velocities);
od_status od_scene_clear_damping(od_scene* scene);
/* the external damping matrix values (reference layout, num_values entries) */
od_status od_scene_get_damping(od_scene* scene, double* values);

/* Forcer + Intergrator::setExternalVirtualWork (core/forcer.cpp:8-96,
 * nonlinearImplicitBackwardEuler.h:118-120): body force density (N/m^3, may be
 * NULL) then n_groups uniform tractions (Pa) over facet lists, evaluated on
 * the device at the current displacement (deformed facet areas).  Loads stay
 * frozen until the next call. */
od_status od_scene_set_loads(od_scene* scene, const double* body, int n_groups,
                             const double* tractions, const int* group_sizes,
                             const int* facet_ids);
/* Re-evaluates the loads of the last od_scene_set_loads at the current
 * displacement with every traction scaled by traction_scale, on the device
 * (the per-step Forcer rebuild of a time-varying traction, without host
 * copies). */
od_status od_scene_update_loads(od_scene* scene, double traction_scale);
/* Time-varying traction: when frequency_hz > 0 every od_step step first
 * re-evaluates the loads (as od_scene_update_loads) with the tractions scaled
 * by sin(2 pi frequency_hz t + phase), t the end time of that step -- the
 * per-step Forcer rebuild of a periodic surface load.  frequency_hz = 0 turns
 * it off (loads stay frozen). */
od_status od_scene_set_traction_schedule(od_scene* scene, double frequency_hz, double phase);
od_status od_scene_set_external_forces(od_scene* scene, const double* f_ext);
od_status od_scene_get_external_forces(od_scene* scene, double* f_ext);

/* Integrator (NonlinearImplicitBackwardEuler ctor, nonlinearImplicitBackwardEuler.h:48-73,
 * or the full-order Newmark).  Resets the state to rest. */
od_status od_integrator_setup(od_scene* scene, const od_integrator_params* params);

/* Plastic strain of a corotational plastic scene, 9 per element (row-major),
 * in the caller's element order.  The reference keeps it in the material's
 * precompute cache (corotationalPlastic.cpp:46-47) and updates it at every
 * evaluation of the element forces. */
od_status od_scene_get_plastic_strain(od_scene* scene, double* plastic);
od_status od_scene_set_plastic_strain(od_scene* scene, const double* plastic);
/* Change the parameters of the set-up integrator (same kind) and keep the
 * state (d, v, a, time); no reference counterpart (the reference fixes them
 * in the integrator's constructor). */
od_status od_integrator_update(od_scene* scene, const od_integrator_params* params);
/* Simulator::runTimeSteps (simulator.cpp:35-38): n steps, each followed by the
 * mesh displacement update (updateMeshVerticesDisplacements,
 * nonlinearImplicitBackwardEuler.h:103-116). */
od_status od_step(od_scene* scene, int n_steps, od_step_stats* stats);
/* State vectors over the compacted DOFs (any may be NULL).  Backward Euler
 * has v only (d and a are reported as zero). */
od_status od_get_state(od_scene* scene, double* d, double* v, double* a);
od_status od_set_state(od_scene* scene, const double* d, const double* v, const double* a);

/* ---- batches: many scenes stepped together on one GPU.  No reference
 * counterpart (the reference steps one Simulator at a time,
 * core/simulator.h:21-22); each scene advances by exactly the od_step
 * sequence, with a fixed number of kernel launches per step for the whole
 * batch and one mixed-precision solve (per-scene step lengths and
 * convergence) per Newton iteration.  Every scene of a batch shares ctx, has
 * a Newmark integrator with the mixed-precision solver, the same Newton count
 * and the same preconditioner kind (none, Jacobi, block-Jacobi), and no
 * external damping.  A batch owns device memory of its own (the scenes'
 * concatenated FP32 systems, about 40 bytes per stored block); the scenes
 * keep their state and may be stepped alone or in other batches between
 * calls, never concurrently. */
typedef struct od_batch od_batch;
od_status od_batch_create(od_ctx* ctx, int n_scenes, od_scene* const* scenes, od_batch** out);
/* stats: n_scenes entries (or NULL), in the order of od_batch_create;
 * device_ms is the time of the whole call */
od_status od_batch_step(od_batch* batch, int n_steps, od_step_stats* stats);
od_status od_batch_destroy(od_batch* batch);
/* Tile shapes of a batch's inner FP32 solve (no reference counterpart):
 * the ring kernel's piece size (matrix steps per bulk copy into shared
 * memory: 12, 16 or 20), its consumer warps per CTA (12, or 15 with pieces of
 * 12 or 16 steps) -- by default 12 and 15 for the lower-triangle matrix, 20
 * and 12 for both triangles -- and the per-slice fixed cost, in steps, that
 * weights the partition of the slices over the CTAs (default 8).  The
 * report's default_ms is the solve with the shape set before tuning. */
typedef struct od_mixed_tuning {
  int piece_steps;
  int consumer_warps;
  double slice_cost;
} od_mixed_tuning;
typedef struct od_tune_report {
  int candidates;
  od_mixed_tuning best;
  double default_ms, best_ms;    /* solve time of the default and of the chosen shapes */
  int default_iters, best_iters; /* their inner iterations (summed over scenes) */
} od_tune_report;
od_status od_batch_get_tuning(od_batch* batch, od_mixed_tuning* out);
od_status od_batch_set_tuning(od_batch* batch, const od_mixed_tuning* tuning);
/* Autotuner: after at least one od_batch_step, solves the batch's last
 * Newton system again with every candidate shape (5 piece-size / consumer-
 * warp pairs x slice costs 2, 4, 8, 16), each timed with CUDA events (best of
 * repeats), and keeps the fastest.  Scene state is not changed. */
od_status od_batch_autotune(od_batch* batch, int repeats, od_tune_report* report);

/* ---- serving: step requests over a pool of scenes.  No reference
 * counterpart (the reference steps one Simulator at a time,
 * core/simulator.h:21-22).  A request is one Newmark step of one scene with
 * its own time step, body force density and surface traction.  Every
 * od_server_tick takes the oldest pending request of each scene (oldest
 * first, at most max_batch), and steps the resident scenes among them
 * together (batched: one od_batch step with the scenes' mixed-precision
 * solvers; plain: od_step scene by scene).  Requests arriving meanwhile join
 * a later tick (continuous batching at step granularity).  Scenes stay on
 * the device while the byte budget allows; a request for a scene that is not
 * resident evicts least-recently-used scenes the tick does not step (to a
 * host checkpoint, as od_scene_save) and admits the scene: with
 * admission_thread = k > 0, k host worker threads with contexts of their own
 * build admitted scenes in parallel while ticks run, and each joins a later
 * tick; with 0 the tick builds it before stepping.  The server belongs to the thread that created it (its
 * context's thread); the worker only builds scenes. */
typedef struct od_server od_server;
typedef struct od_server_config {
  long long budget_bytes;   /* device bytes the resident scenes may hold (<= 0: free memory less reserve_bytes) */
  long long reserve_bytes;  /* kept free when budget_bytes <= 0 */
  int max_batch;            /* scenes stepped per tick at most (0: no limit) */
  int batched;              /* 1: one batch step per tick; 0: scene by scene (plain path) */
  int admission_thread;     /* host worker threads that build admitted scenes (0: the tick builds them) */
} od_server_config;
typedef struct od_scene_spec {
  int n_nodes;
  const double* X;          /* n_nodes x 3 */
  int n_tets;
  const int* tets;          /* n_tets x 4 */
  int n_facets;
  const int* facets;        /* n_facets x 3 */
  int n_cdofs;
  const int* cdofs;         /* sorted constrained DOFs */
  int n_load_facets;
  const int* load_facets;   /* facets that take each request's traction */
  od_material material;
  od_integrator_params integrator;  /* Newmark; each request sets dt */
} od_scene_spec;
typedef struct od_step_request {
  int scene;
  double dt;
  double body[3];           /* body force density, N/m^3 */
  double traction[3];       /* Pa, on the scene's load facets */
  double arrival;           /* seconds on the server clock (od_server_now) */
} od_step_request;
typedef struct od_step_result {
  long long ticket;
  int scene;
  int status;               /* od_status of the step */
  int pcg_iterations;
  double arrival, done;     /* server clock */
} od_step_result;
typedef struct od_server_stats {
  long long ticks, steps, admissions, restores, evictions, deferred;
  double s_admit;           /* caller's thread: adoption, eviction and (without the worker) building */
  double s_loads;           /* request parameters and loads */
  double s_step;            /* batch / scene steps */
  double s_worker;          /* worker thread: building scenes (overlaps the ticks) */
  long long resident, resident_bytes, budget_bytes;
  double s_build;           /* of s_step: building and freeing the tick's batch */
  double s_device;          /* device time of the steps (CUDA events around each batch or scene step) */
} od_server_stats;
od_status od_server_create(od_ctx* ctx, const od_server_config* cfg, od_server** out);
od_status od_server_destroy(od_server* server);
/* registers a scene (copies the arrays); all scenes before the first request */
od_status od_server_add_scene(od_server* server, const od_scene_spec* spec, int* scene_id);
/* seconds since the server was created */
od_status od_server_now(od_server* server, double* t);
od_status od_server_submit(od_server* server, const od_step_request* req, long long* ticket);
/* one tick; results receives at most capacity completed requests (capacity
 * also caps the scenes stepped).  When the tick's step fails as a call, the
 * requests it had taken come back in results with that status and the
 * call returns it. */
od_status od_server_tick(od_server* server, int capacity, od_step_result* results, int* n_results);
od_status od_server_pending(od_server* server, long long* pending);
/* makes scenes resident (in order, on the caller's thread) while they fit without eviction */
od_status od_server_warm(od_server* server, int n, const int* scene_ids, int* admitted);
/* the scene of scene_id, made resident first if it is not (built on the
 * caller's thread, evicting as the budget requires); the server keeps it:
 * the handle is valid until the next od_server_tick or od_server_destroy */
od_status od_server_get_scene(od_server* server, int scene_id, od_scene** out);
od_status od_server_get_stats(od_server* server, od_server_stats* out);

/* Allocation-free PCG.  No counterpart in the reference.  For callers that
 * cannot allocate device memory -- a host application whose own allocator
 * owns the GPU's memory, or a plugin whose host forbids allocation once it
 * is running -- this solves A x = b with the none, Jacobi or block-Jacobi
 * preconditioner (FP64) for a full block-CSR matrix the caller already holds
 * on the device: nb block rows, row pointers d_row_ptr[nb+1] (starting at 0,
 * d_row_ptr[nb] = the length of d_col), block columns d_col[] in 0..nb-1,
 * 9 row-major values per 3x3 block in d_values[]; d_b and d_x have 3*nb
 * entries, d_x is the warm start and the result.  A malformed structure is
 * detected on the device before it is used and returns OD_ERR_INVALID_ARG.
 * Every work vector lives in one fixed device array inside the library
 * (OD_NOALLOC_MAX_BLOCK_ROWS block rows at most, about 5.5 MB, held by every
 * GPU that loads the library until exit); the call allocates nothing.
 * Larger systems are rejected with OD_ERR_INVALID_ARG.  The call is
 * synchronous: it waits on the stream to test convergence and returns when
 * the solve is done (stats->status OD_ERR_NOT_CONVERGED, with OD_OK
 * returned, when max_iter ran out).  The array is shared: calls that overlap
 * on the GPU race, so callers serialise them.  The first call on a device
 * looks up the array's device address and keeps it for the process (a
 * cudaDeviceReset after it is not supported).  stream is a cudaStream_t
 * (NULL: the default stream). */
#define OD_NOALLOC_MAX_BLOCK_ROWS 32768
od_status od_bsr_pcg_noalloc(int nb, const int* d_row_ptr, const int* d_col, const double* d_values,
                             const double* d_b, double* d_x, const od_solver_params* params,
                             void* stream, od_solve_stats* stats);

/* MeshRelabeler::getNewLables (core/meshRelabler.cpp:192-505) on the host,
 * before a scene is created: Gibbs-Poole-Stockmeyer relabeling of the nodes of
 * n_elems elements of nodes_per_elem nodes (elems[n_elems * nodes_per_elem]).
 * new_labels[old node] receives the new label; elems is rewritten with the new
 * labels and reordered by the sum of each element's labels.  Ties go to the
 * lower node index (deterministic; the reference's follow its standard
 * library's hash and heap orders); every connected component is labelled
 * (the reference labels the first only); nodes in no element go last.
 * Node arrays (positions, constraints, facets) are the caller's to permute. */
od_status od_mesh_relabel(int n_nodes, int n_elems, int nodes_per_elem, int* elems, int* new_labels);

/* ---- modal (reduced) linear Newmark: intergrator/linearNewmark.{h,cpp}.
 * LinearNewmark::LinearNewmark (linearNewmark.cpp:8-50) assembles the linear
 * (Hooke) stiffness K (material/hooke.cpp:18-60) and the consistent mass M of
 * the scene's mesh and constraints, and keeps the n_modes eigenpairs
 * K phi = lambda M phi of smallest lambda (EigenSolver::getEigenValVectors,
 * core/eigensolver.cpp:8-13: ARPACK's shift-invert mode at 0).  Here the
 * eigenpairs come from a thick-restart Lanczos iteration on K^-1 M in the M
 * inner product, with every K^-1 applied by the FP64 block-Jacobi PCG on the
 * device; modes are M-orthonormal and ordered by ascending lambda.  The scene
 * supplies mesh, constraints, density and the loads of od_scene_set_loads;
 * its own integrator and displacement are not used or changed. */
typedef struct od_modal od_modal;
typedef struct od_modal_params {
  int n_modes;            /* LinearNewmark's DOFS: modes kept (1 <= n_modes < scene dofs) */
  double beta, gamma;     /* Newmark parameters */
  double alpha_m, beta_k; /* Rayleigh damping: massDamp, stiffDamp */
  double dt;              /* time step */
  double youngs, poisson; /* HookeMaterial(rho, YOUNGS, POSSION); rho is the scene's density */
  double tol;             /* eigenpair residual ||K^-1 M phi - phi / lambda||_M relative to
                             1 / lambda; 0: 1e-10 */
  int krylov;             /* Lanczos basis size (> n_modes + 1); 0: max(2 n_modes + 10, n_modes + 20),
                             at most the scene dofs */
  double inner_tol;       /* PCG tolerance of each K^-1 apply; 0: 1e-12 */
  int inner_max_iter;     /* 0: 100000 */
  int max_restarts;       /* 0: 200 */
} od_modal_params;

typedef struct od_modal_info {
  int n_modes;
  int dofs;
  int krylov;
  int lanczos_steps;       /* K^-1 M applies */
  int restarts;
  long long pcg_iterations;  /* summed over the applies */
  double max_residual;     /* largest relative eigenpair residual at exit */
  double setup_ms;         /* wall time of od_modal_create */
} od_modal_info;

od_status od_modal_create(od_scene* scene, const od_modal_params* params, od_modal** out);
od_status od_modal_destroy(od_modal* modal);
/* setExternalVirtualWork (linearNewmark.cpp:52-55, forcer.cpp:80-96): the
 * modal forces phi_i . f_ext of a compacted DOF vector (NULL: the scene's
 * current loads); the modal accelerations are set to them */
od_status od_modal_set_external_forces(od_modal* modal, const double* f_ext);
/* runOneTimeStep (linearNewmark.cpp:57-79), steps times */
od_status od_modal_step(od_modal* modal, int steps);
/* updateMeshVerticesDisplacements / getMeshVerticesVelocities
 * (linearNewmark.cpp:81-131): sum_i d_i phi_i on the free DOFs, as 3 values
 * per node; constrained entries get the scene's displacement (zero unless
 * set) and zero velocity */
od_status od_modal_get_displacements(od_modal* modal, double* u);
od_status od_modal_get_velocities(od_modal* modal, double* v);
/* eigenvalues (n_modes, ascending) and, if basis != NULL, the modes as
 * n_modes rows of the compacted DOFs */
od_status od_modal_get_modes(od_modal* modal, double* lambda, double* basis);
/* reduced state d, v, a (n_modes each; any may be NULL) */
od_status od_modal_get_state(od_modal* modal, double* d, double* v, double* a);
/* the assembled Hooke stiffness in the reference value layout (num_values) */
od_status od_modal_get_stiffness(od_modal* modal, double* values);
od_status od_modal_get_info(od_modal* modal, od_modal_info* info);

/* Checkpoint / resume: mesh displacement + integrator vectors as a host blob.
 * Call with buf == NULL to query the size. */
od_status od_scene_save(od_scene* scene, void* buf, size_t* size);
od_status od_scene_load(od_scene* scene, const void* buf, size_t size);

#ifdef __cplusplus
}
#endif

#endif /* OD_GB300_H */
