// Internal data model of the GB300 implicit FEM step (not part of the ABI).
//
// HBM layout of one scene (all arrays device-resident, element arrays in
// colour order so every colour is a contiguous range):
//   X, u            n_nodes*3 double   rest positions / mesh displacement
//   tets            n_tets int4        node ids
//   pre             SoA [k][n_tets]    corotational: 90 K0 + 9 Dm^-1 + V;
//                                      invertible:   12 dN + 9 Dm^-1 + V
//   emap            SoA [78][n_tets]   reference element->value map
//   gdof            SoA [12][n_tets]   compacted DOF of each element DOF or -1
//   K, M, D         n_values double    tangent / mass / external damping in the
//                                      reference lower block-CSC value layout
//   full BSR        row_ptr[nb+1], col[nnzb] over padded 3-DOF blocks (both
//                   triangles); desc[nnzb] says where each block's 9 values
//                   live in the lower layout; A[nnzb*9] in FP64 or FP32
//   vectors         n_pad = 3*nb doubles (padding DOFs carry an identity row)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/od_gb300.h"

namespace od {

// Where a full-BSR block takes its values from in the lower layout.
enum BlockKind : int32_t {
  BK_LOWER = 0,      // stored block (br, bc) br > bc, column-major: a[r][c] = v[off + c*3 + r]
  BK_UPPER = 1,      // transpose of a stored block: a[r][c] = v[off + r*3 + c]
  BK_DIAG = 2,       // packed symmetric diagonal block (6 values)
  BK_GENERAL = 3     // irregular: per-entry table at gen[off*9 .. +9] (-1 zero, -2 identity)
};

struct FullBsr {
  int nb = 0;                 // block rows (= ceil(dofs / 3))
  int nnzb = 0;               // stored blocks (both triangles)
  int* row_ptr = nullptr;     // nb + 1
  int* col = nullptr;         // nnzb
  int* desc_off = nullptr;    // nnzb
  int* desc_kind = nullptr;   // nnzb
  int* gen = nullptr;         // 9 per general block
  int n_general = 0;
  int* diag_pos = nullptr;    // nb: index of the diagonal block in each row
};

struct SolveScalars {           // device-resident PCG scalars
  double rz[2];                 // r.z by iteration parity
  double rr, bb, eps, rr0, tr_num, tr_den, alpha, beta;
  int iter, max_iter, done, status;
};

struct SliceSys;
struct MixedSys;
struct SweepSys;
struct Scene;

struct Pcg {
  int n_pad = 0;
  int precision = OD_PRECISION_FP64;
  bool x_zero = false;   // the next solve starts from x = 0 (set by the caller that zeroed x; cleared by the solve)
  double* x = nullptr;
  double* r = nullptr;
  double* z = nullptr;
  double* p = nullptr;
  double* q = nullptr;
  double* b = nullptr;
  double* partial = nullptr;    // 4 arrays of per-CTA partials
  SolveScalars* sc = nullptr;
  SolveScalars* sc_host = nullptr;  // pinned mirror
  unsigned long long* prof = nullptr;       // persistent solve's phase times (profiling), prof_slots
  int prof_slots = 0;                       // kPcgProfSlots + 3 per CTA of the cooperative grid
  unsigned long long* prof_host = nullptr;  // pinned mirror
  int grid = 0;
  // preconditioner
  double* pinv = nullptr;       // Jacobi: n_pad; block-Jacobi: 9*nb
  // IC(0) (scalar CSR of the padded lower pattern)
  int ic_n = 0, ic_nnz = 0;
  int* ic_rp = nullptr;
  int* ic_ci = nullptr;
  int* ic_src = nullptr;        // source entry in the full BSR A (block*9 + r*3 + c)
  double* ic_val = nullptr;
  int n_levels_f = 0;
  int* lvl_rows_f = nullptr;    // rows sorted by forward level
  std::vector<int> lvl_ptr_f;   // host level offsets (per-level factorisation)
  int* ic_bad = nullptr;        // breakdown flag
  // upper (transposed) CSR for the backward sweep: for row i, entries L_ji j > i
  int* icT_rp = nullptr;
  int* icT_ci = nullptr;
  int* icT_pos = nullptr;       // index into ic_val
  double ic_shift = 0.0;
  // the factor split for the one-launch sweeps: strictly lower rows
  // (forward), strictly lower columns (backward: icT_*), diagonal
  int* ic_frp = nullptr;        // ic_n + 1
  int* ic_fci = nullptr;
  double* ic_fval = nullptr;
  double* ic_bval = nullptr;    // L values in icT order
  double* ic_dval = nullptr;    // 1 / L_ii
  double* ic_y = nullptr;       // forward result
  int* ic_err = nullptr;        // a bounded wait ran out
  int* ic_err_host = nullptr;   // pinned
  int ic_grid = 0;
  // one-launch factorisation: per off-diagonal entry (i, j) the pairs
  // (L_ik, L_jk), k < j, as (position in row i, global position in row j)
  int* ic_pp = nullptr;         // ic_nnz + 1
  int* ic_pa = nullptr;
  int* ic_pb = nullptr;
  int ic_fgrid = 0;             // co-resident CTAs; 0: one launch per level
  int ic_fmaxrow = 0, ic_fmaxpairs = 0;
  size_t ic_fsmem = 0;          // dynamic shared memory per CTA
  int* ic_gord_f = nullptr;     // row triples by forward / backward level
  int* ic_gord_b = nullptr;
  int ic_gdepth = 0;            // levels of the two sweeps
  // node order of the factor: block rows by colour (greedy colouring of
  // the block graph), or the natural order
  int ic_colours = 0;           // colours (0: natural order)
  int* ic_pdof = nullptr;       // factor DOF -> the system's DOF (colour order only)
  double* ic_zp = nullptr;      // the backward sweep's values in factor order
  std::vector<int> ic_cstart;   // first factor block of each colour (colour order)
  bool ic_by_colour = false;    // sweeps one launch per colour (colours much larger than the sweep grid)
  // persistent (cooperative) solve
  void* gbar = nullptr;         // grid barrier state
  int* timeout_host = nullptr;  // pinned
  int coop_grid = 0;            // co-resident CTAs, 0 if cooperative launch is unavailable
  int smem_bytes = 0;           // dynamic shared memory of the staged persistent solve (0: not used)
  int recur = -1;               // one-launch PCG form: 1 recurrence (q = A z + beta q; two grid syncs),
                                // 0 the reference's (q = A p; three), -1 chosen by the tolerance
  int disable_persistent = 0;
  // mixed precision: the scene's sliced FP32 operator and its one-scene
  // solve (both built on first use)
  SliceSys* slice = nullptr;
  MixedSys* mix = nullptr;
  struct MixIc0* mic = nullptr;  // mixed precision with IC(0) (FP32 factor copy and inner vectors)
  // incomplete LDL^T / threshold incomplete Cholesky (factor on the host,
  // triangular sweeps on the device)
  SweepSys* sweep = nullptr;
};

// phases of a persistent PCG iteration timed while profiling: SpMV + p.q,
// its grid-wide sum, the update (x, r, z, r.z, r.r), its sum, p = z + beta p,
// the closing barrier; one more slot counts the iterations
constexpr int kPcgPhases = 6;
constexpr int kPcgProfSlots = kPcgPhases + 1;
constexpr int kSliceRows = 10;      // block rows per slice (3 lanes each, 30 of a warp's 32)
constexpr int kSliceWindow = 320;   // rows sorted by length inside windows of this many rows
constexpr int kMaxLocalScenes = 32; // scenes one CTA of the inner FP32 solve may span

// Tiles of a multi-scene kernel: scene s owns the tiles [prefix[s],
// prefix[s+1]) of the launch, tile j of the scene covering its indices
// [j*size, min(n_s, (j+1)*size)); a CTA finds its scene by binary search.
struct TileDir {
  const int* prefix = nullptr;  // device, n_sc+1
  int tiles = 0;                // prefix[n_sc]
  int size = 0;                 // indices per tile
};

// Device view of one scene for the multi-scene step kernels.
struct SceneDev {
  int n_tets, dofs, nb, n_pad, nvals, nnzb, kind;
  double thr, lambda, mu;
  double yield, creep, max_plastic;  // corotational plastic
  double* plastic;                   // [9][n_tets] plastic strain (colour order) or null
  const int4* tets;
  const double* X;
  double* u;
  const double* pre;
  const int* emap;
  const int* gdof;
  const int* color_off;            // colour ranges of the (colour-ordered) elements
  const int *gat_kptr, *gat_ksrc, *gat_fptr, *gat_fsrc;  // gathered assembly lists
  double *K, *fint, *stage_k, *stage_f;
  const double *M, *fext;
  const int *row_ptr, *col, *desc_kind, *desc_off, *gen;
  double* A64;
  const int* free_pos;
  double *d, *v, *a, *dp, *vp, *dv, *rhs, *tmp, *tmp2;
  double bh2, gh, h, c_ad, c_av, alpha_m, beta_k;  // Newmark constants
};

// Per-scene input / output of the inner FP32 PCG of a mixed solve.
struct RingScene {
  double rhs_scale;   // in: 1 / ||r64|| of the scene
  double unscale;     // in: ||r64|| (the correction is unscale * d)
  double itol2;       // in: squared relative inner tolerance
  int max_iter;       // in
  int active0;        // in: the scene takes part in this sweep
  int iters;          // out
  int status;         // out
  double rr;          // out: final inner r.r
};

// A scene's sliced FP32 operator and inner-solve vectors, resident on the
// device from the scene's first mixed-precision use on.  Block rows in
// slices of kSliceRows (rows sorted by block count, longest first, within
// windows of kSliceWindow rows, every slice padded to an even step count);
// the k-th blocks of a slice's rows sit together, values [step][j][lane]
// with lane = 3*row_in_slice + r, column indices are slice rows.  Inner
// vectors are in slice order (element 30*slice + lane).
struct SliceSys {
  int ns = 0;                      // slices
  int lower = 0;                   // lower-triangle storage (symmetric SpMV with transposed products)
  long long steps = 0;
  std::vector<int> off_host;       // ns+1
  double bytes = 0.0;              // algorithmic bytes of one SpMV + p.q phase
  int* perm = nullptr;             // ns*kSliceRows: block row or -1
  int* off = nullptr;              // ns+1 first step of each slice
  int* col = nullptr;              // steps*kSliceRows
  int* src = nullptr;              // steps*kSliceRows: full-BSR block or -1
  float* val = nullptr;            // steps*90
  float* v32 = nullptr;            // u (40/slice), d, r, p, w (30/slice), preconditioner (90/slice), s (30/slice);
                                   // lower storage: w as float4 rows (40/slice) after s
  double* r64 = nullptr;           // FP64 residual (n_pad)
  long long device_bytes = 0;
};

// Device view of one scene of a mixed solve: the FP64 full BSR, the
// right-hand side and solution it refines, and its sliced FP32 system.
struct MixDesc {
  const int* row_ptr;
  const int* col;
  const int* diag_pos;
  const double* A64;
  const double* b;
  double* x;
  int nb;
  int ns;                          // slices
  int steps;                       // steps of the sliced matrix
  int slice0;                      // first slice of the scene in the system's slice order
  const int* sperm;
  const int* soff;
  const int* scol;
  const int* ssrc;
  float* sval;
  float* v32;
  double* r64;
  int lower;                       // lower-triangle sliced matrix (symmetric SpMV)
};

// A mixed-precision solve over one or more scenes (block diagonal): the
// scenes' slices in a virtual concatenation cut into contiguous CTA ranges;
// every scene keeps its own arrays (SliceSys), so building a system is
// O(scenes).
struct MixedSys {
  int n_sc = 0;                    // scenes
  std::vector<Scene*> scenes;      // for the FP64 fallback of a solve that does not converge
  int ns = 0;                      // slices of all scenes
  std::vector<int> off_host;       // ns+1 step offsets of the concatenation (partition)
  std::vector<int> sc_slice;       // n_sc+1 first slice of each scene
  std::vector<int> sc_nb;          // n_sc block rows
  std::vector<double> sc_bytes;    // n_sc algorithmic bytes of one SpMV + p.q phase
  unsigned long long* prof = nullptr;       // phase time incl. its sum, iterations, SpMV work time (ns), per-CTA stamps
  unsigned long long* prof_host = nullptr;  // pinned
  int* sc_slice_dev = nullptr;     // n_sc+1
  MixDesc* desc = nullptr;         // n_sc (device)
  std::vector<MixDesc> desc_host;
  RingScene* ring = nullptr;       // n_sc (device)
  RingScene* ring_host = nullptr;  // n_sc (pinned)
  double* rrbb = nullptr;          // 2*n_sc: residual r.r, b.b (device)
  double* rrbb_host = nullptr;     // pinned
  int* dirs = nullptr;             // tile prefixes (device): residual, fill, precond, update
  TileDir res_dir, fill_dir, pre_dir, upd_dir;
  double* res_part = nullptr;      // 2 per residual tile
  // CTA partition of the ring kernel
  int cta_grid = 0;
  int* cta_first = nullptr;        // G+1 first slice of each CTA
  int* cta_sc_lo = nullptr;        // G first scene of each CTA
  int* sc_cta = nullptr;           // 2*n_sc: first, last CTA of each scene
  double* part = nullptr;          // [3][n_sc][G] per-scene CTA partials + 2 G
  void* gbar = nullptr;
  int* timeout_host = nullptr;     // pinned
  // measured balance (single-scene systems): every CTA adds the time of its
  // SpMV phases; after a solve the slice weights of each CTA are scaled by
  // its measured time per weight and the slices re-partitioned
  std::vector<double> slice_w;     // cost weight of every slice (steps + a per-slice cost at first)
  std::vector<int> first_host;     // G+1 first slice of each CTA (host copy of cta_first)
  unsigned long long* cta_ns = nullptr;       // G (device)
  unsigned long long* cta_ns_host = nullptr;  // G (pinned)
  int rebalances = 0;
  // tile shapes (the batch autotuner's choice, else the defaults)
  int piece_steps = 20;            // ring-kernel steps per bulk copy (12, 16 or 20; lower storage: 12)
  int ring_warps = 12;             // consumer warps per CTA (12, or 15 with 12- or 16-step pieces; lower: 15)
  double slice_cost = 8.0;         // a slice's fixed cost in steps, for the CTA partition
};
bool ring_shape_supported(int ps, int nw);
od_status mixed_retune(MixedSys* m, int piece_steps, int ring_warps, double slice_cost);

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  // counters
  long long launches = 0;
  long long host_syncs = 0;
  long long spmv_launches = 0;
  double spmv_ms = 0.0;
  long long pcg_kernel_launches = 0;  // persistent solves timed while profiling
  long long pcg_kernel_iters = 0;
  double pcg_kernel_ms = 0.0;
  long long mix_iters = 0;            // inner FP32 loop iterations (profiling)
  long long mix_fallbacks = 0;        // mixed solves finished by the FP64 solver
  double mix_fallback_ms = 0.0;       // their host wall time
  long long sweep_factors = 0, sweep_nnz = 0, sweep_applies = 0, sweep_levels = 0;
  double sweep_factor_ms = 0.0, sweep_apply_ms = 0.0, sweep_apply_bytes = 0.0;
  double mix_spmv_ms = 0.0;
  double mix_spmv_work_ms = 0.0;
  double mix_spmv_bytes = 0.0;
  double pcg_phase_ms[kPcgPhases] = {};  // persistent PCG phases (CTA 0, profiling)
  double pcg_work_max_ms[3] = {};       // per solve: slowest CTA's own SpMV / update / direction work
  double pcg_work_mean_ms[3] = {};      // per solve: mean over the CTAs
  long long pcg_phase_iters = 0;
  int profiling = 0;
  std::vector<cudaEvent_t> ev_pool;   // event pairs for SpMV timing
};

#define OD_KL(scene) ((scene)->ctx->launches++)

struct Scene {
  Ctx* ctx = nullptr;
  int n_nodes = 0, n_tets = 0, n_facets = 0, dofs = 0;
  od_material mat{};
  double lambda = 0, mu = 0, D[3] = {0, 0, 0};
  // host copies
  std::vector<double> hX;
  std::vector<int> htets, hfacets, hcd, hfree_pos, hnode_dof;
  std::vector<int> hpcol, hrows, horis, hemap;
  std::vector<int> hbsr_rp, hbsr_col;   // full BSR row pointers / block columns
  int nbc = 0, nrem = 0, nvals = 0;
  std::vector<int> color_off;      // element colour ranges (colour order)
  int* color_off_dev = nullptr;    // the same on the device
  double mix_iters_last = 0.0;     // inner iterations of the scene's last mixed solve
  // gathered assembly (CSR over the destinations, sources in the reference's
  // element order; null when 78 x elements overflows a 32-bit index)
  int* gat_kptr = nullptr;  // nvals + 1
  int* gat_ksrc = nullptr;  // k * n_tets + staged element position
  int* gat_fptr = nullptr;  // n_pad + 1
  int* gat_fsrc = nullptr;  // (k - 78) * n_tets + staged element position
  std::vector<int> elem_perm;      // colour-order position -> original element
  // device
  double* X = nullptr;
  double* u = nullptr;
  int4* tets = nullptr;
  double* pre = nullptr;
  int n_pre = 0;
  double* plastic = nullptr;       // corotational plastic: [9][n_tets] plastic strain (colour order)
  int* emap = nullptr;
  int* gdof = nullptr;
  int* perm = nullptr;
  int* free_pos = nullptr;         // compacted DOF -> 3*node + axis
  int* node_dof = nullptr;         // 3*node + axis -> compacted DOF or -1
  int* facets_dev = nullptr;       // n_facets * 3
  double* node_vol4 = nullptr;     // sum over incident tets of V/4
  double* K = nullptr;
  double* M = nullptr;
  double* Dm = nullptr;            // external damping (zero unless set)
  bool has_damping = false;        // Dm holds non-zero values
  double* fint = nullptr;
  double* fext = nullptr;
  double* work_vals = nullptr;     // host-supplied values (SpMDV / PCG drop-in)
  double* stage_k = nullptr;       // [n_tets][78] element stiffness, node blocks contiguous (c_kslot; colour order)
  double* stage_f = nullptr;       // [n_tets][12] element forces
  FullBsr bsr;
  void* A = nullptr;               // full BSR values (double or float)
  double* A64 = nullptr;           // FP64 full values
  // sources of the last A64 expansion (A = c1 V1 + c2 V2 + c3 V3, lower
  // layout), from which the LDL^T factor rebuilds A in the reference layout
  struct {
    const double *v1 = nullptr, *v2 = nullptr, *v3 = nullptr;
    double c1 = 0.0, c2 = 0.0, c3 = 0.0;
  } lo;
  Pcg pcg;
  // integrator
  od_integrator_params ip{};
  bool has_integrator = false;
  double *v = nullptr, *d = nullptr, *a = nullptr, *dp = nullptr, *vp = nullptr, *dv = nullptr,
         *rhs = nullptr, *tmp = nullptr, *tmp2 = nullptr;
  double time = 0.0;
  long long device_bytes = 0;
  // traction loads (per call)
  int* trac_facets = nullptr;      // facet ids of the (facet, traction) pairs, in load order
  double* trac_vec = nullptr;      // per pair traction (3)
  int trac_cap = 0;
  int* load_ptr = nullptr;         // per padded DOF: its traction entries (n_pad + 1)
  int* load_src = nullptr;         // the (facet, traction) pair of each entry, in load order
  int load_cap = 0;
  int n_trac = 0;                  // facet entries of the last od_scene_set_loads
  double load_body[3] = {0, 0, 0};
  bool has_body = false;
  cudaEvent_t ev_step[2] = {nullptr, nullptr};
  double sched_freq = 0.0, sched_phase = 0.0;   // traction schedule
};

// ---- error handling ----
void set_error(const std::string& msg);
od_status cuda_fail(cudaError_t e, const char* what);
#define OD_TRY(expr)              \
  do {                            \
    od_status _st = (expr);       \
    if (_st != OD_OK) return _st; \
  } while (0)
#define OD_CUDA(call)                                        \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return ::od::cuda_fail(_e, #call); \
  } while (0)

// temporary device buffers freed on every return path
struct DeviceTemps {
  std::vector<void*> ptrs;
  template <class T>
  cudaError_t alloc(T** p, size_t bytes) {
    *p = nullptr;
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e == cudaSuccess) ptrs.push_back((void*)*p);
    return e;
  }
  ~DeviceTemps() {
    for (void* p : ptrs) cudaFree(p);
  }
};

// argument check of an ABI entry point
#define OD_CHECK_ARG(cond, msg)              \
  do {                                       \
    if (!(cond)) {                           \
      ::od::set_error(msg);                  \
      return OD_ERR_INVALID_ARG;             \
    }                                        \
  } while (0)

// ---- host algorithms (od_host.cpp) ----
int global_index(const std::vector<int>& cd, int node, int axis);
void build_pattern(const std::vector<int>& gidx, int n_tets, int dofs, std::vector<int>& pcol,
                   std::vector<int>& rows, std::vector<int>& oris, int& nbc, int& nrem, int& nvals);
void build_emap(const std::vector<int>& gidx, int n_tets, int dofs, int nbc,
                const std::vector<int>& pcol, const std::vector<int>& rows,
                const std::vector<int>& oris, std::vector<int>& emap);
int color_elements(const std::vector<int>& nodes, int per_elem, int n_elem, int n_nodes,
                   std::vector<int>& perm, std::vector<int>& color_off);
struct HostBsr {
  int nb = 0;
  std::vector<int> row_ptr, col, desc_off, desc_kind, gen, diag_pos;
};
void build_full_bsr(int dofs, int nbc, int nrem, const std::vector<int>& pcol,
                    const std::vector<int>& rows, const std::vector<int>& oris, HostBsr& out);
struct HostSliced {
  int ns = 0;
  bool lower = false;
  std::vector<int> perm, off, col, src;
};
void build_sliced(const std::vector<int>& row_ptr, const std::vector<int>& col, int nb, HostSliced& out,
                  bool lower);
void build_ic_levels(const std::vector<int>& rp, const std::vector<int>& ci, int n,
                     std::vector<int>& rows_by_level, std::vector<int>& lvl_ptr, bool forward);
// incomplete LDL^T (od_rif.cpp): scalar columns of the symmetric matrix in
// getFullIndices order, and the factor in the reference's storage (L
// columns 0..n-2 with rows in production order, pcol with n entries, the
// inverted diagonal)
struct RifColumns {
  int n = 0;
  std::vector<int> ptr, row, src;
};
struct RifFactor {
  int n = 0;
  std::vector<double> val;
  std::vector<int> row, pcol;
  std::vector<double> dinv;
};
void rif_columns(int n, int nbc, const std::vector<int>& pcol, const std::vector<int>& rows, RifColumns& out);
void rif_factor(const RifColumns& A, const double* values, double sainv_eps, double ldlt_eps, RifFactor& F);
// threshold incomplete Cholesky (od_ric.cpp): value positions of every
// stored lower column in getColumn order, and the factor in the reference's
// storage (column c = its diagonal then its rows below ascending; pcol n + 1)
struct RicColumns {
  int n = 0;
  std::vector<int> ptr, row, src;
};
struct RicFactor {
  int n = 0;
  std::vector<double> val;
  std::vector<int> row, pcol;
};
void ric_columns(int n, int nbc, const std::vector<int>& pcol, const std::vector<int>& rows,
                 const std::vector<int>& oris, RicColumns& out);
void ric_factor(const RicColumns& A, const double* values, double eps, double relax, RicFactor& F);

// ---- kernels (od_elements.cu) ----
od_status launch_precompute(Scene* s);
od_status launch_mass(Scene* s);
// K, fint at current u; df: the mixed-precision path's double-float stiffness
// contraction (invertible materials; the others are unchanged)
od_status launch_eval(Scene* s, bool zero_first, bool df = false);
od_status launch_hooke(Scene* s, double youngs, double poisson, double* Kh);  // linear K, reference layout
// new body force / uniform traction on the facets of the last od_scene_set_loads
od_status scene_set_uniform_loads(Scene* s, const double* body, const double* traction);
od_status launch_element_values(Scene* s, double* d_k78, double* d_f12);
od_status launch_loads(Scene* s, const double* body, int n_facets_total, double traction_scale);
// multi-scene element evaluation: zero K (values) and f_int (padded DOFs),
// compute every element into the scenes' staging arrays (one launch per
// material family), then scatter colour by colour (tiles over 90 threads
// per element of the colour)
od_status build_gather_lists(Scene* s, int n_pad);
od_status selftest_barrier_timeout(Ctx* c, int* timed_out);
od_status selftest_value_wait_timeout(Ctx* c, int* timed_out);
od_status launch_eval_batch(Ctx* ctx, int n_sc, const SceneDev* sd, const TileDir& zero_k, const TileDir& zero_f,
                            const TileDir& corot, const TileDir& inv, const TileDir& plastic,
                            const std::vector<TileDir>& scatter,
                            const TileDir& gather);
od_status sync_stream(Scene* s);

// ---- kernels (od_sparse.cu) ----
od_status pcg_alloc(Scene* s);
void pcg_free(Scene* s);
// A64 = c1 V1 + c2 V2 + c3 V3 expanded to the full BSR (V2, V3 may be NULL)
od_status launch_expand(Scene* s, const double* v1, double c1, const double* v2, double c2, const double* v3,
                        double c3);
// y (+)= c1 V1 x1 + c2 V2 x2 + c3 V3 x3, V* in the lower layout (V2, V3 may be NULL)
od_status launch_spmv_lower(Scene* s, const double* v1, double c1, const double* x1, const double* v2, double c2,
                            const double* x2, const double* v3, double c3, const double* x3, double* y,
                            bool accumulate);
od_status launch_spmv_full(Scene* s, const double* x, double* y);
// multi-scene: Newmark system A64 of every scene (value tiles) and
// rhs = M tmp + beta_K K tmp2 (block-row tiles of kBatchRows rows)
constexpr int kBatchRows = 80;
constexpr int kExpandTile = 2048;   // full-BSR values per tile of the multi-scene system combination
constexpr int kZeroTileValues = 4096;  // values per tile of the multi-scene zeroing
od_status launch_expand_batch(Ctx* ctx, int n_sc, const SceneDev* sd, const TileDir& dir);
od_status launch_spmv_lower_batch(Ctx* ctx, int n_sc, const SceneDev* sd, const TileDir& dir);

#ifdef __CUDACC__
// scene of tile t of a directory over n scenes (largest s with prefix[s] <= t)
__device__ __forceinline__ int dir_scene(const int* __restrict__ prefix, int n, int t) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}
#endif
// ---- preconditioners applied by triangular sweeps (od_sweep.cu)
constexpr double kLdltSainvDefault = 0.1;
constexpr double kLdltDropDefault = 0.01;
constexpr double kIcEpsDefault = 1e-3;
// factor of A given in the reference's lower layout on the host, or (NULL)
// of the last A64 expansion
od_status ldlt_factor(Scene* s, const double* host_values, double sainv_eps, double ldlt_eps);
od_status ic_factor(Scene* s, const double* host_values, double eps, double relax);
// z = (L D L^T)^-1 r or (L L^T)^-1 r with the loaded factor, on the device
// (length n_pad; padding rows copied); returns at once when sc->done is set
od_status sweep_apply(Scene* s, const double* r, double* z, const SolveScalars* sc);
// OD_ERR_DEVICE_TIMEOUT if a sweep's bounded wait ran out since the last check
od_status sweep_check(Scene* s);
void sweep_free(SweepSys* l);
// A factor laid out for one cooperative two-sweep apply (od_sweep.cu):
// strictly lower rows (frp/fci/fval), strictly lower columns (bcp/bri/bval),
// the diagonal, row triples [3g, 3g + 3) listed by forward / backward
// dependency level (sweep_group_levels).
struct SweepView {
  int n = 0, n_pad = 0;
  int ic = 1;                   // 1: diag holds 1 / L_ii; 0: D^-1 (LDL^T)
  int grid = 0;                 // co-resident CTAs
  long long nnz = 0;            // strictly lower entries
  const int *frp = nullptr, *fci = nullptr, *bcp = nullptr, *bri = nullptr, *ord_f = nullptr, *ord_b = nullptr;
  const double *fval = nullptr, *bval = nullptr, *diag = nullptr;
  double* y = nullptr;
  int* err = nullptr;
  // factor in a permuted DOF order (IC(0) by colours): perm[new DOF] = the
  // caller's DOF; the sweeps keep z in the permuted order in zperm (the
  // ready flags) and also write every value to the caller's z at perm[]
  const int* perm = nullptr;
  double* zperm = nullptr;
  // colour order with colours far larger than the one-launch sweep's warps:
  // first triple of each colour (the sweeps then go one launch per colour)
  const std::vector<int>* colour_start = nullptr;
};
od_status sweep_grid(Scene* s, int n, int* grid);
void sweep_group_levels(int n, const std::vector<int>& frp, const std::vector<int>& fci, const std::vector<int>& bcp,
                        const std::vector<int>& bri, std::vector<int>& ord_f, std::vector<int>& ord_b, int* depth_f,
                        int* depth_b);
od_status sweep_launch(Scene* s, const SweepView& v, const double* r, double* z, const SolveScalars* sc);
od_status sweep_launch_f32(Scene* s, const SweepView& v, const float* fval, const float* bval, const float* diag,
                           const float* r, float* y, float* z, float* zperm, const SolveScalars* sc);
// IC(0): the shifted FP64 factor of the scene's A64 (od_sparse.cu) and the
// check of its sweeps' bounded waits
od_status ic0_factor(Scene* s);
od_status ic0_check(Scene* s);
// mixed-precision solve with the IC(0) preconditioner (od_mixed_ic0.cu)
struct MixIc0;
void mixed_ic0_free(MixIc0* m);
od_status mixed_ic0_solve(Scene* s, const double* d_b, double* d_x, const od_solver_params* prm,
                          od_solve_stats* st);

// PCG on A64; b and x are device vectors of length n_pad
od_status pcg_solve(Scene* s, const double* d_b, double* d_x, const od_solver_params* prm, od_solve_stats* st);

// ---- mixed-precision systems (od_sparse.cu)
// the scene's sliced FP32 operator (built once, kept with the scene)
od_status slice_build(Scene* s);
void slice_free(SliceSys* sl);
// a solve over scenes (their slices built on demand) with the given
// right-hand sides / solutions (nullptr: supplied per solve)
od_status mixed_build(Ctx* ctx, const std::vector<Scene*>& scenes, const std::vector<const double*>& b,
                      const std::vector<double*>& x, MixedSys** out);
void mixed_free(MixedSys* m);
// solves every scene's A64 x = b with FP64 refinement around the FP32 inner
// PCG (same preconditioner kind for all); per-scene parameters and results.
// x_zero: every scene's x is 0 on entry (the first residual is b itself)
od_status mixed_solve(Ctx* ctx, MixedSys* m, int precond, const std::vector<od_solver_params>& prm,
                      std::vector<od_solve_stats>& st, bool x_zero = false);

}  // namespace od

// ABI handles (opaque in include/od_gb300.h)
struct od_ctx {
  od::Ctx c;
};
struct od_scene {
  od::Scene s;
};
