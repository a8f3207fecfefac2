// C ABI (include/od_gb300.h): contexts, scenes, the material / solver /
// integrator entry points and the step drivers.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "od_internal.h"

namespace od {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

od_status cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ") in " + what;
  if (e == cudaErrorMemoryAllocation) return OD_ERR_OUT_OF_MEMORY;
  return OD_ERR_CUDA;
}

static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

od_status sync_stream(Scene* s) {
  s->ctx->host_syncs++;
  OD_CUDA(cudaStreamSynchronize(s->ctx->stream));
  return OD_OK;
}

// ------------------------------------------------------ integrator kernels
// u[free_pos[i]] = v[i] (mode 0) or += h v[i] (mode 1)
__global__ void write_mesh_kernel(int n, const int* __restrict__ free_pos, const double* __restrict__ v, double h,
                                  int mode, double* __restrict__ u) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mode == 0) u[free_pos[i]] = v[i];
  else u[free_pos[i]] += v[i] * h;
}

// backward-Euler rhs = h (f_ext - f_int - A0 v)  (nonlinearImplicitBackwardEuler.h:90-92)
__global__ void be_rhs_kernel(int n, double h, const double* __restrict__ fext, const double* __restrict__ fint,
                              const double* __restrict__ a0v, double* __restrict__ rhs) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rhs[i] = h * (fext[i] - fint[i] - a0v[i]);
}

// y += x
__global__ void add_kernel(int n, const double* __restrict__ x, double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}

// Newmark predictor: dp = d + h v + (1/2 - beta) h^2 a; vp = v + (1 - gamma) h a
__global__ void nm_predict_kernel(int n, double h, double c_a_d, double c_a_v, const double* __restrict__ d,
                                  const double* __restrict__ v, const double* __restrict__ a, double* __restrict__ dp,
                                  double* __restrict__ vp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dp[i] = d[i] + h * v[i] + c_a_d * a[i];
  vp[i] = v[i] + c_a_v * a[i];
}

// d_k = dp + beta h^2 a written to the mesh; t1 = alpha_M v_k + a, t2 = v_k
__global__ void nm_stage_kernel(int n, const int* __restrict__ free_pos, double bh2, double gh, double alpha_m,
                                const double* __restrict__ dp, const double* __restrict__ vp,
                                const double* __restrict__ a, double* __restrict__ u, double* __restrict__ t1,
                                double* __restrict__ t2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ai = a[i];
  u[free_pos[i]] = dp[i] + bh2 * ai;
  const double vk = vp[i] + gh * ai;
  t1[i] = alpha_m * vk + ai;
  t2[i] = vk;
}

// r = f_ext - f_int - y
__global__ void nm_residual_kernel(int n, const double* __restrict__ fext, const double* __restrict__ fint,
                                   const double* __restrict__ y, double* __restrict__ r) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = fext[i] - fint[i] - y[i];
}

// corrector d = dp + beta h^2 a, v = vp + gamma h a, mesh u = d
__global__ void nm_correct_kernel(int n, const int* __restrict__ free_pos, double bh2, double gh,
                                  const double* __restrict__ dp, const double* __restrict__ vp,
                                  const double* __restrict__ a, double* __restrict__ d, double* __restrict__ v,
                                  double* __restrict__ u) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  d[i] = dp[i] + bh2 * a[i];
  v[i] = vp[i] + gh * a[i];
  u[free_pos[i]] = d[i];
}

}  // namespace od

using namespace od;




template <class T>
static od_status dalloc(Scene* s, T** p, size_t n) {
  n = std::max<size_t>(n, 1);
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  s->device_bytes += (long long)(sizeof(T) * n);
  return OD_OK;
}

template <class T>
static od_status dupload(Scene* s, T** p, const T* h, size_t n) {
  OD_TRY(dalloc(s, p, n));
  if (n) OD_CUDA(cudaMemcpy(*p, h, sizeof(T) * n, cudaMemcpyHostToDevice));
  return OD_OK;
}

extern "C" {

const char* od_status_string(od_status s) {
  switch (s) {
    case OD_OK: return "OD_OK";
    case OD_ERR_INVALID_ARG: return "OD_ERR_INVALID_ARG";
    case OD_ERR_OUT_OF_MEMORY: return "OD_ERR_OUT_OF_MEMORY";
    case OD_ERR_NOT_CONVERGED: return "OD_ERR_NOT_CONVERGED";
    case OD_ERR_NAN: return "OD_ERR_NAN";
    case OD_ERR_DEVICE_TIMEOUT: return "OD_ERR_DEVICE_TIMEOUT";
    case OD_ERR_CUDA: return "OD_ERR_CUDA";
    case OD_ERR_UNSUPPORTED: return "OD_ERR_UNSUPPORTED";
    default: return "OD_ERR_INTERNAL";
  }
}

const char* od_last_error(void) { return g_last_error.c_str(); }
int od_abi_version(void) { return OD_ABI_VERSION; }

od_status od_ctx_create(int device, od_ctx** out) {
  OD_CHECK_ARG(out, "od_ctx_create: out is NULL");
  int count = 0;
  OD_CUDA(cudaGetDeviceCount(&count));
  OD_CHECK_ARG(device >= 0 && device < count, "od_ctx_create: no such CUDA device");
  OD_CUDA(cudaSetDevice(device));
  od_ctx* c = new (std::nothrow) od_ctx();
  if (!c) return OD_ERR_OUT_OF_MEMORY;
  c->c.device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreateWithFlags"); }
  cudaDeviceGetAttribute(&c->c.num_sms, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return OD_OK;
}

od_status od_ctx_destroy(od_ctx* ctx) {
  if (!ctx) return OD_OK;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  cudaStreamDestroy(ctx->c.stream);
  for (auto& e : ctx->c.ev_pool) cudaEventDestroy(e);
  delete ctx;
  return OD_OK;
}

od_status od_selftest_bounded_waits(od_ctx* ctx, int* barrier_timed_out, int* value_wait_timed_out) {
  OD_CHECK_ARG(ctx && barrier_timed_out && value_wait_timed_out, "od_selftest_bounded_waits: NULL argument");
  OD_CUDA(cudaSetDevice(ctx->c.device));
  OD_TRY(selftest_barrier_timeout(&ctx->c, barrier_timed_out));
  OD_TRY(selftest_value_wait_timeout(&ctx->c, value_wait_timed_out));
  return OD_OK;
}

od_status od_ctx_set_profiling(od_ctx* ctx, int enable) {
  OD_CHECK_ARG(ctx, "od_ctx_set_profiling: ctx is NULL");
  OD_CUDA(cudaSetDevice(ctx->c.device));
  if (enable && ctx->c.ev_pool.empty()) {
    ctx->c.ev_pool.resize(2 * 64);
    for (auto& e : ctx->c.ev_pool) OD_CUDA(cudaEventCreate(&e));
  }
  ctx->c.profiling = enable <= 0 ? 0 : (enable >= 2 ? 2 : 1);
  return OD_OK;
}

od_status od_ctx_get_counters(od_ctx* ctx, od_counters* out) {
  OD_CHECK_ARG(ctx && out, "od_ctx_get_counters: NULL argument");
  out->kernel_launches = ctx->c.launches;
  out->host_syncs = ctx->c.host_syncs;
  out->spmv_launches = ctx->c.spmv_launches;
  out->spmv_ms = ctx->c.spmv_ms;
  out->pcg_launches = ctx->c.pcg_kernel_launches;
  out->pcg_iterations = ctx->c.pcg_kernel_iters;
  out->pcg_ms = ctx->c.pcg_kernel_ms;
  out->mix_iterations = ctx->c.mix_iters;
  out->mix_spmv_ms = ctx->c.mix_spmv_ms;
  out->mix_spmv_work_ms = ctx->c.mix_spmv_work_ms;
  for (int k = 0; k < od::kPcgPhases; k++) out->pcg_phase_ms[k] = ctx->c.pcg_phase_ms[k];
  out->pcg_phase_iterations = ctx->c.pcg_phase_iters;
  out->mix_fallback_ms = ctx->c.mix_fallback_ms;
  for (int k = 0; k < 3; k++) {
    out->pcg_work_max_ms[k] = ctx->c.pcg_work_max_ms[k];
    out->pcg_work_mean_ms[k] = ctx->c.pcg_work_mean_ms[k];
  }
  out->mix_fallbacks = ctx->c.mix_fallbacks;
  out->mix_spmv_bytes = ctx->c.mix_spmv_bytes;
  out->sweep_factors = ctx->c.sweep_factors;
  out->sweep_factor_ms = ctx->c.sweep_factor_ms;
  out->sweep_nnz = ctx->c.sweep_nnz;
  out->sweep_applies = ctx->c.sweep_applies;
  out->sweep_apply_ms = ctx->c.sweep_apply_ms;
  out->sweep_apply_bytes = ctx->c.sweep_apply_bytes;
  out->sweep_levels = ctx->c.sweep_levels;
  return OD_OK;
}

od_status od_ctx_reset_counters(od_ctx* ctx) {
  OD_CHECK_ARG(ctx, "od_ctx_reset_counters: ctx is NULL");
  ctx->c.launches = ctx->c.host_syncs = ctx->c.spmv_launches = 0;
  ctx->c.pcg_kernel_launches = ctx->c.pcg_kernel_iters = 0;
  ctx->c.spmv_ms = ctx->c.pcg_kernel_ms = 0.0;
  ctx->c.mix_iters = ctx->c.mix_fallbacks = 0;
  ctx->c.mix_fallback_ms = 0.0;
  ctx->c.mix_spmv_ms = ctx->c.mix_spmv_bytes = ctx->c.mix_spmv_work_ms = 0.0;
  for (double& v : ctx->c.pcg_phase_ms) v = 0.0;
  ctx->c.pcg_phase_iters = 0;
  for (int k = 0; k < 3; k++) ctx->c.pcg_work_max_ms[k] = ctx->c.pcg_work_mean_ms[k] = 0.0;
  ctx->c.sweep_factors = ctx->c.sweep_nnz = ctx->c.sweep_applies = ctx->c.sweep_levels = 0;
  ctx->c.sweep_factor_ms = ctx->c.sweep_apply_ms = ctx->c.sweep_apply_bytes = 0.0;
  return OD_OK;
}

od_status od_ctx_synchronize(od_ctx* ctx) {
  OD_CHECK_ARG(ctx, "od_ctx_synchronize: ctx is NULL");
  OD_CUDA(cudaSetDevice(ctx->c.device));
  OD_CUDA(cudaStreamSynchronize(ctx->c.stream));
  return OD_OK;
}

static void scene_free(Scene* s) {
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  for (void* p : {(void*)s->X, (void*)s->u, (void*)s->tets, (void*)s->pre, (void*)s->emap, (void*)s->gdof,
                  (void*)s->perm, (void*)s->free_pos, (void*)s->node_dof, (void*)s->facets_dev, (void*)s->node_vol4,
                  (void*)s->K, (void*)s->M, (void*)s->Dm, (void*)s->fint, (void*)s->fext, (void*)s->work_vals,
                  (void*)s->A64, (void*)s->v, (void*)s->d, (void*)s->a, (void*)s->dp, (void*)s->vp,
                  (void*)s->dv, (void*)s->rhs, (void*)s->tmp, (void*)s->trac_facets, (void*)s->trac_vec,
                  (void*)s->load_ptr, (void*)s->load_src,
                  (void*)s->bsr.row_ptr, (void*)s->bsr.col, (void*)s->bsr.desc_off, (void*)s->bsr.desc_kind,
                  (void*)s->bsr.gen, (void*)s->bsr.diag_pos, (void*)s->tmp2, (void*)s->stage_k,
                  (void*)s->stage_f, (void*)s->color_off_dev, (void*)s->plastic, (void*)s->gat_kptr,
                  (void*)s->gat_ksrc, (void*)s->gat_fptr, (void*)s->gat_fsrc})
    if (p) cudaFree(p);
  pcg_free(s);
  if (s->ev_step[0]) { cudaEventDestroy(s->ev_step[0]); cudaEventDestroy(s->ev_step[1]); }
}

static od_status scene_build(Scene* s, int n_nodes, const double* X, int n_tets, const int* tets, int n_facets,
                             const int* facets, int n_cdofs, const int* cdofs) {
  s->n_nodes = n_nodes;
  s->n_tets = n_tets;
  s->n_facets = n_facets;
  s->hX.assign(X, X + 3 * (size_t)n_nodes);
  s->htets.assign(tets, tets + 4 * (size_t)n_tets);
  s->hfacets.assign(facets, facets + 3 * (size_t)n_facets);
  s->hcd.assign(cdofs, cdofs + n_cdofs);
  // DOF compaction (NodeIndexer, core/nodeIndexer.cpp:12-25, 72-74)
  const int nd3 = 3 * n_nodes;
  s->hnode_dof.assign(nd3, -1);
  s->hfree_pos.clear();
  {
    size_t c = 0;
    int k = 0;
    for (int g = 0; g < nd3; g++) {
      if (c < s->hcd.size() && s->hcd[c] == g) { c++; continue; }
      s->hnode_dof[g] = k++;
      s->hfree_pos.push_back(g);
    }
    s->dofs = k;
  }
  std::vector<int> gidx(12 * (size_t)n_tets);
  for (int e = 0; e < n_tets; e++)
    for (int a = 0; a < 4; a++)
      for (int ax = 0; ax < 3; ax++) gidx[12 * (size_t)e + 3 * a + ax] = s->hnode_dof[3 * tets[4 * (size_t)e + a] + ax];
  build_pattern(gidx, n_tets, s->dofs, s->hpcol, s->hrows, s->horis, s->nbc, s->nrem, s->nvals);
  build_emap(gidx, n_tets, s->dofs, s->nbc, s->hpcol, s->hrows, s->horis, s->hemap);
  color_elements(s->htets, 4, n_tets, n_nodes, s->elem_perm, s->color_off);
  HostBsr hb;
  build_full_bsr(s->dofs, s->nbc, s->nrem, s->hpcol, s->hrows, s->horis, hb);

  // element arrays in colour order, structure of arrays
  const int ne = n_tets;
  std::vector<int4> t4(ne);
  std::vector<int> em((size_t)78 * ne), gd((size_t)12 * ne);
  for (int e = 0; e < ne; e++) {
    const int o = s->elem_perm[e];
    t4[e] = make_int4(tets[4 * (size_t)o], tets[4 * (size_t)o + 1], tets[4 * (size_t)o + 2], tets[4 * (size_t)o + 3]);
    for (int k = 0; k < 78; k++) em[(size_t)k * ne + e] = s->hemap[78 * (size_t)o + k];
    for (int k = 0; k < 12; k++) gd[(size_t)k * ne + e] = gidx[12 * (size_t)o + k];
  }
  OD_TRY(dupload(s, &s->X, s->hX.data(), s->hX.size()));
  OD_TRY(dalloc(s, &s->u, (size_t)nd3));
  OD_CUDA(cudaMemset(s->u, 0, sizeof(double) * std::max(1, nd3)));
  OD_TRY(dupload(s, &s->tets, t4.data(), t4.size()));
  OD_TRY(dupload(s, &s->emap, em.data(), em.size()));
  OD_TRY(dupload(s, &s->gdof, gd.data(), gd.size()));
  OD_TRY(dupload(s, &s->perm, s->elem_perm.data(), s->elem_perm.size()));
  OD_TRY(dupload(s, &s->free_pos, s->hfree_pos.data(), s->hfree_pos.size()));
  OD_TRY(dupload(s, &s->node_dof, s->hnode_dof.data(), s->hnode_dof.size()));
  OD_TRY(dupload(s, &s->facets_dev, s->hfacets.data(), s->hfacets.size()));
  OD_TRY(dalloc(s, &s->node_vol4, (size_t)n_nodes));
  s->n_pre = s->mat.kind == OD_MATERIAL_COROTATIONAL ? 100 : (s->mat.kind == OD_MATERIAL_COROTATIONAL_PLASTIC ? 112 : 22);
  OD_TRY(dalloc(s, &s->pre, (size_t)s->n_pre * ne));
  if (s->mat.kind == OD_MATERIAL_COROTATIONAL_PLASTIC) {  // zero plastic strain (corotationalPlastic.cpp:46-47)
    OD_TRY(dalloc(s, &s->plastic, 9 * (size_t)ne));
    OD_CUDA(cudaMemset(s->plastic, 0, sizeof(double) * 9 * std::max<size_t>(1, ne)));
  }
  // matrices (reference layout) and full BSR
  OD_TRY(dalloc(s, &s->K, (size_t)s->nvals));
  OD_TRY(dalloc(s, &s->M, (size_t)s->nvals));
  OD_TRY(dalloc(s, &s->Dm, (size_t)s->nvals));
  OD_TRY(dalloc(s, &s->work_vals, (size_t)s->nvals));
  OD_TRY(dalloc(s, &s->stage_k, 78 * (size_t)ne));
  OD_TRY(dalloc(s, &s->stage_f, 12 * (size_t)ne));
  OD_CUDA(cudaMemset(s->K, 0, sizeof(double) * std::max(1, s->nvals)));
  OD_CUDA(cudaMemset(s->Dm, 0, sizeof(double) * std::max(1, s->nvals)));
  s->bsr.nb = hb.nb;
  s->bsr.nnzb = (int)hb.col.size();
  s->bsr.n_general = (int)hb.gen.size() / 9;
  OD_TRY(dupload(s, &s->bsr.row_ptr, hb.row_ptr.data(), hb.row_ptr.size()));
  OD_TRY(dupload(s, &s->bsr.col, hb.col.data(), hb.col.size()));
  OD_TRY(dupload(s, &s->bsr.desc_off, hb.desc_off.data(), hb.desc_off.size()));
  OD_TRY(dupload(s, &s->bsr.desc_kind, hb.desc_kind.data(), hb.desc_kind.size()));
  OD_TRY(dupload(s, &s->bsr.gen, hb.gen.data(), hb.gen.size()));
  OD_TRY(dupload(s, &s->bsr.diag_pos, hb.diag_pos.data(), hb.diag_pos.size()));
  OD_TRY(dupload(s, &s->color_off_dev, s->color_off.data(), s->color_off.size()));
  s->hbsr_rp = std::move(hb.row_ptr);   // kept for the mixed-precision slice layout
  s->hbsr_col = std::move(hb.col);
  OD_TRY(dalloc(s, &s->A64, 9 * (size_t)s->bsr.nnzb));
  OD_TRY(pcg_alloc(s));
  // OD_GB300_PCG_PERSISTENT=0 selects the multi-kernel PCG for every preconditioner
  if (const char* e = std::getenv("OD_GB300_PCG_PERSISTENT")) s->pcg.disable_persistent = (e[0] == '0');
  const size_t np = (size_t)std::max(1, s->pcg.n_pad);
  for (double** v : {&s->fint, &s->fext, &s->v, &s->d, &s->a, &s->dp, &s->vp, &s->dv, &s->rhs, &s->tmp, &s->tmp2}) {
    OD_TRY(dalloc(s, v, np));
    OD_CUDA(cudaMemset(*v, 0, sizeof(double) * np));
  }
  // OD_GB300_ASSEMBLY=scatter keeps the per-colour scatter (the path of
  // meshes whose gather lists overflow 32-bit indices) for every scene
  const char* asm_env = std::getenv("OD_GB300_ASSEMBLY");
  const bool scatter_only = asm_env && std::strcmp(asm_env, "scatter") == 0;
  // gather lists of the assembly (per destination its (entry, staged
  // element) sources in element index order), built on the device
  if (!scatter_only) OD_TRY(build_gather_lists(s, (int)np));
  OD_TRY(launch_precompute(s));
  OD_TRY(launch_mass(s));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_scene_create(od_ctx* ctx, int n_nodes, const double* X, int n_tets, const int* tets, int n_facets,
                          const int* facets, int n_cdofs, const int* cdofs, const od_material* mat,
                          od_scene** out) {
  OD_CHECK_ARG(ctx && out && mat, "od_scene_create: NULL argument");
  OD_CHECK_ARG(n_nodes > 0 && X, "od_scene_create: need at least one node");
  OD_CHECK_ARG(n_tets >= 0 && (n_tets == 0 || tets), "od_scene_create: bad element list");
  OD_CHECK_ARG(n_facets >= 0 && (n_facets == 0 || facets), "od_scene_create: bad facet list");
  OD_CHECK_ARG(n_cdofs >= 0 && (n_cdofs == 0 || cdofs), "od_scene_create: bad constraint list");
  OD_CHECK_ARG(mat->kind >= 0 && mat->kind <= 3, "od_scene_create: unknown material kind");
  OD_CHECK_ARG(mat->kind != OD_MATERIAL_COROTATIONAL_PLASTIC ||
                   (mat->yield_criterion >= 0.0 && mat->creep_ratio >= 0.0 && mat->max_plastic_strain >= 0.0),
               "od_scene_create: plastic parameters must be non-negative");
  OD_CHECK_ARG(mat->density > 0 && mat->youngs > 0 && mat->poisson > -1.0 && mat->poisson < 0.5,
               "od_scene_create: material parameters out of range");
  if ((long long)n_nodes * 3 > 0x7fffffffLL) { set_error("od_scene_create: too many nodes"); return OD_ERR_UNSUPPORTED; }
  for (long long i = 0; i < 4LL * n_tets; i++)
    OD_CHECK_ARG(tets[i] >= 0 && tets[i] < n_nodes, "od_scene_create: element node index out of range");
  for (long long i = 0; i < 3LL * n_facets; i++)
    OD_CHECK_ARG(facets[i] >= 0 && facets[i] < n_nodes, "od_scene_create: facet node index out of range");
  for (int i = 0; i < n_cdofs; i++) {
    OD_CHECK_ARG(cdofs[i] >= 0 && cdofs[i] < 3 * n_nodes, "od_scene_create: constrained DOF out of range");
    OD_CHECK_ARG(i == 0 || cdofs[i] > cdofs[i - 1], "od_scene_create: constrained DOFs must be sorted and unique");
  }
  OD_CUDA(cudaSetDevice(ctx->c.device));
  od_scene* sc = new (std::nothrow) od_scene();
  if (!sc) return OD_ERR_OUT_OF_MEMORY;
  Scene* s = &sc->s;
  s->ctx = &ctx->c;
  s->mat = *mat;
  // Lame parameters (corotationalHyperelastic.cpp:8-18, invertibleNeoHookean.cpp:5-9)
  s->lambda = mat->poisson * mat->youngs / ((1.0 + mat->poisson) * (1.0 - 2.0 * mat->poisson));
  s->mu = mat->youngs / (2.0 * (1.0 + mat->poisson));
  s->D[0] = s->lambda + 2.0 * s->mu;
  s->D[1] = s->lambda;
  s->D[2] = s->mu;
  od_status st;
  try {
    st = scene_build(s, n_nodes, X, n_tets, tets, n_facets, facets, n_cdofs, cdofs);
  } catch (const std::bad_alloc&) {
    set_error("od_scene_create: host allocation failed");
    st = OD_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& ex) {
    set_error(std::string("od_scene_create: ") + ex.what());
    st = OD_ERR_UNSUPPORTED;
  }
  if (st != OD_OK) {
    scene_free(s);
    delete sc;
    return st;
  }
  *out = sc;
  return OD_OK;
}

od_status od_scene_destroy(od_scene* scene) {
  if (!scene) return OD_OK;
  scene_free(&scene->s);
  delete scene;
  return OD_OK;
}

od_status od_scene_get_info(od_scene* scene, od_scene_info* info) {
  OD_CHECK_ARG(scene && info, "od_scene_get_info: NULL argument");
  Scene* s = &scene->s;
  info->n_nodes = s->n_nodes;
  info->n_tets = s->n_tets;
  info->n_facets = s->n_facets;
  info->dofs = s->dofs;
  info->num_block_columns = s->nbc;
  info->num_remained_columns = s->nrem;
  info->num_row_indices = (int)s->hrows.size();
  info->num_values = s->nvals;
  info->num_full_blocks = s->bsr.nnzb;
  info->num_colors = (int)s->color_off.size() - 1;
  info->device_bytes = s->device_bytes;
  info->pcg_smem_bytes = s->pcg.smem_bytes;
  return OD_OK;
}

od_status od_scene_pattern(od_scene* scene, int* block_pcol, int* block_rows, int* block_column_oris, int* elem_map) {
  OD_CHECK_ARG(scene, "od_scene_pattern: scene is NULL");
  Scene* s = &scene->s;
  if (block_pcol) memcpy(block_pcol, s->hpcol.data(), sizeof(int) * s->hpcol.size());
  if (block_rows) memcpy(block_rows, s->hrows.data(), sizeof(int) * s->hrows.size());
  if (block_column_oris) memcpy(block_column_oris, s->horis.data(), sizeof(int) * s->horis.size());
  if (elem_map) memcpy(elem_map, s->hemap.data(), sizeof(int) * s->hemap.size());
  return OD_OK;
}

od_status od_scene_set_displacements(od_scene* scene, const double* u) {
  OD_CHECK_ARG(scene && u, "od_scene_set_displacements: NULL argument");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(s->u, u, sizeof(double) * 3 * (size_t)s->n_nodes, cudaMemcpyHostToDevice, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_scene_get_displacements(od_scene* scene, double* u) {
  OD_CHECK_ARG(scene && u, "od_scene_get_displacements: NULL argument");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(u, s->u, sizeof(double) * 3 * (size_t)s->n_nodes, cudaMemcpyDeviceToHost, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_scene_get_positions(od_scene* scene, float* xyz) {
  OD_CHECK_ARG(scene && xyz, "od_scene_get_positions: NULL argument");
  Scene* s = &scene->s;
  std::vector<double> u(3 * (size_t)s->n_nodes);
  OD_TRY(od_scene_get_displacements(scene, u.data()));
  for (size_t i = 0; i < u.size(); i++) xyz[i] = (float)(s->hX[i] + u[i]);
  return OD_OK;
}

od_status od_scene_evaluate(od_scene* scene, double* values, double* f_int) {
  OD_CHECK_ARG(scene, "od_scene_evaluate: scene is NULL");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  // OD_GB300_ELEMENT_DF=1: the mixed-precision path's double-float stiffness
  // contraction (to compare it with the FP64 one)
  const char* dfe = std::getenv("OD_GB300_ELEMENT_DF");
  OD_TRY(launch_eval(s, true, dfe && dfe[0] == '1'));
  if (values) OD_CUDA(cudaMemcpyAsync(values, s->K, sizeof(double) * s->nvals, cudaMemcpyDeviceToHost, s->ctx->stream));
  if (f_int) OD_CUDA(cudaMemcpyAsync(f_int, s->fint, sizeof(double) * s->dofs, cudaMemcpyDeviceToHost, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_scene_element_values(od_scene* scene, double* k78, double* f12) {
  OD_CHECK_ARG(scene && k78 && f12, "od_scene_element_values: NULL argument");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  double *dk = nullptr, *df = nullptr;
  OD_CUDA(cudaMalloc(&dk, sizeof(double) * 78 * (size_t)std::max(1, s->n_tets)));
  cudaError_t e = cudaMalloc(&df, sizeof(double) * 12 * (size_t)std::max(1, s->n_tets));
  if (e != cudaSuccess) { cudaFree(dk); return cuda_fail(e, "cudaMalloc"); }
  od_status st = launch_element_values(s, dk, df);
  if (st == OD_OK) {
    cudaMemcpyAsync(k78, dk, sizeof(double) * 78 * (size_t)s->n_tets, cudaMemcpyDeviceToHost, s->ctx->stream);
    cudaMemcpyAsync(f12, df, sizeof(double) * 12 * (size_t)s->n_tets, cudaMemcpyDeviceToHost, s->ctx->stream);
    e = cudaStreamSynchronize(s->ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(e, "od_scene_element_values");
  }
  cudaFree(dk);
  cudaFree(df);
  return st;
}

od_status od_scene_mass(od_scene* scene, double* values) {
  OD_CHECK_ARG(scene && values, "od_scene_mass: NULL argument");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(values, s->M, sizeof(double) * s->nvals, cudaMemcpyDeviceToHost, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_scene_spmdv(od_scene* scene, const double* values, const double* x, double* y) {
  OD_CHECK_ARG(scene && values && x && y, "od_scene_spmdv: NULL argument");
  Scene* s = &scene->s;
  cudaStream_t st = s->ctx->stream;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(s->work_vals, values, sizeof(double) * s->nvals, cudaMemcpyHostToDevice, st));
  OD_CUDA(cudaMemcpyAsync(s->tmp, x, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, st));
  OD_CUDA(cudaMemcpyAsync(s->tmp2, y, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, st));
  OD_TRY(launch_spmv_lower(s, s->work_vals, 1.0, s->tmp, nullptr, 0.0, nullptr, nullptr, 0.0, nullptr, s->tmp2, true));
  OD_CUDA(cudaMemcpyAsync(y, s->tmp2, sizeof(double) * s->dofs, cudaMemcpyDeviceToHost, st));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

static od_status check_solver(const od_solver_params* p) {
  OD_CHECK_ARG(p, "solver params are NULL");
  OD_CHECK_ARG(p->tol >= 0.0 && p->max_iter >= 0, "solver tolerance / max_iter out of range");
  OD_CHECK_ARG(p->precond >= 0 && p->precond <= OD_PRECOND_IC, "unknown preconditioner");
  OD_CHECK_ARG(p->precision == OD_PRECISION_FP64 || p->precision == OD_PRECISION_MIXED, "unknown precision");
  OD_CHECK_ARG(p->precision == OD_PRECISION_FP64 || p->precond <= OD_PRECOND_IC0,
               "mixed precision supports the none, Jacobi, block-Jacobi and IC(0) preconditioners");
  OD_CHECK_ARG(p->sainv_eps >= 0.0 && p->ldlt_eps >= 0.0 && std::isfinite(p->sainv_eps) &&
                   std::isfinite(p->ldlt_eps),
               "LDL^T drop bounds must be finite and >= 0");
  OD_CHECK_ARG(p->ic_eps >= 0.0 && p->ic_relax >= 0.0 && std::isfinite(p->ic_eps) && std::isfinite(p->ic_relax),
               "incomplete Cholesky epsilon / relaxedScale must be finite and >= 0");
  return OD_OK;
}

od_status od_scene_pcg(od_scene* scene, const double* values, const double* b, double* x,
                       const od_solver_params* params, od_solve_stats* stats) {
  OD_CHECK_ARG(scene && values && b && x, "od_scene_pcg: NULL argument");
  OD_TRY(check_solver(params));
  Scene* s = &scene->s;
  cudaStream_t st = s->ctx->stream;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(s->work_vals, values, sizeof(double) * s->nvals, cudaMemcpyHostToDevice, st));
  OD_CUDA(cudaMemcpyAsync(s->rhs, b, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, st));
  OD_CUDA(cudaMemcpyAsync(s->dv, x, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, st));
  OD_TRY(launch_expand(s, s->work_vals, 1.0, nullptr, 0.0, nullptr, 0.0));
  od_solve_stats ls{};
  OD_TRY(pcg_solve(s, s->rhs, s->dv, params, &ls));
  OD_CUDA(cudaMemcpyAsync(x, s->dv, sizeof(double) * s->dofs, cudaMemcpyDeviceToHost, st));
  OD_TRY(sync_stream(s));
  if (stats) *stats = ls;
  return (od_status)ls.status == OD_ERR_NAN ? OD_ERR_NAN : OD_OK;
}

od_status od_scene_set_loads(od_scene* scene, const double* body, int n_groups, const double* tractions,
                             const int* group_sizes, const int* facet_ids) {
  OD_CHECK_ARG(scene, "od_scene_set_loads: scene is NULL");
  OD_CHECK_ARG(n_groups >= 0 && (n_groups == 0 || (tractions && group_sizes)), "od_scene_set_loads: bad groups");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  // flatten the (facet, traction) pairs in the order given, and list for
  // every free DOF the pairs that load it, in that order
  std::vector<int> fid;
  std::vector<double> tv;
  int q = 0;
  for (int g = 0; g < n_groups; g++) {
    OD_CHECK_ARG(group_sizes[g] >= 0, "od_scene_set_loads: negative group size");
    for (int k = 0; k < group_sizes[g]; k++, q++) {
      OD_CHECK_ARG(facet_ids, "od_scene_set_loads: facet ids are NULL");
      int f = facet_ids[q];
      OD_CHECK_ARG(f >= 0 && f < s->n_facets, "od_scene_set_loads: facet id out of range");
      fid.push_back(f);
      for (int i = 0; i < 3; i++) tv.push_back(tractions[3 * g + i]);
    }
  }
  const int nf = (int)fid.size();
  if (nf > 0) {
    const int np = std::max(1, s->pcg.n_pad);
    std::vector<int> lptr((size_t)np + 1, 0);
    for (int k = 0; k < nf; k++)
      for (int v = 0; v < 3; v++)
        for (int ax = 0; ax < 3; ax++) {
          const int gd = s->hnode_dof[3 * (size_t)s->hfacets[3 * (size_t)fid[k] + v] + ax];
          if (gd >= 0) lptr[(size_t)gd + 1]++;
        }
    for (int i = 0; i < np; i++) lptr[i + 1] += lptr[i];
    std::vector<int> lsrc(std::max(1, lptr[np])), cur(lptr.begin(), lptr.end() - 1);
    for (int k = 0; k < nf; k++)
      for (int v = 0; v < 3; v++)
        for (int ax = 0; ax < 3; ax++) {
          const int gd = s->hnode_dof[3 * (size_t)s->hfacets[3 * (size_t)fid[k] + v] + ax];
          if (gd >= 0) lsrc[cur[gd]++] = k;
        }
    if (nf > s->trac_cap) {
      cudaFree(s->trac_facets);
      cudaFree(s->trac_vec);
      s->trac_facets = nullptr;
      s->trac_vec = nullptr;
      OD_TRY(dalloc(s, &s->trac_facets, (size_t)nf));
      OD_TRY(dalloc(s, &s->trac_vec, 3 * (size_t)nf));
      s->trac_cap = nf;
    }
    if (!s->load_ptr) OD_TRY(dalloc(s, &s->load_ptr, (size_t)np + 1));
    if ((int)lsrc.size() > s->load_cap) {
      cudaFree(s->load_src);
      s->load_src = nullptr;
      OD_TRY(dalloc(s, &s->load_src, lsrc.size()));
      s->load_cap = (int)lsrc.size();
    }
    OD_CUDA(cudaMemcpyAsync(s->trac_facets, fid.data(), sizeof(int) * nf, cudaMemcpyHostToDevice, s->ctx->stream));
    OD_CUDA(cudaMemcpyAsync(s->trac_vec, tv.data(), sizeof(double) * 3 * nf, cudaMemcpyHostToDevice, s->ctx->stream));
    OD_CUDA(cudaMemcpyAsync(s->load_ptr, lptr.data(), sizeof(int) * lptr.size(), cudaMemcpyHostToDevice,
                            s->ctx->stream));
    OD_CUDA(cudaMemcpyAsync(s->load_src, lsrc.data(), sizeof(int) * lsrc.size(), cudaMemcpyHostToDevice,
                            s->ctx->stream));
  }
  s->n_trac = nf;
  s->has_body = body != nullptr;
  if (body) for (int i = 0; i < 3; i++) s->load_body[i] = body[i];
  OD_TRY(launch_loads(s, body, nf, 1.0));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_scene_update_loads(od_scene* scene, double traction_scale) {
  OD_CHECK_ARG(scene, "od_scene_update_loads: scene is NULL");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_TRY(launch_loads(s, s->has_body ? s->load_body : nullptr, s->n_trac, traction_scale));
  return OD_OK;
}

od_status od_scene_set_traction_schedule(od_scene* scene, double frequency_hz, double phase) {
  OD_CHECK_ARG(scene, "od_scene_set_traction_schedule: scene is NULL");
  OD_CHECK_ARG(frequency_hz >= 0.0, "od_scene_set_traction_schedule: negative frequency");
  scene->s.sched_freq = frequency_hz;
  scene->s.sched_phase = phase;
  return OD_OK;
}

od_status od_scene_set_external_forces(od_scene* scene, const double* f_ext) {
  OD_CHECK_ARG(scene && f_ext, "od_scene_set_external_forces: NULL argument");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(s->fext, f_ext, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_scene_get_external_forces(od_scene* scene, double* f_ext) {
  OD_CHECK_ARG(scene && f_ext, "od_scene_get_external_forces: NULL argument");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(f_ext, s->fext, sizeof(double) * s->dofs, cudaMemcpyDeviceToHost, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_integrator_setup(od_scene* scene, const od_integrator_params* p) {
  OD_CHECK_ARG(scene && p, "od_integrator_setup: NULL argument");
  OD_CHECK_ARG(p->kind == OD_INTEGRATOR_BACKWARD_EULER || p->kind == OD_INTEGRATOR_NEWMARK,
               "od_integrator_setup: unknown integrator");
  OD_CHECK_ARG(p->dt > 0.0, "od_integrator_setup: dt must be positive");
  OD_CHECK_ARG(p->kind == OD_INTEGRATOR_BACKWARD_EULER || (p->newton_iters >= 1 && p->nm_beta > 0.0 && p->nm_gamma > 0.0),
               "od_integrator_setup: Newmark needs beta > 0, gamma > 0, newton_iters >= 1");
  OD_TRY(check_solver(&p->solver));
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  s->ip = *p;
  s->has_integrator = true;
  s->time = 0.0;
  const size_t np = sizeof(double) * (size_t)std::max(1, s->pcg.n_pad);
  for (double* v : {s->v, s->d, s->a, s->dp, s->vp, s->dv}) OD_CUDA(cudaMemsetAsync(v, 0, np, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_integrator_update(od_scene* scene, const od_integrator_params* p) {
  OD_CHECK_ARG(scene && p, "od_integrator_update: NULL argument");
  Scene* s = &scene->s;
  OD_CHECK_ARG(s->has_integrator, "od_integrator_update: call od_integrator_setup first");
  OD_CHECK_ARG(p->kind == s->ip.kind, "od_integrator_update: the integrator kind cannot change");
  OD_CHECK_ARG(p->dt > 0.0, "od_integrator_update: dt must be positive");
  OD_CHECK_ARG(p->kind == OD_INTEGRATOR_BACKWARD_EULER || (p->newton_iters >= 1 && p->nm_beta > 0.0 && p->nm_gamma > 0.0),
               "od_integrator_update: Newmark needs beta > 0, gamma > 0, newton_iters >= 1");
  OD_TRY(check_solver(&p->solver));
  s->ip = *p;
  return OD_OK;
}

// one backward-Euler step (nonlinearImplicitBackwardEuler.h:82-101) followed
// by the mesh update u += h v on free DOFs (:103-116)
static od_status be_step(Scene* s, od_step_stats* acc) {
  const od_integrator_params& p = s->ip;
  const int n = s->dofs, T = 256;
  cudaStream_t st = s->ctx->stream;
  const double h = p.dt;
  OD_TRY(launch_eval(s, true, p.solver.precision == OD_PRECISION_MIXED));
  // A0 v with A0 = (h + beta_K) K + alpha_M M + D
  OD_TRY(launch_spmv_lower(s, s->K, h + p.beta_k, s->v, s->M, p.alpha_m, s->v, s->Dm, 1.0, s->v, s->tmp, false));
  OD_KL(s);
  be_rhs_kernel<<<nblk(n, T), T, 0, st>>>(n, h, s->fext, s->fint, s->tmp, s->rhs);
  // A = h A0 + M
  OD_TRY(launch_expand(s, s->K, h * (h + p.beta_k), s->M, h * p.alpha_m + 1.0, s->Dm, h));
  od_solve_stats ss{};
  OD_TRY(pcg_solve(s, s->rhs, s->dv, &p.solver, &ss));
  OD_KL(s);
  add_kernel<<<nblk(n, T), T, 0, st>>>(n, s->dv, s->v);
  OD_KL(s);
  write_mesh_kernel<<<nblk(n, T), T, 0, st>>>(n, s->free_pos, s->v, h, 1, s->u);
  OD_CUDA(cudaGetLastError());
  acc->pcg_iterations += ss.iterations;
  acc->solves += 1;
  acc->max_rel_residual = std::max(acc->max_rel_residual, ss.rel_residual);
  if (ss.status == OD_ERR_NAN) return OD_ERR_NAN;
  if (ss.status != OD_OK && acc->status == OD_OK) acc->status = ss.status;
  return OD_OK;
}

// one Newmark step with Newton iterations on the acceleration (see
// od_integrator_params in include/od_gb300.h and the oracle's definition)
static od_status nm_step(Scene* s, od_step_stats* acc) {
  const od_integrator_params& p = s->ip;
  const int n = s->dofs, T = 256;
  cudaStream_t st = s->ctx->stream;
  const double h = p.dt, bh2 = p.nm_beta * h * h, gh = p.nm_gamma * h;
  OD_KL(s);
  nm_predict_kernel<<<nblk(n, T), T, 0, st>>>(n, h, (0.5 - p.nm_beta) * h * h, (1.0 - p.nm_gamma) * h, s->d, s->v,
                                              s->a, s->dp, s->vp);
  for (int it = 0; it < p.newton_iters; it++) {
    OD_KL(s);
    nm_stage_kernel<<<nblk(n, T), T, 0, st>>>(n, s->free_pos, bh2, gh, p.alpha_m, s->dp, s->vp, s->a, s->u, s->tmp,
                                              s->tmp2);
    OD_TRY(launch_eval(s, true, p.solver.precision == OD_PRECISION_MIXED));
    // y = M (alpha_M v_k + a_k) + beta_K K v_k (+ D v_k)
    OD_TRY(launch_spmv_lower(s, s->M, 1.0, s->tmp, s->K, p.beta_k, s->tmp2, s->Dm, 1.0, s->tmp2, s->rhs, false));
    OD_KL(s);
    nm_residual_kernel<<<nblk(n, T), T, 0, st>>>(n, s->fext, s->fint, s->rhs, s->rhs);
    // A = (1 + gamma h alpha_M) M + (gamma h beta_K + beta h^2) K + gamma h D
    OD_TRY(launch_expand(s, s->K, gh * p.beta_k + bh2, s->M, 1.0 + gh * p.alpha_m, s->Dm, gh));
    OD_CUDA(cudaMemsetAsync(s->dv, 0, sizeof(double) * (size_t)s->pcg.n_pad, st));
    s->pcg.x_zero = true;
    od_solve_stats ss{};
    OD_TRY(pcg_solve(s, s->rhs, s->dv, &p.solver, &ss));
    OD_KL(s);
    add_kernel<<<nblk(n, T), T, 0, st>>>(n, s->dv, s->a);
    acc->pcg_iterations += ss.iterations;
    acc->solves += 1;
    acc->max_rel_residual = std::max(acc->max_rel_residual, ss.rel_residual);
    if (ss.status == OD_ERR_NAN) return OD_ERR_NAN;
    if (ss.status != OD_OK && acc->status == OD_OK) acc->status = ss.status;
  }
  OD_KL(s);
  nm_correct_kernel<<<nblk(n, T), T, 0, st>>>(n, s->free_pos, bh2, gh, s->dp, s->vp, s->a, s->d, s->v, s->u);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status od_step(od_scene* scene, int n_steps, od_step_stats* stats) {
  OD_CHECK_ARG(scene, "od_step: scene is NULL");
  OD_CHECK_ARG(n_steps >= 0, "od_step: negative step count");
  Scene* s = &scene->s;
  if (!s->has_integrator) { set_error("od_step: call od_integrator_setup first"); return OD_ERR_INVALID_ARG; }
  OD_CUDA(cudaSetDevice(s->ctx->device));
  od_step_stats acc{};
  od_status st = OD_OK;
  if (!s->ev_step[0]) {
    OD_CUDA(cudaEventCreate(&s->ev_step[0]));
    OD_CUDA(cudaEventCreate(&s->ev_step[1]));
  }
  OD_CUDA(cudaEventRecord(s->ev_step[0], s->ctx->stream));
  for (int k = 0; k < n_steps && st == OD_OK; k++) {
    if (s->sched_freq > 0.0) {
      const double t = s->time + s->ip.dt;
      st = launch_loads(s, s->has_body ? s->load_body : nullptr, s->n_trac,
                        std::sin(2.0 * 3.14159265358979323846 * s->sched_freq * t + s->sched_phase));
      if (st != OD_OK) break;
    }
    // no free DOF: nothing moves (every displacement is prescribed)
    if (s->dofs > 0) st = s->ip.kind == OD_INTEGRATOR_NEWMARK ? nm_step(s, &acc) : be_step(s, &acc);
    if (st == OD_OK) { acc.steps++; s->time += s->ip.dt; }
  }
  cudaEventRecord(s->ev_step[1], s->ctx->stream);
  s->ctx->host_syncs++;
  cudaError_t e = cudaStreamSynchronize(s->ctx->stream);
  if (e != cudaSuccess && st == OD_OK) st = cuda_fail(e, "od_step");
  float ms = 0.f;
  if (st == OD_OK && cudaEventElapsedTime(&ms, s->ev_step[0], s->ev_step[1]) == cudaSuccess) acc.device_ms = ms;
  if (st != OD_OK && acc.status == OD_OK) acc.status = st;
  if (stats) *stats = acc;
  return st;
}

od_status od_get_state(od_scene* scene, double* d, double* v, double* a) {
  OD_CHECK_ARG(scene, "od_get_state: scene is NULL");
  Scene* s = &scene->s;
  cudaStream_t st = s->ctx->stream;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  const size_t nb = sizeof(double) * (size_t)s->dofs;
  if (d) OD_CUDA(cudaMemcpyAsync(d, s->d, nb, cudaMemcpyDeviceToHost, st));
  if (v) OD_CUDA(cudaMemcpyAsync(v, s->v, nb, cudaMemcpyDeviceToHost, st));
  if (a) OD_CUDA(cudaMemcpyAsync(a, s->a, nb, cudaMemcpyDeviceToHost, st));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_set_state(od_scene* scene, const double* d, const double* v, const double* a) {
  OD_CHECK_ARG(scene, "od_set_state: scene is NULL");
  Scene* s = &scene->s;
  cudaStream_t st = s->ctx->stream;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  const size_t nb = sizeof(double) * (size_t)s->dofs;
  if (d) OD_CUDA(cudaMemcpyAsync(s->d, d, nb, cudaMemcpyHostToDevice, st));
  if (v) OD_CUDA(cudaMemcpyAsync(s->v, v, nb, cudaMemcpyHostToDevice, st));
  if (a) OD_CUDA(cudaMemcpyAsync(s->a, a, nb, cudaMemcpyHostToDevice, st));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

// blob: magic, version, n_nodes, dofs, time, u (3 n_nodes), d, v, a, dv, f_ext (dofs each)
static const uint64_t kMagic = 0x3130305344474f44ull;  // "DOGSD001"

static size_t blob_size(const Scene* s) {
  return 4 * sizeof(uint64_t) +
         sizeof(double) * (1 + 3 * (size_t)s->n_nodes + 5 * (size_t)s->dofs + (s->plastic ? 9 * (size_t)s->n_tets : 0));
}

od_status od_scene_save(od_scene* scene, void* buf, size_t* size) {
  OD_CHECK_ARG(scene && size, "od_scene_save: NULL argument");
  Scene* s = &scene->s;
  const size_t need = blob_size(s);
  if (!buf) { *size = need; return OD_OK; }
  OD_CHECK_ARG(*size >= need, "od_scene_save: buffer too small");
  OD_CUDA(cudaSetDevice(s->ctx->device));
  uint64_t* hd = (uint64_t*)buf;
  hd[0] = kMagic; hd[1] = s->plastic ? 2 : 1; hd[2] = (uint64_t)s->n_nodes; hd[3] = (uint64_t)s->dofs;
  double* p = (double*)(hd + 4);
  p[0] = s->time;
  p += 1;
  cudaStream_t st = s->ctx->stream;
  OD_CUDA(cudaMemcpyAsync(p, s->u, sizeof(double) * 3 * s->n_nodes, cudaMemcpyDeviceToHost, st));
  p += 3 * (size_t)s->n_nodes;
  for (double* v : {s->d, s->v, s->a, s->dv, s->fext}) {
    OD_CUDA(cudaMemcpyAsync(p, v, sizeof(double) * s->dofs, cudaMemcpyDeviceToHost, st));
    p += s->dofs;
  }
  if (s->plastic) OD_CUDA(cudaMemcpyAsync(p, s->plastic, sizeof(double) * 9 * s->n_tets, cudaMemcpyDeviceToHost, st));
  OD_TRY(sync_stream(s));
  *size = need;
  return OD_OK;
}

od_status od_scene_load(od_scene* scene, const void* buf, size_t size) {
  OD_CHECK_ARG(scene && buf, "od_scene_load: NULL argument");
  Scene* s = &scene->s;
  const size_t need = blob_size(s);
  OD_CHECK_ARG(size >= need, "od_scene_load: blob too small");
  const uint64_t* hd = (const uint64_t*)buf;
  OD_CHECK_ARG(hd[0] == kMagic && hd[1] == (s->plastic ? 2u : 1u), "od_scene_load: not a blob of this kind of scene");
  OD_CHECK_ARG(hd[2] == (uint64_t)s->n_nodes && hd[3] == (uint64_t)s->dofs, "od_scene_load: blob is for another scene");
  OD_CUDA(cudaSetDevice(s->ctx->device));
  const double* p = (const double*)(hd + 4);
  s->time = p[0];
  p += 1;
  cudaStream_t st = s->ctx->stream;
  OD_CUDA(cudaMemcpyAsync(s->u, p, sizeof(double) * 3 * s->n_nodes, cudaMemcpyHostToDevice, st));
  p += 3 * (size_t)s->n_nodes;
  for (double* v : {s->d, s->v, s->a, s->dv, s->fext}) {
    OD_CUDA(cudaMemcpyAsync(v, p, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, st));
    p += s->dofs;
  }
  if (s->plastic) OD_CUDA(cudaMemcpyAsync(s->plastic, p, sizeof(double) * 9 * s->n_tets, cudaMemcpyHostToDevice, st));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

// plastic strain in the caller's element order (the device keeps it [9][tet]
// in colour order)
od_status od_scene_get_plastic_strain(od_scene* scene, double* out) {
  OD_CHECK_ARG(scene && out, "od_scene_get_plastic_strain: NULL argument");
  Scene* s = &scene->s;
  OD_CHECK_ARG(s->plastic, "od_scene_get_plastic_strain: not a plastic scene");
  OD_CUDA(cudaSetDevice(s->ctx->device));
  std::vector<double> h(9 * (size_t)s->n_tets);
  OD_CUDA(cudaMemcpyAsync(h.data(), s->plastic, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s->ctx->stream));
  OD_TRY(sync_stream(s));
  const size_t ne = s->n_tets;
  for (size_t k = 0; k < ne; k++)
    for (int i = 0; i < 9; i++) out[9 * (size_t)s->elem_perm[k] + i] = h[(size_t)i * ne + k];
  return OD_OK;
}

od_status od_scene_set_plastic_strain(od_scene* scene, const double* in) {
  OD_CHECK_ARG(scene && in, "od_scene_set_plastic_strain: NULL argument");
  Scene* s = &scene->s;
  OD_CHECK_ARG(s->plastic, "od_scene_set_plastic_strain: not a plastic scene");
  OD_CUDA(cudaSetDevice(s->ctx->device));
  const size_t ne = s->n_tets;
  std::vector<double> h(9 * ne);
  for (size_t k = 0; k < ne; k++)
    for (int i = 0; i < 9; i++) h[(size_t)i * ne + k] = in[9 * (size_t)s->elem_perm[k] + i];
  OD_CUDA(cudaMemcpyAsync(s->plastic, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

}  // extern "C"
