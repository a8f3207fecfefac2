// Incomplete LDL^T preconditioner (solver/inLDLTPreconditioner.cpp).
//
// The factor is made on the host (od_rif.cpp: a strictly sequential sweep
// with data-dependent fill) from A in the reference's lower value layout,
// then uploaded as
//   forward  : L by rows (CSR, columns ascending)       -> L y = r
//   backward : L by columns (the reference's storage)   -> L^T z = D^-1 y
// and applied on the device by one cooperative launch per apply.  Rows are
// listed by dependency level (level of a row = 1 + the highest level of the
// rows it reads; forward and backward levels apart), and warp w of the W
// co-resident warps takes entries w, w+W, ... of the forward list, then of
// the backward list.  y and z are filled with an all-ones NaN before the
// launch (a pattern no arithmetic result has); a row waits (bounded) until
// the values it reads are no longer that pattern, read with acquire loads,
// and publishes its own value with one release store: the value is its
// own ready flag.  Progress: the first unfinished entry of a list is at the
// head of its warp's queue and reads only rows of lower levels, listed
// before it and so finished; every warp finishes its forward entries
// before its first backward wait.
//
// Dependent FP64 operations cost 64 cycles each on this part (a shuffle
// plus an add about 108), so a row's products are summed by a fixed
// 5-level butterfly over the warp rather than one after another: the result
// is deterministic and within rounding of the reference's sequential sums
// (solvePreconditionerSystem, :151-184).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "od_internal.h"

namespace od {

struct LdltSys {
  RifColumns cols;
  RifFactor f;
  int n = 0, n_pad = 0, nvals = 0;
  long long cap = 0;                 // entry capacity of the device arrays
  double* lo_dev = nullptr;          // A in the reference lower layout (device)
  double* lo_host = nullptr;         // pinned mirror
  int *f_rp = nullptr, *f_ci = nullptr, *b_cp = nullptr, *b_ri = nullptr;
  int *ord_f = nullptr, *ord_b = nullptr;   // rows by forward / backward level
  double *f_val = nullptr, *b_val = nullptr, *dinv = nullptr, *y = nullptr;
  int *err = nullptr, *err_host = nullptr;
  int grid = 0;                      // co-resident CTAs of the apply
  int depth_f = 0, depth_b = 0;      // longest dependency chains of the two sweeps (rows)
  bool have = false;                 // a factor is loaded
  std::vector<int> h_rp, h_ci, h_cp, h_of, h_ob;  // host staging of the sweep arrays
  std::vector<double> h_fval;
};

namespace {

constexpr int kLdltThreads = 256;
constexpr unsigned kLdltSpinLimit = 1u << 21;
constexpr unsigned long long kPending = 0xffffffffffffffffull;   // "not yet written" (a NaN)

__device__ __forceinline__ unsigned long long ld_acquire_u64(const double* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_f64(double* p, double x) {
  asm volatile("st.release.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(__double_as_longlong(x)) : "memory");
}

// bounded wait for *p to be written; after a timeout anywhere (err set) no
// thread waits any more, so the launch ends promptly and the host reports it
__device__ __forceinline__ double wait_value(const double* p, int* err) {
  unsigned long long v = ld_acquire_u64(p);
  for (unsigned k = 1; v == kPending && k < kLdltSpinLimit; k++) {
    if ((k & 1023u) == 0 && *(volatile int*)err) return 0.0;
    v = ld_acquire_u64(p);
  }
  if (v == kPending) {
    atomicOr(err, 1);
    return 0.0;
  }
  return __longlong_as_double((long long)v);
}

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__global__ void __launch_bounds__(kLdltThreads) ldlt_apply_kernel(
    int n, int n_pad, const int* __restrict__ frp, const int* __restrict__ fci, const double* __restrict__ fval,
    const int* __restrict__ bcp, const int* __restrict__ bri, const double* __restrict__ bval,
    const int* __restrict__ ord_f, const int* __restrict__ ord_b, const double* __restrict__ dinv,
    const double* __restrict__ r, double* y, double* z, int* __restrict__ err, const SolveScalars* sc) {
  if (sc && *(volatile const int*)&sc->done) return;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int W = gridDim.x * wpb;
  const int w = blockIdx.x * wpb + (threadIdx.x >> 5);
  // padding rows carry the identity
  for (int i = n + blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += gridDim.x * blockDim.x) z[i] = r[i];

  // forward: y_j = r_j - sum_c L_jc y_c
  for (int t = w; t < n; t += W) {
    const int j = ord_f[t];
    double s = r[j];
    const int e = frp[j + 1];
    for (int q0 = frp[j]; q0 < e; q0 += 32) {
      const int q = q0 + lane;
      double prod = 0.0;
      if (q < e) {
        const int c = fci[q];
        const double l = fval[q];
        prod = l * wait_value(y + c, err);
      }
      s -= warp_sum(prod);
    }
    if (lane == 0) st_release_f64(y + j, s);
  }

  // backward: z_i = y_i d_i^-1 - sum_r z_r L_ri
  for (int t = w; t < n; t += W) {
    const int i = ord_b[t];
    const int e = bcp[i + 1];
    double dot = 0.0;
    for (int q0 = bcp[i]; q0 < e; q0 += 32) {
      const int q = q0 + lane;
      double prod = 0.0;
      if (q < e) {
        const int rr = bri[q];
        const double l = bval[q];
        prod = wait_value(z + rr, err) * l;
      }
      dot += warp_sum(prod);
    }
    if (lane == 0) st_release_f64(z + i, wait_value(y + i, err) * dinv[i] - dot);
  }
}

// A in the reference's lower layout from the last expansion's sources, with
// the arithmetic of expand_kernel (so it equals A64's entries)
__global__ void combine_lower_kernel(int nv, const double* __restrict__ v1, double c1, const double* __restrict__ v2,
                                     double c2, const double* __restrict__ v3, double c3, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  double val = c1 * v1[i];
  if (v2) val += c2 * v2[i];
  if (v3) val += c3 * v3[i];
  out[i] = val;
}

template <class T>
od_status grow(T** p, long long need, long long& bytes) {
  cudaFree(*p);
  *p = nullptr;
  OD_CUDA(cudaMalloc(p, sizeof(T) * (size_t)std::max(1LL, need)));
  bytes += (long long)sizeof(T) * need;
  return OD_OK;
}

od_status ldlt_alloc(Scene* s) {
  Pcg& P = s->pcg;
  if (P.ldlt) return OD_OK;
  LdltSys* l = new LdltSys();
  P.ldlt = l;
  l->n = s->dofs;
  l->n_pad = P.n_pad;
  l->nvals = s->nvals;
  rif_columns(s->dofs, s->nbc, s->hpcol, s->hrows, l->cols);
  const int n = l->n;
  OD_CUDA(cudaMalloc(&l->lo_dev, sizeof(double) * (size_t)std::max(1, l->nvals)));
  OD_CUDA(cudaMallocHost(&l->lo_host, sizeof(double) * (size_t)std::max(1, l->nvals)));
  for (int** a : {&l->f_rp, &l->b_cp, &l->ord_f, &l->ord_b}) OD_CUDA(cudaMalloc(a, sizeof(int) * (size_t)(n + 1)));
  for (double** a : {&l->dinv, &l->y}) OD_CUDA(cudaMalloc(a, sizeof(double) * (size_t)std::max(1, n)));
  OD_CUDA(cudaMalloc(&l->err, sizeof(int)));
  OD_CUDA(cudaMemset(l->err, 0, sizeof(int)));
  OD_CUDA(cudaMallocHost(&l->err_host, sizeof(int)));
  s->device_bytes += (long long)sizeof(double) * l->nvals + (long long)(sizeof(int) * 4 + sizeof(double) * 2) * n;
  // co-resident CTAs for the cooperative apply
  int dev_coop = 0, per_sm = 0;
  OD_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, s->ctx->device));
  OD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ldlt_apply_kernel, kLdltThreads, 0));
  if (!dev_coop || per_sm < 1) {
    set_error("the LDL^T apply needs cooperative launch");
    return OD_ERR_UNSUPPORTED;
  }
  // two CTAs (16 warps) per SM: each level's rows spread over 4864 warps;
  // more warps only add polling traffic
  int per = 2;
  if (const char* e = std::getenv("OD_GB300_LDLT_CTAS_PER_SM")) per = std::max(1, std::atoi(e));
  const int want = (n + (kLdltThreads / 32) - 1) / (kLdltThreads / 32);   // one warp per row at most
  l->grid = std::max(1, std::min(std::min(per, per_sm) * s->ctx->num_sms, want));
  return OD_OK;
}

}  // namespace

void ldlt_free(LdltSys* l) {
  if (!l) return;
  for (double* p : {l->lo_dev, l->f_val, l->b_val, l->dinv, l->y}) cudaFree(p);
  for (int* p : {l->f_rp, l->f_ci, l->b_cp, l->b_ri, l->ord_f, l->ord_b, l->err}) cudaFree(p);
  if (l->lo_host) cudaFreeHost(l->lo_host);
  if (l->err_host) cudaFreeHost(l->err_host);
  delete l;
}

od_status ldlt_factor(Scene* s, const double* host_values, double sainv_eps, double ldlt_eps) {
  OD_TRY(ldlt_alloc(s));
  LdltSys* l = s->pcg.ldlt;
  cudaStream_t strm = s->ctx->stream;
  const auto t0 = std::chrono::steady_clock::now();
  const double* vals = host_values;
  if (!vals) {
    if (!s->lo.v1) {
      set_error("LDL^T factor: no system matrix has been formed");
      return OD_ERR_INTERNAL;
    }
    if (l->nvals > 0) {
      OD_KL(s);
      combine_lower_kernel<<<(l->nvals + 255) / 256, 256, 0, strm>>>(l->nvals, s->lo.v1, s->lo.c1, s->lo.v2, s->lo.c2,
                                                                     s->lo.v3, s->lo.c3, l->lo_dev);
      OD_CUDA(cudaGetLastError());
      OD_CUDA(cudaMemcpyAsync(l->lo_host, l->lo_dev, sizeof(double) * l->nvals, cudaMemcpyDeviceToHost, strm));
    }
    OD_TRY(sync_stream(s));
    vals = l->lo_host;
  }
  const int n = l->n;
  rif_factor(l->cols, vals, sainv_eps, ldlt_eps, l->f);
  const RifFactor& F = l->f;
  const long long nnz = (long long)F.val.size();
  if (nnz > 0x7fffffffLL) {
    set_error("LDL^T factor exceeds 2^31 entries");
    return OD_ERR_OUT_OF_MEMORY;
  }
  // forward CSR (columns ascending in every row) by a counting transpose
  l->h_rp.assign(n + 1, 0);
  for (long long q = 0; q < nnz; q++) l->h_rp[F.row[q] + 1]++;
  for (int i = 0; i < n; i++) l->h_rp[i + 1] += l->h_rp[i];
  l->h_ci.resize(nnz);
  l->h_fval.resize(nnz);
  {
    std::vector<int> fill(l->h_rp.begin(), l->h_rp.end() - 1);
    for (int c = 0; c + 1 < n; c++)
      for (int q = F.pcol[c]; q < F.pcol[c + 1]; q++) {
        const int at = fill[F.row[q]]++;
        l->h_ci[at] = c;
        l->h_fval[at] = F.val[q];
      }
  }
  // dependency levels of the two sweeps and the rows listed by level (a
  // counting sort; forward ties by ascending row, backward by descending)
  {
    std::vector<int> lev(n, 0);
    auto list_by_level = [&](int depth, bool ascending, std::vector<int>& ord) {
      std::vector<int> start(depth + 1, 0);
      for (int i = 0; i < n; i++) start[lev[i] + 1]++;
      for (int k = 0; k < depth; k++) start[k + 1] += start[k];
      ord.resize(n);
      for (int t = 0; t < n; t++) {
        const int i = ascending ? t : n - 1 - t;
        ord[start[lev[i]]++] = i;
      }
    };
    int df = 0, db = 0;
    for (int j = 0; j < n; j++) {
      int m = 0;
      for (int q = l->h_rp[j]; q < l->h_rp[j + 1]; q++) m = std::max(m, lev[l->h_ci[q]] + 1);
      lev[j] = m;
      df = std::max(df, m + 1);
    }
    list_by_level(df, true, l->h_of);
    std::fill(lev.begin(), lev.end(), 0);
    for (int i = n - 2; i >= 0; i--) {
      int m = 0;
      for (int q = F.pcol[i]; q < F.pcol[i + 1]; q++) m = std::max(m, lev[F.row[q]] + 1);
      lev[i] = m;
      db = std::max(db, m + 1);
    }
    if (n > 0) db = std::max(db, 1);
    list_by_level(db, false, l->h_ob);
    l->depth_f = df;
    l->depth_b = db;
  }
  // backward column pointers: the reference's pcol (n entries) closed by nnz
  l->h_cp.assign(F.pcol.begin(), F.pcol.end());
  l->h_cp.resize(n + 1, (int)nnz);
  if (nnz > l->cap) {
    long long cap = std::max(nnz, l->cap + l->cap / 2);
    long long bytes = 0;
    OD_TRY(grow(&l->f_ci, cap, bytes));
    OD_TRY(grow(&l->b_ri, cap, bytes));
    OD_TRY(grow(&l->f_val, cap, bytes));
    OD_TRY(grow(&l->b_val, cap, bytes));
    s->device_bytes += bytes - (long long)(2 * sizeof(int) + 2 * sizeof(double)) * l->cap;
    l->cap = cap;
  }
  if (n > 0) {
    OD_CUDA(cudaMemcpyAsync(l->f_rp, l->h_rp.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->b_cp, l->h_cp.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->dinv, F.dinv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->ord_f, l->h_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->ord_b, l->h_ob.data(), sizeof(int) * n, cudaMemcpyHostToDevice, strm));
  }
  if (nnz > 0) {
    OD_CUDA(cudaMemcpyAsync(l->f_ci, l->h_ci.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->f_val, l->h_fval.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->b_ri, F.row.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->b_val, F.val.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, strm));
  }
  // the staging vectors are read by the copies: finish them before returning
  OD_TRY(sync_stream(s));
  l->have = true;
  Ctx* ctx = s->ctx;
  ctx->ldlt_factors++;
  ctx->ldlt_nnz = nnz;
  ctx->ldlt_levels = (long long)l->depth_f + l->depth_b;
  ctx->ldlt_factor_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return OD_OK;
}

od_status ldlt_apply(Scene* s, const double* r, double* z, const SolveScalars* sc) {
  LdltSys* l = s->pcg.ldlt;
  if (!l || !l->have) {
    set_error("LDL^T apply without a factor");
    return OD_ERR_INTERNAL;
  }
  Ctx* ctx = s->ctx;
  cudaStream_t strm = ctx->stream;
  int n = l->n, n_pad = l->n_pad;
  const bool prof = ctx->profiling && ctx->ev_pool.size() >= 2;
  if (prof) OD_CUDA(cudaEventRecord(ctx->ev_pool[ctx->ev_pool.size() - 2], strm));
  const int* frp = l->f_rp;
  const int* fci = l->f_ci;
  const double* fval = l->f_val;
  const int* bcp = l->b_cp;
  const int* bri = l->b_ri;
  const double* bval = l->b_val;
  const int* of = l->ord_f;
  const int* ob = l->ord_b;
  const double* dinv = l->dinv;
  double* y = l->y;
  int* err = l->err;
  void* args[] = {(void*)&n,   (void*)&n_pad, (void*)&frp, (void*)&fci, (void*)&fval, (void*)&bcp,
                  (void*)&bri, (void*)&bval,  (void*)&of,  (void*)&ob,  (void*)&dinv, (void*)&r,
                  (void*)&y,   (void*)&z,     (void*)&err, (void*)&sc};
  // every value starts "not yet written" (all-ones bytes)
  if (n > 0) {
    OD_CUDA(cudaMemsetAsync(y, 0xff, sizeof(double) * (size_t)n, strm));
    OD_CUDA(cudaMemsetAsync(z, 0xff, sizeof(double) * (size_t)n, strm));
  }
  OD_KL(s);
  OD_CUDA(cudaLaunchCooperativeKernel((void*)ldlt_apply_kernel, dim3(l->grid), dim3(kLdltThreads), args, 0, strm));
  if (prof) {
    OD_CUDA(cudaEventRecord(ctx->ev_pool[ctx->ev_pool.size() - 1], strm));
    OD_CUDA(cudaEventSynchronize(ctx->ev_pool[ctx->ev_pool.size() - 1]));
    float ms = 0.f;
    OD_CUDA(cudaEventElapsedTime(&ms, ctx->ev_pool[ctx->ev_pool.size() - 2], ctx->ev_pool[ctx->ev_pool.size() - 1]));
    // an apply that returned at once (solve already converged) is not counted
    bool ran = true;
    if (sc) {
      SolveScalars h;
      OD_CUDA(cudaMemcpy(&h, sc, sizeof(SolveScalars), cudaMemcpyDeviceToHost));
      ran = !h.done;
    }
    if (ran) {
      ctx->ldlt_applies++;
      ctx->ldlt_apply_ms += ms;
      ctx->ldlt_apply_bytes += 2.0 * 12.0 * (double)l->f.val.size() + 48.0 * n;
    }
  }
  return OD_OK;
}

od_status ldlt_check(Scene* s) {
  LdltSys* l = s->pcg.ldlt;
  if (!l) return OD_OK;
  cudaStream_t strm = s->ctx->stream;
  OD_CUDA(cudaMemcpyAsync(l->err_host, l->err, sizeof(int), cudaMemcpyDeviceToHost, strm));
  OD_TRY(sync_stream(s));
  if (*l->err_host) {
    OD_CUDA(cudaMemsetAsync(l->err, 0, sizeof(int), strm));
    set_error("LDL^T sweep: a bounded wait on a row flag ran out");
    return OD_ERR_DEVICE_TIMEOUT;
  }
  return OD_OK;
}

}  // namespace od

// ------------------------------------------------------------------ C ABI
using namespace od;

extern "C" od_status od_scene_ldlt_factor(od_scene* scene, const double* values, double sainv_eps, double ldlt_eps,
                                          long long* nnz) {
  OD_CHECK_ARG(scene && values, "od_scene_ldlt_factor: NULL argument");
  OD_CHECK_ARG(sainv_eps >= 0.0 && ldlt_eps >= 0.0 && std::isfinite(sainv_eps) && std::isfinite(ldlt_eps),
               "od_scene_ldlt_factor: drop bounds must be finite and >= 0");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_TRY(ldlt_factor(s, values, sainv_eps, ldlt_eps));
  if (nnz) *nnz = (long long)s->pcg.ldlt->f.val.size();
  return OD_OK;
}

extern "C" od_status od_scene_ldlt_get(od_scene* scene, double* values, int* rows, int* pcol, double* inv_diag) {
  OD_CHECK_ARG(scene, "od_scene_ldlt_get: scene is NULL");
  Scene* s = &scene->s;
  LdltSys* l = s->pcg.ldlt;
  OD_CHECK_ARG(l && l->have, "od_scene_ldlt_get: no factor (call od_scene_ldlt_factor first)");
  const RifFactor& F = l->f;
  if (values && !F.val.empty()) std::copy(F.val.begin(), F.val.end(), values);
  if (rows && !F.row.empty()) std::copy(F.row.begin(), F.row.end(), rows);
  if (pcol && !F.pcol.empty()) std::copy(F.pcol.begin(), F.pcol.end(), pcol);
  if (inv_diag && !F.dinv.empty()) std::copy(F.dinv.begin(), F.dinv.end(), inv_diag);
  return OD_OK;
}

extern "C" od_status od_scene_ldlt_apply(od_scene* scene, const double* rhs, double* result) {
  OD_CHECK_ARG(scene && rhs && result, "od_scene_ldlt_apply: NULL argument");
  Scene* s = &scene->s;
  LdltSys* l = s->pcg.ldlt;
  OD_CHECK_ARG(l && l->have, "od_scene_ldlt_apply: no factor (call od_scene_ldlt_factor first)");
  OD_CUDA(cudaSetDevice(s->ctx->device));
  Pcg& P = s->pcg;
  cudaStream_t strm = s->ctx->stream;
  OD_CUDA(cudaMemsetAsync(P.r, 0, sizeof(double) * P.n_pad, strm));
  if (s->dofs > 0)
    OD_CUDA(cudaMemcpyAsync(P.r, rhs, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, strm));
  OD_TRY(ldlt_apply(s, P.r, P.z, nullptr));
  if (s->dofs > 0)
    OD_CUDA(cudaMemcpyAsync(result, P.z, sizeof(double) * s->dofs, cudaMemcpyDeviceToHost, strm));
  OD_TRY(sync_stream(s));
  return ldlt_check(s);
}
