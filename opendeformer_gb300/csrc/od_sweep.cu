// Preconditioners applied by two triangular sweeps, with the factor made on
// the host: the reference's incomplete LDL^T (solver/inLDLTPreconditioner.cpp,
// factor in od_rif.cpp) and its threshold incomplete Cholesky
// (solver/inCholeskyPreconditioner.cpp, factor in od_ric.cpp).  Both
// factorisations are strictly sequential sweeps with data-dependent fill,
// so they run on the host, bit-identical to the reference's; the device
// takes the part that runs every PCG iteration.
//
// A factor is uploaded as its strictly lower part L (unit diagonal for
// LDL^T) and a diagonal array:
//   forward  : L by rows (CSR, columns ascending)       -> L y = r
//   backward : L by columns (the reference's order)     -> L^T z = y
//   LDL^T    : y_j = r_j - sum L_jc y_c;          z_i = y_i D_ii^-1 - sum z_r L_ri
//   IC       : y_j = (r_j - sum L_jc y_c) / L_jj;  z_i = (y_i - sum z_r L_ri) / L_ii
// and applied by one cooperative launch per apply.  Rows are listed by
// dependency level (level of a row = 1 + the highest level of the rows it
// reads; forward and backward levels apart), and warp w of the W
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
// is deterministic and within rounding of the reference's sequential sums.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "od_internal.h"

namespace od {

struct SweepSys {
  int kind = -1;                     // factor loaded: OD_PRECOND_LDLT or OD_PRECOND_IC, -1 none
  RifColumns rif_cols;               // (built on first use of each kind)
  RicColumns ric_cols;
  RifFactor rif;                     // the last factors in the reference's storage
  RicFactor ric;
  int n = 0, n_pad = 0, nvals = 0;
  long long nnz = 0;                 // strictly lower entries of the loaded factor
  long long cap = 0;                 // entry capacity of the device arrays
  double* lo_dev = nullptr;          // A in the reference lower layout (device)
  double* lo_host = nullptr;         // pinned mirror
  int *f_rp = nullptr, *f_ci = nullptr, *b_cp = nullptr, *b_ri = nullptr;
  int *ord_f = nullptr, *ord_b = nullptr;   // rows by forward / backward level
  double *f_val = nullptr, *b_val = nullptr, *diag = nullptr, *y = nullptr;
  int *err = nullptr, *err_host = nullptr;
  int grid = 0;                      // co-resident CTAs of the apply
  int depth_f = 0, depth_b = 0;      // longest dependency chains of the two sweeps (rows)
  // host staging of the sweep arrays
  std::vector<int> h_rp, h_ci, h_cp, h_ri, h_of, h_ob;
  std::vector<double> h_fval, h_bval, h_diag;
};

namespace {

constexpr int kSweepThreads = 256;
constexpr unsigned kSweepSpinLimit = 1u << 21;
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
  for (unsigned k = 1; v == kPending && k < kSweepSpinLimit; k++) {
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

// IC = 0: LDL^T (diag = D^-1), IC = 1: Cholesky (diag = L_ii)
template <int IC>
__global__ void __launch_bounds__(kSweepThreads) sweep_apply_kernel(
    int n, int n_pad, const int* __restrict__ frp, const int* __restrict__ fci, const double* __restrict__ fval,
    const int* __restrict__ bcp, const int* __restrict__ bri, const double* __restrict__ bval,
    const int* __restrict__ ord_f, const int* __restrict__ ord_b, const double* __restrict__ diag,
    const double* __restrict__ r, double* y, double* z, int* __restrict__ err, const SolveScalars* sc) {
  if (sc && *(volatile const int*)&sc->done) return;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int W = gridDim.x * wpb;
  const int w = blockIdx.x * wpb + (threadIdx.x >> 5);
  // padding rows carry the identity
  for (int i = n + blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += gridDim.x * blockDim.x) z[i] = r[i];

  // forward
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
    if (lane == 0) st_release_f64(y + j, IC ? s / diag[j] : s);
  }

  // backward
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
    if (lane == 0) {
      const double yi = wait_value(y + i, err);
      st_release_f64(z + i, IC ? (yi - dot) / diag[i] : yi * diag[i] - dot);
    }
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

od_status sweep_alloc(Scene* s) {
  Pcg& P = s->pcg;
  if (P.sweep) return OD_OK;
  SweepSys* l = new SweepSys();
  P.sweep = l;
  l->n = s->dofs;
  l->n_pad = P.n_pad;
  l->nvals = s->nvals;
  const int n = l->n;
  OD_CUDA(cudaMalloc(&l->lo_dev, sizeof(double) * (size_t)std::max(1, l->nvals)));
  OD_CUDA(cudaMallocHost(&l->lo_host, sizeof(double) * (size_t)std::max(1, l->nvals)));
  for (int** a : {&l->f_rp, &l->b_cp, &l->ord_f, &l->ord_b}) OD_CUDA(cudaMalloc(a, sizeof(int) * (size_t)(n + 1)));
  for (double** a : {&l->diag, &l->y}) OD_CUDA(cudaMalloc(a, sizeof(double) * (size_t)std::max(1, n)));
  OD_CUDA(cudaMalloc(&l->err, sizeof(int)));
  OD_CUDA(cudaMemset(l->err, 0, sizeof(int)));
  OD_CUDA(cudaMallocHost(&l->err_host, sizeof(int)));
  s->device_bytes += (long long)sizeof(double) * l->nvals + (long long)(sizeof(int) * 4 + sizeof(double) * 2) * n;
  // co-resident CTAs for the cooperative apply (both instantiations share
  // the launch bounds; the smaller occupancy is used)
  int dev_coop = 0, per0 = 0, per1 = 0;
  OD_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, s->ctx->device));
  OD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, sweep_apply_kernel<0>, kSweepThreads, 0));
  OD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, sweep_apply_kernel<1>, kSweepThreads, 0));
  const int per_sm = std::min(per0, per1);
  if (!dev_coop || per_sm < 1) {
    set_error("the triangular-sweep apply needs cooperative launch");
    return OD_ERR_UNSUPPORTED;
  }
  // two CTAs (16 warps) per SM: each level's rows spread over 4864 warps;
  // more warps only add polling traffic
  int per = 2;
  if (const char* e = std::getenv("OD_GB300_SWEEP_CTAS_PER_SM")) per = std::max(1, std::atoi(e));
  const int want = (n + (kSweepThreads / 32) - 1) / (kSweepThreads / 32);   // one warp per row at most
  l->grid = std::max(1, std::min(std::min(per, per_sm) * s->ctx->num_sms, want));
  return OD_OK;
}

// A on the host in the reference's lower layout: given, or rebuilt from
// the last expansion on the device
od_status lower_values(Scene* s, SweepSys* l, const double* host_values, const double** out) {
  if (host_values) {
    *out = host_values;
    return OD_OK;
  }
  if (!s->lo.v1) {
    set_error("preconditioner factor: no system matrix has been formed");
    return OD_ERR_INTERNAL;
  }
  cudaStream_t strm = s->ctx->stream;
  if (l->nvals > 0) {
    OD_KL(s);
    combine_lower_kernel<<<(l->nvals + 255) / 256, 256, 0, strm>>>(l->nvals, s->lo.v1, s->lo.c1, s->lo.v2, s->lo.c2,
                                                                   s->lo.v3, s->lo.c3, l->lo_dev);
    OD_CUDA(cudaGetLastError());
    OD_CUDA(cudaMemcpyAsync(l->lo_host, l->lo_dev, sizeof(double) * l->nvals, cudaMemcpyDeviceToHost, strm));
  }
  OD_TRY(sync_stream(s));
  *out = l->lo_host;
  return OD_OK;
}

// upload the staged strictly lower part (h_cp / h_ri / h_bval, by columns)
// and diagonal (h_diag): forward CSR, dependency levels and row lists
od_status upload(Scene* s, SweepSys* l, int kind) {
  const int n = l->n;
  const long long nnz = (long long)l->h_ri.size();
  if (nnz > 0x7fffffffLL) {
    set_error("preconditioner factor exceeds 2^31 entries");
    return OD_ERR_OUT_OF_MEMORY;
  }
  // forward CSR (columns ascending in every row) by a counting transpose
  l->h_rp.assign(n + 1, 0);
  for (long long q = 0; q < nnz; q++) l->h_rp[l->h_ri[q] + 1]++;
  for (int i = 0; i < n; i++) l->h_rp[i + 1] += l->h_rp[i];
  l->h_ci.resize(nnz);
  l->h_fval.resize(nnz);
  {
    std::vector<int> fill(l->h_rp.begin(), l->h_rp.end() - 1);
    for (int c = 0; c < n; c++)
      for (int q = l->h_cp[c]; q < l->h_cp[c + 1]; q++) {
        const int at = fill[l->h_ri[q]]++;
        l->h_ci[at] = c;
        l->h_fval[at] = l->h_bval[q];
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
    for (int i = n - 1; i >= 0; i--) {
      int m = 0;
      for (int q = l->h_cp[i]; q < l->h_cp[i + 1]; q++) m = std::max(m, lev[l->h_ri[q]] + 1);
      lev[i] = m;
      db = std::max(db, m + 1);
    }
    list_by_level(db, false, l->h_ob);
    l->depth_f = df;
    l->depth_b = db;
  }
  cudaStream_t strm = s->ctx->stream;
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
    OD_CUDA(cudaMemcpyAsync(l->diag, l->h_diag.data(), sizeof(double) * n, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->ord_f, l->h_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->ord_b, l->h_ob.data(), sizeof(int) * n, cudaMemcpyHostToDevice, strm));
  }
  if (nnz > 0) {
    OD_CUDA(cudaMemcpyAsync(l->f_ci, l->h_ci.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->f_val, l->h_fval.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->b_ri, l->h_ri.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->b_val, l->h_bval.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, strm));
  }
  // the staging vectors are read by the copies: finish them before returning
  OD_TRY(sync_stream(s));
  l->kind = kind;
  l->nnz = nnz;
  Ctx* ctx = s->ctx;
  ctx->sweep_factors++;
  ctx->sweep_nnz = nnz;
  ctx->sweep_levels = (long long)l->depth_f + l->depth_b;
  return OD_OK;
}

}  // namespace

void sweep_free(SweepSys* l) {
  if (!l) return;
  for (double* p : {l->lo_dev, l->f_val, l->b_val, l->diag, l->y}) cudaFree(p);
  for (int* p : {l->f_rp, l->f_ci, l->b_cp, l->b_ri, l->ord_f, l->ord_b, l->err}) cudaFree(p);
  if (l->lo_host) cudaFreeHost(l->lo_host);
  if (l->err_host) cudaFreeHost(l->err_host);
  delete l;
}

od_status ldlt_factor(Scene* s, const double* host_values, double sainv_eps, double ldlt_eps) {
  OD_TRY(sweep_alloc(s));
  SweepSys* l = s->pcg.sweep;
  const auto t0 = std::chrono::steady_clock::now();
  const double* vals = nullptr;
  OD_TRY(lower_values(s, l, host_values, &vals));
  if (l->rif_cols.n != l->n || l->rif_cols.ptr.empty()) rif_columns(l->n, s->nbc, s->hpcol, s->hrows, l->rif_cols);
  rif_factor(l->rif_cols, vals, sainv_eps, ldlt_eps, l->rif);
  const RifFactor& F = l->rif;
  const int n = l->n;
  // strictly lower by columns: the reference's storage (pcol n entries) closed by nnz
  l->h_cp.assign(F.pcol.begin(), F.pcol.end());
  l->h_cp.resize(n + 1, (int)F.val.size());
  l->h_ri.assign(F.row.begin(), F.row.end());
  l->h_bval.assign(F.val.begin(), F.val.end());
  l->h_diag.assign(F.dinv.begin(), F.dinv.end());
  OD_TRY(upload(s, l, OD_PRECOND_LDLT));
  s->ctx->sweep_factor_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return OD_OK;
}

od_status ic_factor(Scene* s, const double* host_values, double eps, double relax) {
  OD_TRY(sweep_alloc(s));
  SweepSys* l = s->pcg.sweep;
  const auto t0 = std::chrono::steady_clock::now();
  const double* vals = nullptr;
  OD_TRY(lower_values(s, l, host_values, &vals));
  if (l->ric_cols.n != l->n || l->ric_cols.ptr.empty())
    ric_columns(l->n, s->nbc, s->hpcol, s->hrows, s->horis, l->ric_cols);
  ric_factor(l->ric_cols, vals, eps, relax, l->ric);
  const RicFactor& F = l->ric;
  const int n = l->n;
  // split every column into its diagonal (first) and the rows below it
  l->h_cp.assign(n + 1, 0);
  l->h_ri.clear();
  l->h_bval.clear();
  l->h_diag.assign(n, 0.0);
  for (int c = 0; c < n; c++) {
    l->h_diag[c] = F.val[F.pcol[c]];
    for (int q = F.pcol[c] + 1; q < F.pcol[c + 1]; q++) {
      l->h_ri.push_back(F.row[q]);
      l->h_bval.push_back(F.val[q]);
    }
    l->h_cp[c + 1] = (int)l->h_ri.size();
  }
  OD_TRY(upload(s, l, OD_PRECOND_IC));
  s->ctx->sweep_factor_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return OD_OK;
}

od_status sweep_apply(Scene* s, const double* r, double* z, const SolveScalars* sc) {
  SweepSys* l = s->pcg.sweep;
  if (!l || l->kind < 0) {
    set_error("triangular-sweep apply without a factor");
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
  const double* dg = l->diag;
  double* y = l->y;
  int* err = l->err;
  void* args[] = {(void*)&n,   (void*)&n_pad, (void*)&frp, (void*)&fci, (void*)&fval, (void*)&bcp,
                  (void*)&bri, (void*)&bval,  (void*)&of,  (void*)&ob,  (void*)&dg,   (void*)&r,
                  (void*)&y,   (void*)&z,     (void*)&err, (void*)&sc};
  // every value starts "not yet written" (all-ones bytes)
  if (n > 0) {
    OD_CUDA(cudaMemsetAsync(y, 0xff, sizeof(double) * (size_t)n, strm));
    OD_CUDA(cudaMemsetAsync(z, 0xff, sizeof(double) * (size_t)n, strm));
  }
  OD_KL(s);
  void* fn = l->kind == OD_PRECOND_IC ? (void*)sweep_apply_kernel<1> : (void*)sweep_apply_kernel<0>;
  OD_CUDA(cudaLaunchCooperativeKernel(fn, dim3(l->grid), dim3(kSweepThreads), args, 0, strm));
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
      ctx->sweep_applies++;
      ctx->sweep_apply_ms += ms;
      ctx->sweep_apply_bytes += 2.0 * 12.0 * (double)l->nnz + 56.0 * n;
    }
  }
  return OD_OK;
}

od_status sweep_check(Scene* s) {
  SweepSys* l = s->pcg.sweep;
  if (!l) return OD_OK;
  cudaStream_t strm = s->ctx->stream;
  OD_CUDA(cudaMemcpyAsync(l->err_host, l->err, sizeof(int), cudaMemcpyDeviceToHost, strm));
  OD_TRY(sync_stream(s));
  if (*l->err_host) {
    OD_CUDA(cudaMemsetAsync(l->err, 0, sizeof(int), strm));
    set_error("triangular sweep: a bounded wait on a row value ran out");
    return OD_ERR_DEVICE_TIMEOUT;
  }
  return OD_OK;
}

}  // namespace od

// ------------------------------------------------------------------ C ABI
using namespace od;

namespace {

od_status apply_host(od_scene* scene, int kind, const double* rhs, double* result, const char* what) {
  Scene* s = &scene->s;
  SweepSys* l = s->pcg.sweep;
  if (!l || l->kind != kind) {
    set_error(what);
    return OD_ERR_INVALID_ARG;
  }
  OD_CUDA(cudaSetDevice(s->ctx->device));
  Pcg& P = s->pcg;
  cudaStream_t strm = s->ctx->stream;
  OD_CUDA(cudaMemsetAsync(P.r, 0, sizeof(double) * P.n_pad, strm));
  if (s->dofs > 0) OD_CUDA(cudaMemcpyAsync(P.r, rhs, sizeof(double) * s->dofs, cudaMemcpyHostToDevice, strm));
  OD_TRY(sweep_apply(s, P.r, P.z, nullptr));
  if (s->dofs > 0) OD_CUDA(cudaMemcpyAsync(result, P.z, sizeof(double) * s->dofs, cudaMemcpyDeviceToHost, strm));
  OD_TRY(sync_stream(s));
  return sweep_check(s);
}

}  // namespace

extern "C" od_status od_scene_ldlt_factor(od_scene* scene, const double* values, double sainv_eps, double ldlt_eps,
                                          long long* nnz) {
  OD_CHECK_ARG(scene && values, "od_scene_ldlt_factor: NULL argument");
  OD_CHECK_ARG(sainv_eps >= 0.0 && ldlt_eps >= 0.0 && std::isfinite(sainv_eps) && std::isfinite(ldlt_eps),
               "od_scene_ldlt_factor: drop bounds must be finite and >= 0");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_TRY(ldlt_factor(s, values, sainv_eps, ldlt_eps));
  if (nnz) *nnz = (long long)s->pcg.sweep->rif.val.size();
  return OD_OK;
}

extern "C" od_status od_scene_ldlt_get(od_scene* scene, double* values, int* rows, int* pcol, double* inv_diag) {
  OD_CHECK_ARG(scene, "od_scene_ldlt_get: scene is NULL");
  SweepSys* l = scene->s.pcg.sweep;
  OD_CHECK_ARG(l && l->kind == OD_PRECOND_LDLT, "od_scene_ldlt_get: no LDL^T factor (call od_scene_ldlt_factor)");
  const RifFactor& F = l->rif;
  if (values && !F.val.empty()) std::copy(F.val.begin(), F.val.end(), values);
  if (rows && !F.row.empty()) std::copy(F.row.begin(), F.row.end(), rows);
  if (pcol && !F.pcol.empty()) std::copy(F.pcol.begin(), F.pcol.end(), pcol);
  if (inv_diag && !F.dinv.empty()) std::copy(F.dinv.begin(), F.dinv.end(), inv_diag);
  return OD_OK;
}

extern "C" od_status od_scene_ldlt_apply(od_scene* scene, const double* rhs, double* result) {
  OD_CHECK_ARG(scene && rhs && result, "od_scene_ldlt_apply: NULL argument");
  return apply_host(scene, OD_PRECOND_LDLT, rhs, result, "od_scene_ldlt_apply: no LDL^T factor loaded");
}

extern "C" od_status od_scene_ic_factor(od_scene* scene, const double* values, double eps, double relax,
                                        long long* nnz) {
  OD_CHECK_ARG(scene && values, "od_scene_ic_factor: NULL argument");
  OD_CHECK_ARG(eps >= 0.0 && relax >= 0.0 && std::isfinite(eps) && std::isfinite(relax),
               "od_scene_ic_factor: epsilon and relaxedScale must be finite and >= 0");
  Scene* s = &scene->s;
  OD_CHECK_ARG(s->dofs >= 2, "od_scene_ic_factor: needs at least 2 DOFs");
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_TRY(ic_factor(s, values, eps, relax));
  if (nnz) *nnz = (long long)s->pcg.sweep->ric.val.size();
  return OD_OK;
}

extern "C" od_status od_scene_ic_get(od_scene* scene, double* values, int* rows, int* pcol) {
  OD_CHECK_ARG(scene, "od_scene_ic_get: scene is NULL");
  SweepSys* l = scene->s.pcg.sweep;
  OD_CHECK_ARG(l && l->kind == OD_PRECOND_IC, "od_scene_ic_get: no incomplete Cholesky factor (call od_scene_ic_factor)");
  const RicFactor& F = l->ric;
  if (values && !F.val.empty()) std::copy(F.val.begin(), F.val.end(), values);
  if (rows && !F.row.empty()) std::copy(F.row.begin(), F.row.end(), rows);
  if (pcol && !F.pcol.empty()) std::copy(F.pcol.begin(), F.pcol.end(), pcol);
  return OD_OK;
}

extern "C" od_status od_scene_ic_apply(od_scene* scene, const double* rhs, double* result) {
  OD_CHECK_ARG(scene && rhs && result, "od_scene_ic_apply: NULL argument");
  return apply_host(scene, OD_PRECOND_IC, rhs, result, "od_scene_ic_apply: no incomplete Cholesky factor loaded");
}
