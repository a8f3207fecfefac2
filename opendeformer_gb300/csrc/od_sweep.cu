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
// and applied by one cooperative launch per apply.  Rows go in triples
// [3g, 3g + 3) (a node's three DOFs, which depend on one another in a
// chain, when they are numbered consecutively); triples are listed by
// dependency level (level of a triple = 1 + the highest level of the
// triples it reads outside itself; forward and backward levels apart), and
// warp w of the W co-resident warps takes entries w, w+W, ... of the
// forward list, then of the backward list.  y and z are filled with an
// all-ones NaN before the launch (a pattern no arithmetic result has); a
// warp waits (bounded) until the values it reads outside its triple are no
// longer that pattern, read with acquire loads, resolves the triple's own
// chain in registers and publishes each value with one release store: the
// value is its own ready flag.  Progress: the first unfinished entry of a
// list is at the head of its warp's queue and reads only triples of lower
// levels, listed before it and so finished; every warp finishes its forward
// entries before its first backward wait.  Taking triples rather than rows
// cuts the dependency chain (and the apply time) about three-fold on
// meshes whose node DOFs are consecutive.
//
// Dependent FP64 operations cost 64 cycles each on this part (a shuffle
// plus an add about 108), so the products are summed by fixed 5-level
// butterflies over the warp (three interleaved, one per row of the triple)
// rather than one after another: the result is deterministic and within
// rounding of the reference's sequential sums.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "od_grid.cuh"
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
  int *ord_f = nullptr, *ord_b = nullptr;   // row triples by forward / backward level
  double *f_val = nullptr, *b_val = nullptr, *y = nullptr;
  double* diag = nullptr;            // D^-1 (LDL^T) or 1 / L_ii (IC)
  int *err = nullptr, *err_host = nullptr;
  int grid = 0;                      // co-resident CTAs of the apply
  int depth_f = 0, depth_b = 0;      // dependency levels of the two sweeps (row triples)
  // host staging of the sweep arrays
  std::vector<int> h_rp, h_ci, h_cp, h_ri, h_of, h_ob;
  std::vector<double> h_fval, h_bval, h_diag;
};

namespace {

constexpr int kSweepThreads = 256;
constexpr unsigned kSweepSpinLimit = 1u << 21;

// bounded wait until v (first read of *p) is written; after a timeout
// anywhere (err set) no thread waits any more, so the launch ends promptly
// and the host reports it
template <class T>
__device__ __forceinline__ T finish_wait(typename SweepFlag<T>::U v, const T* p, int* err) {
  using F = SweepFlag<T>;
  for (unsigned k = 1; v == F::kPend; k++) {
    if (k >= kSweepSpinLimit) {
      atomicOr(err, 1);
      return T(0);
    }
    if ((k & 1023u) == 0 && *(volatile int*)err) return T(0);
    v = F::ld(p);
  }
  return F::val(v);
}

constexpr int kSweepBatch = 4;   // entries per lane with their value loads in flight together
constexpr unsigned kSweepPollBurst = 1024;   // polls of one value between checks of the error flag

// Sums, per row k of the triple [i0, i0 + m), of the products of its
// entries [rb0, rb3) (row k owns [rb_k, rb_k+1)) with the values of vec
// outside the triple (forward: index < i0; backward: index >= i0 + m);
// the entries inside the triple go to the warp's slots in[] (L_10, L_20,
// L_21).  Each lane loads kSweepBatch entries, then their values together.
template <bool FWD, class T>
__device__ __forceinline__ void triple_sums(int rb0, int rb1, int rb2, int rb3, int i0, int m,
                                            const int* __restrict__ idx, const T* __restrict__ val,
                                            const T* vec, T* in, int* err, int lane, T& a0,
                                            T& a1, T& a2) {
  using F = SweepFlag<T>;
  using U = typename F::U;
  for (int q0 = rb0; q0 < rb3; q0 += 32 * kSweepBatch) {
    int ix[kSweepBatch], kr[kSweepBatch];
    T lv[kSweepBatch];
    U v[kSweepBatch];
#pragma unroll
    for (int u = 0; u < kSweepBatch; u++) {
      const int q = q0 + u * 32 + lane;
      ix[u] = -1;
      kr[u] = 0;
      lv[u] = T(0);
      if (q < rb3) {
        const int c = idx[q];
        const T l = val[q];
        const int k = q < rb1 ? 0 : (q < rb2 ? 1 : 2);
        if (FWD ? c < i0 : c >= i0 + m) {
          ix[u] = c;
          kr[u] = k;
          lv[u] = l;
        } else {
          in[FWD ? k + (c - i0) - 1 : (c - i0) + k - 1] = l;   // (1,0) -> 0, (2,0) -> 1, (2,1) -> 2
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kSweepBatch; u++) v[u] = ix[u] >= 0 ? F::ld(vec + ix[u]) : U(0);
    // warp-cooperative wait: one lane polls the first value still pending
    // in the warp, then every lane re-reads its pending values once; the
    // values of one level land together, so one or two rounds usually do,
    // and the polls (which queue in front of the stores they wait for)
    // stay one per warp
    for (unsigned round = 1;; round++) {
      int pu = -1;
#pragma unroll
      for (int u = kSweepBatch - 1; u >= 0; u--)
        if (ix[u] >= 0 && v[u] == F::kPend) pu = u;
      const unsigned ball = __ballot_sync(0xffffffffu, pu >= 0);
      if (!ball) break;
      int stop = 0;
      if (lane == __ffs(ball) - 1) {
        const T* p = vec;
#pragma unroll
        for (int u = 0; u < kSweepBatch; u++)
          if (u == pu) p += ix[u];
        unsigned k = 0;
        while (F::ld(p) == F::kPend && ++k < kSweepPollBurst) {
        }
        stop = round >= kSweepSpinLimit / kSweepPollBurst || *(volatile int*)err;
        if (round >= kSweepSpinLimit / kSweepPollBurst) atomicOr(err, 1);
      }
      if (__any_sync(0xffffffffu, stop)) {
#pragma unroll
        for (int u = 0; u < kSweepBatch; u++)
          if (v[u] == F::kPend) v[u] = U(0);
        break;
      }
#pragma unroll
      for (int u = 0; u < kSweepBatch; u++)
        if (ix[u] >= 0 && v[u] == F::kPend) v[u] = F::ld(vec + ix[u]);
    }
#pragma unroll
    for (int u = 0; u < kSweepBatch; u++) {
      if (ix[u] < 0) continue;
      const T p = lv[u] * F::val(v[u]);
      if (kr[u] == 0) a0 += p;
      else if (kr[u] == 1) a1 += p;
      else a2 += p;
    }
  }
}

// IC = 0: LDL^T (dinv = D^-1), IC = 1: Cholesky (dinv = 1 / L_ii).  Rows go
// in triples [3g, 3g + 3) (a node's three DOFs when those are consecutive):
// a warp sums the products of all three rows with values outside the
// triple (three interleaved butterflies), then lane 0 resolves the chain
// inside the triple in registers and publishes the three values.
template <int IC, class T>
__global__ void __launch_bounds__(kSweepThreads, 2) sweep_apply_kernel(
    int n, int n_pad, int ng, const int* __restrict__ frp, const int* __restrict__ fci,
    const T* __restrict__ fval, const int* __restrict__ bcp, const int* __restrict__ bri,
    const T* __restrict__ bval, const int* __restrict__ ord_f, const int* __restrict__ ord_b,
    const T* __restrict__ dinv, const T* __restrict__ r, T* y, T* z, int* __restrict__ err,
    const SolveScalars* sc, const int* __restrict__ perm, T* __restrict__ zout) {
  using F = SweepFlag<T>;
  __shared__ T inner_s[kSweepThreads / 32][3];
  if (sc && *(volatile const int*)&sc->done) return;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int W = gridDim.x * wpb;
  const int w = blockIdx.x * wpb + (threadIdx.x >> 5);
  T* in = inner_s[threadIdx.x >> 5];
  // padding rows carry the identity
  for (int i = n + blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += gridDim.x * blockDim.x) {
    if (perm) zout[perm[i]] = r[perm[i]];
    else z[i] = r[i];
  }

  // forward: y_j = r_j - sum_c L_jc y_c (times 1 / L_jj for IC)
  for (int t = w; t < ng; t += W) {
    const int g = ord_f[t];
    const int i0 = 3 * g, m = min(3, n - i0);
    const int rb0 = frp[i0], rb1 = frp[i0 + 1], rb2 = frp[i0 + min(2, m)], rb3 = frp[i0 + m];
    T rv[3] = {T(0), T(0), T(0)}, dv[3] = {T(0), T(0), T(0)};
    if (lane == 0)
      for (int k = 0; k < m; k++) {
        rv[k] = r[perm ? perm[i0 + k] : i0 + k];
        dv[k] = IC ? dinv[i0 + k] : T(1);
      }
    __syncwarp();
    if (lane < 3) in[lane] = T(0);
    __syncwarp();
    T a0 = T(0), a1 = T(0), a2 = T(0);
    triple_sums<true, T>(rb0, rb1, rb2, rb3, i0, m, fci, fval, y, in, err, lane, a0, a1, a2);
    for (int o = 16; o; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    __syncwarp();
    if (lane == 0) {
      const T y0 = IC ? (rv[0] - a0) * dv[0] : rv[0] - a0;
      F::st(y + i0, y0);
      if (m > 1) {
        const T s1 = rv[1] - a1 - in[0] * y0;
        const T y1 = IC ? s1 * dv[1] : s1;
        F::st(y + i0 + 1, y1);
        if (m > 2) {
          const T s2 = rv[2] - a2 - in[1] * y0 - in[2] * y1;
          F::st(y + i0 + 2, IC ? s2 * dv[2] : s2);
        }
      }
    }
  }

  // backward: z_i = (y_i - sum_r z_r L_ri) / L_ii (IC), y_i D_ii^-1 - sum_r z_r L_ri (LDL^T)
  for (int t = w; t < ng; t += W) {
    const int g = ord_b[t];
    const int i0 = 3 * g, m = min(3, n - i0);
    const int cb0 = bcp[i0], cb1 = bcp[i0 + 1], cb2 = bcp[i0 + min(2, m)], cb3 = bcp[i0 + m];
    T yv[3] = {T(0), T(0), T(0)}, dv[3] = {T(0), T(0), T(0)};
    if (lane == 0) {
      typename F::U v[3] = {0, 0, 0};
      for (int k = 0; k < m; k++) {
        v[k] = F::ld(y + i0 + k);
        dv[k] = dinv[i0 + k];
      }
      for (int k = 0; k < m; k++) yv[k] = finish_wait<T>(v[k], y + i0 + k, err);
    }
    __syncwarp();
    if (lane < 3) in[lane] = T(0);
    __syncwarp();
    T a0 = T(0), a1 = T(0), a2 = T(0);
    triple_sums<false, T>(cb0, cb1, cb2, cb3, i0, m, bri, bval, z, in, err, lane, a0, a1, a2);
    for (int o = 16; o; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    __syncwarp();
    if (lane == 0) {
      T z2 = T(0), z1 = T(0);
      if (m > 2) {
        z2 = IC ? (yv[2] - a2) * dv[2] : yv[2] * dv[2] - a2;
        F::st(z + i0 + 2, z2);
      }
      if (m > 1) {
        const T e1 = a1 + z2 * in[2];
        z1 = IC ? (yv[1] - e1) * dv[1] : yv[1] * dv[1] - e1;
        F::st(z + i0 + 1, z1);
      }
      const T e0 = a0 + z1 * in[0] + z2 * in[1];
      const T z0 = IC ? (yv[0] - e0) * dv[0] : yv[0] * dv[0] - e0;
      F::st(z + i0, z0);
      if (perm) {  // the caller's order
        zout[perm[i0]] = z0;
        if (m > 1) zout[perm[i0 + 1]] = z1;
        if (m > 2) zout[perm[i0 + 2]] = z2;
      }
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
  return sweep_grid(s, n, &l->grid);
}

}  // namespace

// Dependency levels of row triples [3g, 3g + 3): a triple's forward level is
// 1 + the highest level of the triples its rows read below it (entries
// inside the triple are resolved by the warp that takes it), likewise
// backward through the columns; triples listed by level (a counting sort;
// forward ties by ascending triple, backward by descending).  depth = levels.
void sweep_group_levels(int n, const std::vector<int>& frp, const std::vector<int>& fci, const std::vector<int>& bcp,
                        const std::vector<int>& bri, std::vector<int>& ord_f, std::vector<int>& ord_b, int* depth_f,
                        int* depth_b) {
  const int ng = (n + 2) / 3;
  std::vector<int> lev(ng, 0);
  auto list_by_level = [&](int depth, bool ascending, std::vector<int>& ord) {
    std::vector<int> start(depth + 1, 0);
    for (int g = 0; g < ng; g++) start[lev[g] + 1]++;
    for (int k = 0; k < depth; k++) start[k + 1] += start[k];
    ord.resize(ng);
    for (int t = 0; t < ng; t++) {
      const int g = ascending ? t : ng - 1 - t;
      ord[start[lev[g]]++] = g;
    }
  };
  int df = 0, db = 0;
  for (int g = 0; g < ng; g++) {
    const int i0 = 3 * g, i1 = std::min(n, i0 + 3);
    int m = 0;
    for (int q = frp[i0]; q < frp[i1]; q++)
      if (fci[q] < i0) m = std::max(m, lev[fci[q] / 3] + 1);
    lev[g] = m;
    df = std::max(df, m + 1);
  }
  list_by_level(df, true, ord_f);
  std::fill(lev.begin(), lev.end(), 0);
  for (int g = ng - 1; g >= 0; g--) {
    const int i0 = 3 * g, i1 = std::min(n, i0 + 3);
    int m = 0;
    for (int q = bcp[i0]; q < bcp[i1]; q++)
      if (bri[q] >= i1) m = std::max(m, lev[bri[q] / 3] + 1);
    lev[g] = m;
    db = std::max(db, m + 1);
  }
  list_by_level(db, false, ord_b);
  *depth_f = ng > 0 ? df : 0;
  *depth_b = ng > 0 ? db : 0;
}

// co-resident CTAs for the cooperative apply of an n-row factor (both
// instantiations share the launch bounds; the smaller occupancy is used)
od_status sweep_grid(Scene* s, int n, int* grid) {
  int dev_coop = 0, per0 = 0, per1 = 0;
  OD_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, s->ctx->device));
  OD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, sweep_apply_kernel<0, double>, kSweepThreads, 0));
  OD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, sweep_apply_kernel<1, double>, kSweepThreads, 0));
  const int per_sm = std::min(per0, per1);
  if (!dev_coop || per_sm < 1) {
    set_error("the triangular-sweep apply needs cooperative launch");
    return OD_ERR_UNSUPPORTED;
  }
  // one CTA (8 warps) per SM: 1,216 warps hold a level's triples (tens of
  // them on the 98k-tet beam) many times over; measured 4% faster than two
  // CTAs per SM and 6% faster than three
  int per = 1;
  if (const char* e = std::getenv("OD_GB300_SWEEP_CTAS_PER_SM")) per = std::max(1, std::atoi(e));
  const int want = ((n + 2) / 3 + (kSweepThreads / 32) - 1) / (kSweepThreads / 32);   // one warp per triple at most
  *grid = std::max(1, std::min(std::min(per, per_sm) * s->ctx->num_sms, want));
  return OD_OK;
}

namespace {

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
// and diagonal (h_diag): forward CSR, dependency levels and row-triple lists
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
  sweep_group_levels(n, l->h_rp, l->h_ci, l->h_cp, l->h_ri, l->h_of, l->h_ob, &l->depth_f, &l->depth_b);
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
    OD_CUDA(cudaMemcpyAsync(l->ord_f, l->h_of.data(), sizeof(int) * l->h_of.size(), cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(l->ord_b, l->h_ob.data(), sizeof(int) * l->h_ob.size(), cudaMemcpyHostToDevice, strm));
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
    l->h_diag[c] = 1.0 / F.val[F.pcol[c]];   // the apply multiplies by 1 / L_cc
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

namespace {
// one warp in the apply's cooperative wait on a value nobody writes: row 0
// of the triple [3, 6) reads column 0, still the pending pattern
__global__ void __launch_bounds__(32) selftest_value_wait_kernel(const int* idx, const double* val,
                                                                 const double* vec, int* err) {
  __shared__ double in[3];
  const int lane = threadIdx.x & 31;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  if (lane < 3) in[lane] = 0.0;
  __syncwarp();
  triple_sums<true>(0, 1, 1, 1, 3, 3, idx, val, vec, in, err, lane, a0, a1, a2);
}
}  // namespace

// Self-test of the triangular sweeps' bounded wait: the wait runs out
// (kSweepSpinLimit polls) and sets the error flag the host reports as
// OD_ERR_DEVICE_TIMEOUT.
od_status selftest_value_wait_timeout(Ctx* c, int* timed_out) {
  *timed_out = 0;
  DeviceTemps tmp;
  int* idx = nullptr;
  int* err = nullptr;
  double *val = nullptr, *vec = nullptr;
  OD_CUDA(tmp.alloc(&idx, sizeof(int)));
  OD_CUDA(tmp.alloc(&err, sizeof(int)));
  OD_CUDA(tmp.alloc(&val, sizeof(double)));
  OD_CUDA(tmp.alloc(&vec, sizeof(double)));
  const int zero = 0;
  const double one = 1.0;
  OD_CUDA(cudaMemcpyAsync(idx, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  OD_CUDA(cudaMemcpyAsync(val, &one, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  OD_CUDA(cudaMemsetAsync(vec, 0xff, sizeof(double), c->stream));
  OD_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
  selftest_value_wait_kernel<<<1, 32, 0, c->stream>>>(idx, val, vec, err);
  cudaError_t e = cudaGetLastError();
  int he = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&he, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "value-wait self-test");
  *timed_out = he == 1;
  return OD_OK;
}

// Level-synchronous IC sweeps for a factor in colour order (IC(0) of a
// large mesh): colour c is the contiguous triple range [cs[c], cs[c+1]) and
// reads only earlier colours (forward) or later ones (backward), so one
// launch per colour and direction, one thread per triple, needs no waits.
// This serves colours far larger than the one-launch sweep's warp count,
// where that kernel would take many triples per warp one after another.
template <class T>
__global__ void ic_level_fwd_kernel(int g0, int g1, int n, const int* __restrict__ frp, const int* __restrict__ fci,
                                    const T* __restrict__ fval, const T* __restrict__ dinv,
                                    const int* __restrict__ perm, const T* __restrict__ r, T* __restrict__ y,
                                    const SolveScalars* __restrict__ sc) {
  if (sc && *(volatile const int*)&sc->done) return;
  const int g = g0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= g1) return;
  for (int k = 0; k < 3; k++) {
    const int i = 3 * g + k;
    if (i >= n) break;
    T acc = r[perm ? perm[i] : i];
    for (int q = frp[i]; q < frp[i + 1]; q++) acc -= fval[q] * y[fci[q]];   // earlier colours, then the triple
    y[i] = acc * dinv[i];
  }
}

template <class T>
__global__ void ic_level_bwd_kernel(int g0, int g1, int n, const int* __restrict__ bcp, const int* __restrict__ bri,
                                    const T* __restrict__ bval, const T* __restrict__ dinv,
                                    const int* __restrict__ perm, const T* __restrict__ y, T* __restrict__ z,
                                    T* __restrict__ zout, const SolveScalars* __restrict__ sc) {
  if (sc && *(volatile const int*)&sc->done) return;
  const int g = g0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= g1) return;
  for (int k = 2; k >= 0; k--) {
    const int i = 3 * g + k;
    if (i >= n) continue;
    T acc = y[i];
    for (int q = bcp[i]; q < bcp[i + 1]; q++) acc -= bval[q] * z[bri[q]];   // the triple, then later colours
    acc *= dinv[i];
    z[i] = acc;
    if (perm) zout[perm[i]] = acc;
  }
}

template <class T>
static od_status ic_levels_launch(Scene* s, const SweepView& v, const T* fval, const T* bval, const T* diag,
                                  const T* r, T* y, T* z, T* zperm, const SolveScalars* sc) {
  cudaStream_t strm = s->ctx->stream;
  const std::vector<int>& cs = *v.colour_start;
  T* zin = v.perm ? zperm : z;   // z in the factor's order
  const int nc = (int)cs.size() - 1;
  for (int c = 0; c < nc; c++) {
    const int g0 = cs[c], g1 = cs[c + 1];
    if (g1 <= g0) continue;
    OD_KL(s);
    ic_level_fwd_kernel<T><<<(g1 - g0 + 255) / 256, 256, 0, strm>>>(g0, g1, v.n, v.frp, v.fci, fval, diag, v.perm, r,
                                                                     y, sc);
  }
  for (int c = nc - 1; c >= 0; c--) {
    const int g0 = cs[c], g1 = cs[c + 1];
    if (g1 <= g0) continue;
    OD_KL(s);
    ic_level_bwd_kernel<T><<<(g1 - g0 + 255) / 256, 256, 0, strm>>>(g0, g1, v.n, v.bcp, v.bri, bval, diag, v.perm, y,
                                                                     zin, z, sc);
  }
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

// The IC sweeps on FP32 copies of the factor (the mixed-precision IC(0)
// inner solve): same index arrays and dependency lists as v, FP32 values and
// vectors, FP32 arithmetic.
od_status sweep_launch_f32(Scene* s, const SweepView& v, const float* fval, const float* bval, const float* diag,
                           const float* r, float* y, float* z, float* zperm, const SolveScalars* sc) {
  if (v.colour_start) return ic_levels_launch<float>(s, v, fval, bval, diag, r, y, z, zperm, sc);
  Ctx* ctx = s->ctx;
  cudaStream_t strm = ctx->stream;
  int n = v.n, n_pad = v.n_pad, ng = (v.n + 2) / 3;
  const int* frp = v.frp;
  const int* fci = v.fci;
  const int* bcp = v.bcp;
  const int* bri = v.bri;
  const int* of = v.ord_f;
  const int* ob = v.ord_b;
  int* err = v.err;
  const int* perm = v.perm;
  float* zflag = perm ? zperm : z;
  float* zout = z;
  void* args[] = {(void*)&n,    (void*)&n_pad, (void*)&ng,   (void*)&frp, (void*)&fci, (void*)&fval,
                  (void*)&bcp,  (void*)&bri,   (void*)&bval, (void*)&of,  (void*)&ob,  (void*)&diag,
                  (void*)&r,    (void*)&y,     (void*)&zflag, (void*)&err, (void*)&sc, (void*)&perm,
                  (void*)&zout};
  if (n > 0) {
    OD_CUDA(cudaMemsetAsync(y, 0xff, sizeof(float) * (size_t)n, strm));
    OD_CUDA(cudaMemsetAsync(zflag, 0xff, sizeof(float) * (size_t)n, strm));
  }
  OD_KL(s);
  OD_CUDA(cudaLaunchCooperativeKernel((void*)sweep_apply_kernel<1, float>, dim3(v.grid), dim3(kSweepThreads), args, 0,
                                      strm));
  return OD_OK;
}

od_status sweep_launch(Scene* s, const SweepView& v, const double* r, double* z, const SolveScalars* sc) {
  if (v.colour_start) {
    const bool prof = s->ctx->profiling && s->ctx->ev_pool.size() >= 2;
    if (prof) OD_CUDA(cudaEventRecord(s->ctx->ev_pool[s->ctx->ev_pool.size() - 2], s->ctx->stream));
    OD_TRY(ic_levels_launch<double>(s, v, v.fval, v.bval, v.diag, r, v.y, z, v.zperm, sc));
    if (prof) {
      Ctx* ctx = s->ctx;
      OD_CUDA(cudaEventRecord(ctx->ev_pool[ctx->ev_pool.size() - 1], ctx->stream));
      OD_CUDA(cudaEventSynchronize(ctx->ev_pool[ctx->ev_pool.size() - 1]));
      float ms = 0.f;
      OD_CUDA(cudaEventElapsedTime(&ms, ctx->ev_pool[ctx->ev_pool.size() - 2], ctx->ev_pool[ctx->ev_pool.size() - 1]));
      bool ran = true;
      if (sc) {
        SolveScalars h;
        OD_CUDA(cudaMemcpy(&h, sc, sizeof(SolveScalars), cudaMemcpyDeviceToHost));
        ran = !h.done;
      }
      if (ran) {
        ctx->sweep_applies++;
        ctx->sweep_apply_ms += ms;
        ctx->sweep_apply_bytes += 2.0 * 12.0 * (double)v.nnz + 56.0 * v.n;
      }
    }
    return OD_OK;
  }
  Ctx* ctx = s->ctx;
  cudaStream_t strm = ctx->stream;
  int n = v.n, n_pad = v.n_pad, ng = (v.n + 2) / 3;
  const bool prof = ctx->profiling && ctx->ev_pool.size() >= 2;
  if (prof) OD_CUDA(cudaEventRecord(ctx->ev_pool[ctx->ev_pool.size() - 2], strm));
  const int* frp = v.frp;
  const int* fci = v.fci;
  const double* fval = v.fval;
  const int* bcp = v.bcp;
  const int* bri = v.bri;
  const double* bval = v.bval;
  const int* of = v.ord_f;
  const int* ob = v.ord_b;
  const double* dg = v.diag;
  double* y = v.y;
  int* err = v.err;
  const int* perm = v.perm;
  double* zflag = perm ? v.zperm : z;   // z in the factor's order: the values other rows wait on
  double* zout = z;
  void* args[] = {(void*)&n,    (void*)&n_pad, (void*)&ng,   (void*)&frp, (void*)&fci, (void*)&fval,
                  (void*)&bcp,  (void*)&bri,   (void*)&bval, (void*)&of,  (void*)&ob,  (void*)&dg,
                  (void*)&r,    (void*)&y,     (void*)&zflag, (void*)&err, (void*)&sc, (void*)&perm,
                  (void*)&zout};
  // every value starts "not yet written" (all-ones bytes)
  if (n > 0) {
    OD_CUDA(cudaMemsetAsync(y, 0xff, sizeof(double) * (size_t)n, strm));
    OD_CUDA(cudaMemsetAsync(zflag, 0xff, sizeof(double) * (size_t)n, strm));
  }
  OD_KL(s);
  void* fn = v.ic ? (void*)sweep_apply_kernel<1, double> : (void*)sweep_apply_kernel<0, double>;
  OD_CUDA(cudaLaunchCooperativeKernel(fn, dim3(v.grid), dim3(kSweepThreads), args, 0, strm));
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
      ctx->sweep_apply_bytes += 2.0 * 12.0 * (double)v.nnz + 56.0 * n;
    }
  }
  return OD_OK;
}

od_status sweep_apply(Scene* s, const double* r, double* z, const SolveScalars* sc) {
  SweepSys* l = s->pcg.sweep;
  if (!l || l->kind < 0) {
    set_error("triangular-sweep apply without a factor");
    return OD_ERR_INTERNAL;
  }
  SweepView v;
  v.n = l->n;
  v.n_pad = l->n_pad;
  v.ic = l->kind == OD_PRECOND_IC ? 1 : 0;
  v.grid = l->grid;
  v.nnz = l->nnz;
  v.frp = l->f_rp;
  v.fci = l->f_ci;
  v.fval = l->f_val;
  v.bcp = l->b_cp;
  v.bri = l->b_ri;
  v.bval = l->b_val;
  v.ord_f = l->ord_f;
  v.ord_b = l->ord_b;
  v.diag = l->diag;
  v.y = l->y;
  v.err = l->err;
  return sweep_launch(s, v, r, z, sc);
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
