// Sparse linear algebra of the step: system-matrix combination fused with
// the lower->full BSR expansion, SpMV on the full BSR (the PCG hot kernel),
// SpMV straight from the reference lower layout (residuals), and the
// preconditioned CG of solver/cgSolver.cpp:13-57 as three fused kernels per
// iteration:
//   K1  q = A p, block partials of p.q; the last CTA forms alpha = rz / pq
//   K2  x += alpha p, r -= alpha q, z = M^-1 r, partials of r.z and r.r;
//       the last CTA forms beta, the iteration count and the stop flag
//   K3  p = z + beta p
// Reductions are deterministic: every CTA writes its partial, the last CTA
// to finish (atomic ticket, no spinning) sums them in index order.  All
// kernels of an iteration return at once when the stop flag is set, so a
// batch of iterations can be queued (or captured) without host round trips.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "od_internal.h"

namespace od {

constexpr int kRowLanes = 16;     // lanes per block row in the SpMV kernels
constexpr int kThreads = 256;

__constant__ int c_di3[3] = {0, 3, 5};

__device__ __forceinline__ int lower_src(int kind, int off, int r, int c, const int* __restrict__ gen) {
  switch (kind) {
    case BK_LOWER: return off + c * 3 + r;
    case BK_UPPER: return off + r * 3 + c;
    case BK_DIAG: return r >= c ? off + r - c + c_di3[c] : off + c - r + c_di3[r];
    default: return gen[off * 9 + r * 3 + c];
  }
}

// deterministic block-wide sum (fixed shuffle tree, then fixed warp order)
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// true in every thread of the last CTA to arrive; partials written before
// the call are then visible to it
__device__ __forceinline__ bool last_block(unsigned int* counter) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  return is_last;
}

// sum of partial[j*stride + slot] over j < n, in index order per thread, then
// the fixed tree
__device__ __forceinline__ double reduce_partials(const double* partial, int n, int stride, int slot) {
  double acc = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) acc += __ldcg(partial + (size_t)j * stride + slot);
  return block_sum(acc);
}

// ------------------------------------------------------------- expansion
// A_full = c1 V1 + c2 V2 + c3 V3 for every full-BSR entry, V* in the
// reference lower layout (BlockedSymSparseMatrix Scale/Add,
// core/sparseMatrix.h:281-295, fused with the transpose expansion)
template <class TA>
__global__ void expand_kernel(long long total, const int* __restrict__ kind, const int* __restrict__ off,
                              const int* __restrict__ gen, const double* __restrict__ v1, double c1,
                              const double* __restrict__ v2, double c2, const double* __restrict__ v3, double c3,
                              TA* __restrict__ A) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  int k = (int)(idx / 9), e = (int)(idx - 9LL * k);
  int src = lower_src(kind[k], off[k], e / 3, e % 3, gen);
  double val;
  if (src >= 0) {
    val = c1 * v1[src];
    if (v2) val += c2 * v2[src];
    if (v3) val += c3 * v3[src];
  } else {
    val = src == -2 ? 1.0 : 0.0;
  }
  A[idx] = (TA)val;
}

// y (+)= c1 V1 x1 + c2 V2 x2 + c3 V3 x3 with V* read from the lower layout
// through the full-BSR descriptors (SpMDV semantics, numerMethod.h:134-262)
__global__ void spmv_lower_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                  const int* __restrict__ kind, const int* __restrict__ off,
                                  const int* __restrict__ gen, const double* __restrict__ v1, double c1,
                                  const double* __restrict__ x1, const double* __restrict__ v2, double c2,
                                  const double* __restrict__ x2, const double* __restrict__ v3, double c3,
                                  const double* __restrict__ x3, double* __restrict__ y, int accumulate) {
  const int lane = threadIdx.x & (kRowLanes - 1);
  const int row = blockIdx.x * (blockDim.x / kRowLanes) + threadIdx.x / kRowLanes;
  double y0 = 0.0, y1 = 0.0, y2 = 0.0;
  if (row < nb) {
    for (int k = rp[row] + lane; k < rp[row + 1]; k += kRowLanes) {
      const int cb = col[k], kd = kind[k], of = off[k];
#pragma unroll
      for (int r = 0; r < 3; r++) {
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          int src = lower_src(kd, of, r, c, gen);
          double a1 = 0.0, a2 = 0.0, a3 = 0.0;
          if (src >= 0) {
            a1 = c1 * v1[src];
            if (v2) a2 = c2 * v2[src];
            if (v3) a3 = c3 * v3[src];
          } else if (src == -2) {
            a1 = c1;
          }
          acc += a1 * x1[3 * cb + c];
          if (v2) acc += a2 * x2[3 * cb + c];
          if (v3) acc += a3 * x3[3 * cb + c];
        }
        if (r == 0) y0 += acc; else if (r == 1) y1 += acc; else y2 += acc;
      }
    }
  }
#pragma unroll
  for (int o = kRowLanes / 2; o > 0; o >>= 1) {
    y0 += __shfl_down_sync(0xffffffffu, y0, o, kRowLanes);
    y1 += __shfl_down_sync(0xffffffffu, y1, o, kRowLanes);
    y2 += __shfl_down_sync(0xffffffffu, y2, o, kRowLanes);
  }
  if (lane == 0 && row < nb) {
    if (accumulate) { y[3 * row] += y0; y[3 * row + 1] += y1; y[3 * row + 2] += y2; }
    else { y[3 * row] = y0; y[3 * row + 1] = y1; y[3 * row + 2] = y2; }
  }
}

// row-block product of the full BSR with a 16-lane group per block row
template <class TA>
__device__ __forceinline__ void bsr_row(int row, int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                        const TA* __restrict__ A, const double* __restrict__ x, double& y0,
                                        double& y1, double& y2) {
  const int lane = threadIdx.x & (kRowLanes - 1);
  y0 = y1 = y2 = 0.0;
  if (row < nb) {
    for (int k = rp[row] + lane; k < rp[row + 1]; k += kRowLanes) {
      const TA* a = A + (size_t)k * 9;
      const int c = col[k];
      const double x0 = x[3 * c], x1 = x[3 * c + 1], x2 = x[3 * c + 2];
      y0 += (double)a[0] * x0 + (double)a[1] * x1 + (double)a[2] * x2;
      y1 += (double)a[3] * x0 + (double)a[4] * x1 + (double)a[5] * x2;
      y2 += (double)a[6] * x0 + (double)a[7] * x1 + (double)a[8] * x2;
    }
  }
#pragma unroll
  for (int o = kRowLanes / 2; o > 0; o >>= 1) {
    y0 += __shfl_down_sync(0xffffffffu, y0, o, kRowLanes);
    y1 += __shfl_down_sync(0xffffffffu, y1, o, kRowLanes);
    y2 += __shfl_down_sync(0xffffffffu, y2, o, kRowLanes);
  }
}

template <class TA>
__global__ void spmv_full_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                 const TA* __restrict__ A, const double* __restrict__ x, double* __restrict__ y) {
  const int row = blockIdx.x * (blockDim.x / kRowLanes) + threadIdx.x / kRowLanes;
  double y0, y1, y2;
  bsr_row<TA>(row, nb, rp, col, A, x, y0, y1, y2);
  if ((threadIdx.x & (kRowLanes - 1)) == 0 && row < nb) {
    y[3 * row] = y0; y[3 * row + 1] = y1; y[3 * row + 2] = y2;
  }
}

// ------------------------------------------------------- preconditioners
// Jacobi (JacobiPreconditioner::getInvJacobiMat, jacobiPreconditioner.cpp:16-21)
// or the inverse of every 3x3 diagonal block (adjugate / determinant)
template <class TA>
__global__ void precond_setup_kernel(int nb, int kind, const int* __restrict__ diag_pos, const TA* __restrict__ A,
                                     double* __restrict__ pinv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const TA* a = A + (size_t)diag_pos[i] * 9;
  if (kind == OD_PRECOND_JACOBI) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double v = (double)a[d * 4];
      pinv[3 * i + d] = v > 0.0 ? 1.0 / v : 1.0;
    }
  } else {
    double m[9];
#pragma unroll
    for (int k = 0; k < 9; k++) m[k] = (double)a[k];
    double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
    double inv = 1.0 / det;
    double* o = pinv + 9 * (size_t)i;
    o[0] = (m[4] * m[8] - m[5] * m[7]) * inv;
    o[1] = (m[2] * m[7] - m[1] * m[8]) * inv;
    o[2] = (m[1] * m[5] - m[2] * m[4]) * inv;
    o[3] = (m[5] * m[6] - m[3] * m[8]) * inv;
    o[4] = (m[0] * m[8] - m[2] * m[6]) * inv;
    o[5] = (m[2] * m[3] - m[0] * m[5]) * inv;
    o[6] = (m[3] * m[7] - m[4] * m[6]) * inv;
    o[7] = (m[1] * m[6] - m[0] * m[7]) * inv;
    o[8] = (m[0] * m[4] - m[1] * m[3]) * inv;
  }
}

__device__ __forceinline__ void apply_local_precond(int kind, int i, const double* __restrict__ pinv, const double r[3],
                                                    double z[3]) {
  if (kind == OD_PRECOND_JACOBI) {
    z[0] = pinv[3 * i] * r[0]; z[1] = pinv[3 * i + 1] * r[1]; z[2] = pinv[3 * i + 2] * r[2];
  } else if (kind == OD_PRECOND_BLOCK_JACOBI) {
    const double* m = pinv + 9 * (size_t)i;
    z[0] = m[0] * r[0] + m[1] * r[1] + m[2] * r[2];
    z[1] = m[3] * r[0] + m[4] * r[1] + m[5] * r[2];
    z[2] = m[6] * r[0] + m[7] * r[1] + m[8] * r[2];
  } else {
    z[0] = r[0]; z[1] = r[1]; z[2] = r[2];
  }
}

// ------------------------------------------------------------ PCG kernels
// init: r = b - A x0; z = M^-1 r; p = z; rz = r.z; eps = tol^2 b.b; rr = r.r
// (cgSolver.cpp:20-30).  For IC(0) (local == 0) z and p are formed later.
template <class TA>
__global__ void pcg_init_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                const TA* __restrict__ A, const double* __restrict__ b, const double* __restrict__ x,
                                double* __restrict__ r, double* __restrict__ z, double* __restrict__ p, int pkind,
                                const double* __restrict__ pinv, double tol, int max_iter, double* __restrict__ partial,
                                SolveScalars* sc) {
  const int row = blockIdx.x * (blockDim.x / kRowLanes) + threadIdx.x / kRowLanes;
  double q0, q1, q2;
  bsr_row<TA>(row, nb, rp, col, A, x, q0, q1, q2);
  double rz = 0.0, bb = 0.0, rr = 0.0;
  if ((threadIdx.x & (kRowLanes - 1)) == 0 && row < nb) {
    double rv[3], zv[3];
    const double bv[3] = {b[3 * row], b[3 * row + 1], b[3 * row + 2]};
    rv[0] = bv[0] - q0; rv[1] = bv[1] - q1; rv[2] = bv[2] - q2;
    apply_local_precond(pkind, row, pinv, rv, zv);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      r[3 * row + d] = rv[d];
      if (pkind != OD_PRECOND_IC0) { z[3 * row + d] = zv[d]; p[3 * row + d] = zv[d]; }
      rz += rv[d] * zv[d];
      bb += bv[d] * bv[d];
      rr += rv[d] * rv[d];
    }
  }
  double s0 = block_sum(rz), s1 = block_sum(bb), s2 = block_sum(rr);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = s0; partial[3 * blockIdx.x + 1] = s1; partial[3 * blockIdx.x + 2] = s2;
  }
  if (last_block(&sc->count1)) {
    double t0 = reduce_partials(partial, gridDim.x, 3, 0);
    double t1 = reduce_partials(partial, gridDim.x, 3, 1);
    double t2 = reduce_partials(partial, gridDim.x, 3, 2);
    if (threadIdx.x == 0) {
      sc->rz = t0; sc->bb = t1; sc->rr = t2; sc->rr0 = t2;
      sc->eps = t1 * tol * tol;
      sc->iter = 0;
      sc->max_iter = max_iter;
      sc->status = isfinite(t2) ? OD_OK : OD_ERR_NAN;
      sc->done = !(0 < max_iter && t2 > sc->eps) || !isfinite(t2);
      sc->count1 = 0;
    }
  }
}

// K1: q = A p and alpha = rz / (p.q)
template <class TA>
__global__ void pcg_spmv_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                const TA* __restrict__ A, const double* __restrict__ p, double* __restrict__ q,
                                double* __restrict__ partial, SolveScalars* sc) {
  if (*(volatile int*)&sc->done) return;
  const int row = blockIdx.x * (blockDim.x / kRowLanes) + threadIdx.x / kRowLanes;
  double y0, y1, y2;
  bsr_row<TA>(row, nb, rp, col, A, p, y0, y1, y2);
  double pq = 0.0;
  if ((threadIdx.x & (kRowLanes - 1)) == 0 && row < nb) {
    q[3 * row] = y0; q[3 * row + 1] = y1; q[3 * row + 2] = y2;
    pq = p[3 * row] * y0 + p[3 * row + 1] * y1 + p[3 * row + 2] * y2;
  }
  double s = block_sum(pq);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block(&sc->count1)) {
    double t = reduce_partials(partial, gridDim.x, 1, 0);
    if (threadIdx.x == 0) {
      double alpha = sc->rz / t;
      sc->pq = t;
      sc->alpha = alpha;
      if (!isfinite(alpha)) { sc->status = OD_ERR_NAN; sc->done = 1; }
      sc->count1 = 0;
    }
  }
}

// K2: x += alpha p; r -= alpha q; z = M^-1 r (local preconditioners);
// beta = (r.z)_new / (r.z); stop test of cgSolver.cpp:32
__global__ void pcg_update_kernel(int nb, double* __restrict__ x, double* __restrict__ r, double* __restrict__ z,
                                  const double* __restrict__ p, const double* __restrict__ q, int pkind,
                                  const double* __restrict__ pinv, double* __restrict__ partial, SolveScalars* sc,
                                  int finish) {
  if (*(volatile int*)&sc->done) return;
  const double alpha = sc->alpha;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double rz = 0.0, rr = 0.0;
  if (i < nb) {
    double rv[3], zv[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      x[3 * i + d] += alpha * p[3 * i + d];
      rv[d] = r[3 * i + d] - alpha * q[3 * i + d];
      r[3 * i + d] = rv[d];
    }
    if (pkind != OD_PRECOND_IC0) {
      apply_local_precond(pkind, i, pinv, rv, zv);
#pragma unroll
      for (int d = 0; d < 3; d++) { z[3 * i + d] = zv[d]; rz += rv[d] * zv[d]; }
    }
#pragma unroll
    for (int d = 0; d < 3; d++) rr += rv[d] * rv[d];
  }
  double s0 = block_sum(rz), s1 = block_sum(rr);
  if (threadIdx.x == 0) { partial[2 * blockIdx.x] = s0; partial[2 * blockIdx.x + 1] = s1; }
  if (last_block(&sc->count2)) {
    double t0 = reduce_partials(partial, gridDim.x, 2, 0);
    double t1 = reduce_partials(partial, gridDim.x, 2, 1);
    if (threadIdx.x == 0) {
      sc->rr = t1;
      if (finish) {
        double beta = t0 / sc->rz;
        sc->beta = beta;
        sc->rz = t0;
        sc->iter += 1;
        if (!isfinite(t1) || !isfinite(beta)) { sc->status = OD_ERR_NAN; sc->done = 1; }
        else sc->done = !(sc->iter < sc->max_iter && t1 > sc->eps);
      }
      sc->count2 = 0;
    }
  }
}

// K3: p = z + beta p
__global__ void pcg_direction_kernel(int n, const double* __restrict__ z, double* __restrict__ p, SolveScalars* sc,
                                     int check_done) {
  if (check_done && *(volatile int*)&sc->done) return;
  const double beta = sc->beta;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = beta * p[i] + z[i];
}

// ----------------------------------------------------------------- IC(0)
// Shifted IC(0) of the padded scalar lower pattern (a row-oriented,
// level-scheduled factorisation; no reference counterpart).  Rows of one
// level depend only on rows of earlier levels.
//   L_ij = (A_ij - sum_{k<j} L_ik L_jk) / L_jj
//   L_ii = sqrt((1 + shift) A_ii - sum_{k<i} L_ik^2)
template <class TA>
__global__ void ic0_factor_level(int l0, int l1, const int* __restrict__ rows, const int* __restrict__ rp,
                                 const int* __restrict__ ci, const int* __restrict__ src, const TA* __restrict__ A,
                                 double* __restrict__ L, double shift, int* __restrict__ bad) {
  int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= l1) return;
  const int i = rows[t];
  const int bi = rp[i], ei = rp[i + 1];
  for (int q = bi; q < ei; q++) {
    const int j = ci[q];
    double sum = (double)A[src[q]];
    if (j == i) sum *= (1.0 + shift);
    int a = bi, b = rp[j];
    const int eb = rp[j + 1] - 1;
    while (a < q && b < eb) {
      const int ca = ci[a], cb = ci[b];
      if (ca == cb) { sum -= L[a] * L[b]; a++; b++; }
      else if (ca < cb) a++;
      else b++;
    }
    if (j < i) {
      L[q] = sum / L[rp[j + 1] - 1];
    } else {
      const double d = (double)A[src[q]] * (1.0 + shift);
      if (!(sum > 1e-12 * d)) { *bad = 1; sum = d > 0.0 ? d : 1.0; }
      L[q] = sqrt(sum);
    }
  }
}

// forward sweep L y = r for the rows of one level
__global__ void ic0_forward_level(int l0, int l1, const int* __restrict__ rows, const int* __restrict__ rp,
                                  const int* __restrict__ ci, const double* __restrict__ L, const double* __restrict__ r,
                                  double* __restrict__ y, const SolveScalars* sc) {
  if (sc && *(volatile const int*)&sc->done) return;
  int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= l1) return;
  const int i = rows[t];
  const int e = rp[i + 1] - 1;
  double s = r[i];
  for (int q = rp[i]; q < e; q++) s -= L[q] * y[ci[q]];
  y[i] = s / L[e];
}

// backward sweep L^T z = y through the transposed index (row i lists the
// entries L_ji, j > i)
__global__ void ic0_backward_level(int l0, int l1, const int* __restrict__ rows, const int* __restrict__ trp,
                                   const int* __restrict__ tci, const int* __restrict__ tpos,
                                   const int* __restrict__ rp, const double* __restrict__ L,
                                   const double* __restrict__ y, double* __restrict__ z, const SolveScalars* sc) {
  if (sc && *(volatile const int*)&sc->done) return;
  int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= l1) return;
  const int i = rows[t];
  double s = y[i];
  for (int q = trp[i]; q < trp[i + 1]; q++) s -= L[tpos[q]] * z[tci[q]];
  z[i] = s / L[rp[i + 1] - 1];
}

// r.z partial and finish for IC(0) (K2 split: the update kernel ran with
// finish = 0 and formed r.r)
__global__ void pcg_rz_finish_kernel(int n, const double* __restrict__ r, const double* __restrict__ z,
                                     double* __restrict__ partial, SolveScalars* sc, int init) {
  if (!init && *(volatile int*)&sc->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double rz = i < n ? r[i] * z[i] : 0.0;
  double s = block_sum(rz);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block(&sc->count2)) {
    double t0 = reduce_partials(partial, gridDim.x, 1, 0);
    if (threadIdx.x == 0) {
      if (init) {
        sc->rz = t0;
      } else {
        double beta = t0 / sc->rz;
        sc->beta = beta;
        sc->rz = t0;
        sc->iter += 1;
        if (!isfinite(sc->rr) || !isfinite(beta)) { sc->status = OD_ERR_NAN; sc->done = 1; }
        else sc->done = !(sc->iter < sc->max_iter && sc->rr > sc->eps);
      }
      sc->count2 = 0;
    }
  }
}

__global__ void copy_kernel(int n, const double* __restrict__ a, double* __restrict__ b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

// ------------------------------------------------------------- host side
static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

od_status launch_expand(Scene* s, const double* v1, double c1, const double* v2, double c2, const double* v3,
                        double c3) {
  const long long total = 9LL * s->bsr.nnzb;
  if (total == 0) return OD_OK;
  expand_kernel<double><<<nblk(total, kThreads), kThreads, 0, s->ctx->stream>>>(
      total, s->bsr.desc_kind, s->bsr.desc_off, s->bsr.gen, v1, c1, v2, c2, v3, c3, s->A64);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status launch_spmv_lower(Scene* s, const double* v1, double c1, const double* x1, const double* v2, double c2,
                            const double* x2, const double* v3, double c3, const double* x3, double* y,
                            bool accumulate) {
  const int nb = s->bsr.nb;
  if (nb == 0) return OD_OK;
  const int rows_per_cta = kThreads / kRowLanes;
  spmv_lower_kernel<<<nblk(nb, rows_per_cta), kThreads, 0, s->ctx->stream>>>(
      nb, s->bsr.row_ptr, s->bsr.col, s->bsr.desc_kind, s->bsr.desc_off, s->bsr.gen, v1, c1, x1, v2, c2, x2, v3, c3,
      x3, y, accumulate ? 1 : 0);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status launch_spmv_full(Scene* s, const double* x, double* y) {
  const int nb = s->bsr.nb;
  if (nb == 0) return OD_OK;
  const int rows_per_cta = kThreads / kRowLanes;
  spmv_full_kernel<double><<<nblk(nb, rows_per_cta), kThreads, 0, s->ctx->stream>>>(nb, s->bsr.row_ptr, s->bsr.col,
                                                                                    s->A64, x, y);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

// IC(0) structure: scalar CSR of the padded lower pattern of the full BSR
// (columns sorted, diagonal last), level sets, and the transposed index.
static od_status ic0_build(Scene* s) {
  Pcg& P = s->pcg;
  if (P.ic_rp) return OD_OK;
  // host copies of the BSR structure
  const int nb = s->bsr.nb;
  std::vector<int> rp(nb + 1), col(s->bsr.nnzb);
  OD_CUDA(cudaMemcpy(rp.data(), s->bsr.row_ptr, sizeof(int) * (nb + 1), cudaMemcpyDeviceToHost));
  OD_CUDA(cudaMemcpy(col.data(), s->bsr.col, sizeof(int) * s->bsr.nnzb, cudaMemcpyDeviceToHost));
  const int n = 3 * nb;
  std::vector<int> srp(n + 1, 0), sci, ssrc;
  sci.reserve((size_t)s->bsr.nnzb * 5);
  ssrc.reserve((size_t)s->bsr.nnzb * 5);
  for (int br = 0; br < nb; br++)
    for (int r = 0; r < 3; r++) {
      const int i = 3 * br + r;
      for (int k = rp[br]; k < rp[br + 1]; k++) {
        const int bc = col[k];
        if (bc > br) break;
        for (int c = 0; c < 3; c++) {
          const int j = 3 * bc + c;
          if (j > i) break;
          sci.push_back(j);
          ssrc.push_back(9 * k + 3 * r + c);
        }
      }
      srp[i + 1] = (int)sci.size();
    }
  const int nnz = (int)sci.size();
  // transposed index: for row i the entries (row j > i, column i)
  std::vector<int> trp(n + 1, 0), tci(nnz), tpos(nnz);
  for (int q = 0; q < nnz; q++) trp[sci[q] + 1]++;
  for (int i = 0; i < n; i++) trp[i + 1] += trp[i];
  std::vector<int> fill(trp.begin(), trp.end() - 1);
  for (int j = 0; j < n; j++)
    for (int q = srp[j]; q < srp[j + 1] - 1; q++) {  // off-diagonal entries of row j
      int i = sci[q];
      tci[fill[i]] = j;
      tpos[fill[i]] = q;
      fill[i]++;
    }
  // compact the transposed rows (diagonal slots were counted but not filled)
  std::vector<int> trp2(n + 1, 0), tci2, tpos2;
  tci2.reserve(nnz); tpos2.reserve(nnz);
  for (int i = 0; i < n; i++) {
    for (int q = trp[i]; q < fill[i]; q++) { tci2.push_back(tci[q]); tpos2.push_back(tpos[q]); }
    trp2[i + 1] = (int)tci2.size();
  }
  std::vector<int> lrf, lrb;
  build_ic_levels(srp, sci, n, lrf, P.lvl_ptr_f, true);
  build_ic_levels(srp, sci, n, lrb, P.lvl_ptr_b, false);
  P.ic_n = n;
  P.ic_nnz = nnz;
  P.n_levels_f = (int)P.lvl_ptr_f.size() - 1;
  P.n_levels_b = (int)P.lvl_ptr_b.size() - 1;
  auto up = [&](int** d, const std::vector<int>& h) -> od_status {
    OD_CUDA(cudaMalloc(d, sizeof(int) * std::max<size_t>(1, h.size())));
    if (!h.empty()) OD_CUDA(cudaMemcpy(*d, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice));
    s->device_bytes += (long long)sizeof(int) * h.size();
    return OD_OK;
  };
  od_status st;
  if ((st = up(&P.ic_rp, srp)) != OD_OK) return st;
  if ((st = up(&P.ic_ci, sci)) != OD_OK) return st;
  if ((st = up(&P.ic_src, ssrc)) != OD_OK) return st;
  if ((st = up(&P.lvl_rows_f, lrf)) != OD_OK) return st;
  if ((st = up(&P.lvl_rows_b, lrb)) != OD_OK) return st;
  if ((st = up(&P.icT_rp, trp2)) != OD_OK) return st;
  if ((st = up(&P.icT_ci, tci2)) != OD_OK) return st;
  if ((st = up(&P.icT_pos, tpos2)) != OD_OK) return st;
  OD_CUDA(cudaMalloc(&P.ic_val, sizeof(double) * std::max(1, nnz)));
  OD_CUDA(cudaMalloc(&P.ic_bad, sizeof(int)));
  s->device_bytes += sizeof(double) * (long long)nnz;
  return OD_OK;
}

// shifted IC(0) factorisation of the current A64 with the Manteuffel retry
static od_status ic0_factor(Scene* s) {
  Pcg& P = s->pcg;
  od_status st = ic0_build(s);
  if (st != OD_OK) return st;
  cudaStream_t strm = s->ctx->stream;
  double shift = 0.0;
  for (int attempt = 0; attempt < 40; attempt++) {
    OD_CUDA(cudaMemsetAsync(P.ic_bad, 0, sizeof(int), strm));
    for (int l = 0; l < P.n_levels_f; l++) {
      int l0 = P.lvl_ptr_f[l], l1 = P.lvl_ptr_f[l + 1];
      ic0_factor_level<double><<<nblk(l1 - l0, 128), 128, 0, strm>>>(l0, l1, P.lvl_rows_f, P.ic_rp, P.ic_ci, P.ic_src,
                                                                      s->A64, P.ic_val, shift, P.ic_bad);
    }
    OD_CUDA(cudaGetLastError());
    int bad = 0;
    OD_CUDA(cudaMemcpyAsync(&bad, P.ic_bad, sizeof(int), cudaMemcpyDeviceToHost, strm));
    OD_CUDA(cudaStreamSynchronize(strm));
    if (!bad) break;
    shift = shift == 0.0 ? 1e-3 : 2.0 * shift;
  }
  P.ic_shift = shift;
  return OD_OK;
}

static void ic0_apply(Scene* s, const double* r, double* z, const SolveScalars* sc) {
  Pcg& P = s->pcg;
  cudaStream_t strm = s->ctx->stream;
  for (int l = 0; l < P.n_levels_f; l++) {
    int l0 = P.lvl_ptr_f[l], l1 = P.lvl_ptr_f[l + 1];
    ic0_forward_level<<<nblk(l1 - l0, 128), 128, 0, strm>>>(l0, l1, P.lvl_rows_f, P.ic_rp, P.ic_ci, P.ic_val, r,
                                                            P.q /*y*/, sc);
  }
  for (int l = 0; l < P.n_levels_b; l++) {
    int l0 = P.lvl_ptr_b[l], l1 = P.lvl_ptr_b[l + 1];
    ic0_backward_level<<<nblk(l1 - l0, 128), 128, 0, strm>>>(l0, l1, P.lvl_rows_b, P.icT_rp, P.icT_ci, P.icT_pos,
                                                             P.ic_rp, P.ic_val, P.q, z, sc);
  }
}

od_status pcg_alloc(Scene* s) {
  Pcg& P = s->pcg;
  const int n = 3 * s->bsr.nb;
  P.n_pad = n;
  const int rows_per_cta = kThreads / kRowLanes;
  P.grid = std::max(nblk(s->bsr.nb, rows_per_cta), nblk(n, kThreads));
  size_t nv = std::max(1, n);
  for (double** v : {&P.x, &P.r, &P.z, &P.p, &P.q, &P.b}) {
    OD_CUDA(cudaMalloc(v, sizeof(double) * nv));
    OD_CUDA(cudaMemset(*v, 0, sizeof(double) * nv));
  }
  OD_CUDA(cudaMalloc(&P.partial, sizeof(double) * 3 * (size_t)std::max(1, P.grid)));
  OD_CUDA(cudaMalloc(&P.sc, sizeof(SolveScalars)));
  OD_CUDA(cudaMemset(P.sc, 0, sizeof(SolveScalars)));
  OD_CUDA(cudaMallocHost(&P.sc_host, sizeof(SolveScalars)));
  OD_CUDA(cudaMalloc(&P.pinv, sizeof(double) * 9 * (size_t)std::max(1, s->bsr.nb)));
  s->device_bytes += (long long)sizeof(double) * (6 * nv + 9 * (size_t)s->bsr.nb + 3 * (size_t)P.grid);
  return OD_OK;
}

void pcg_free(Scene* s) {
  Pcg& P = s->pcg;
  for (double* v : {P.x, P.r, P.z, P.p, P.q, P.b, P.partial, P.pinv, P.ic_val}) cudaFree(v);
  for (int* v : {P.ic_rp, P.ic_ci, P.ic_src, P.lvl_rows_f, P.lvl_rows_b, P.icT_rp, P.icT_ci, P.icT_pos, P.ic_bad})
    cudaFree(v);
  cudaFree(P.sc);
  if (P.sc_host) cudaFreeHost(P.sc_host);
  P = Pcg();
}

// Solve A64 x = b (device vectors of length n_pad; padding entries zero).
// The preconditioner is rebuilt from A64 first, as CGSolver does on every
// solve (cgSolver.cpp:23).
od_status pcg_solve(Scene* s, const double* d_b, double* d_x, const od_solver_params* prm, od_solve_stats* st) {
  Pcg& P = s->pcg;
  cudaStream_t strm = s->ctx->stream;
  const int nb = s->bsr.nb, n = P.n_pad;
  const int pk = prm->precond;
  if (pk < 0 || pk > OD_PRECOND_IC0) { set_error("unknown preconditioner"); return OD_ERR_INVALID_ARG; }
  const int rows_per_cta = kThreads / kRowLanes;
  const int g_rows = nblk(nb, rows_per_cta), g_blk = nblk(nb, kThreads), g_vec = nblk(n, kThreads);
  if (nb == 0) {
    if (st) { *st = od_solve_stats{}; }
    return OD_OK;
  }
  double shift = 0.0;
  if (pk == OD_PRECOND_JACOBI || pk == OD_PRECOND_BLOCK_JACOBI) {
    precond_setup_kernel<double><<<g_blk, kThreads, 0, strm>>>(nb, pk, s->bsr.diag_pos, s->A64, P.pinv);
  } else if (pk == OD_PRECOND_IC0) {
    od_status e = ic0_factor(s);
    if (e != OD_OK) return e;
    shift = P.ic_shift;
  }
  pcg_init_kernel<double><<<g_rows, kThreads, 0, strm>>>(nb, s->bsr.row_ptr, s->bsr.col, s->A64, d_b, d_x, P.r, P.z,
                                                          P.p, pk, P.pinv, prm->tol, prm->max_iter, P.partial, P.sc);
  if (pk == OD_PRECOND_IC0) {
    ic0_apply(s, P.r, P.z, nullptr);
    pcg_rz_finish_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.r, P.z, P.partial, P.sc, 1);
    copy_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.z, P.p);
  }
  OD_CUDA(cudaGetLastError());
  // iterations are queued in chunks; every kernel returns at once after the
  // stop flag is set, and the host reads the flag between chunks
  const int chunk = 16;
  for (;;) {
    for (int k = 0; k < chunk; k++) {
      pcg_spmv_kernel<double><<<g_rows, kThreads, 0, strm>>>(nb, s->bsr.row_ptr, s->bsr.col, s->A64, P.p, P.q,
                                                              P.partial, P.sc);
      if (pk == OD_PRECOND_IC0) {
        pcg_update_kernel<<<g_blk, kThreads, 0, strm>>>(nb, d_x, P.r, P.z, P.p, P.q, pk, P.pinv, P.partial, P.sc, 0);
        ic0_apply(s, P.r, P.z, P.sc);
        pcg_rz_finish_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.r, P.z, P.partial, P.sc, 0);
        pcg_direction_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.z, P.p, P.sc, 0);
      } else {
        pcg_update_kernel<<<g_blk, kThreads, 0, strm>>>(nb, d_x, P.r, P.z, P.p, P.q, pk, P.pinv, P.partial, P.sc, 1);
        pcg_direction_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.z, P.p, P.sc, 0);
      }
    }
    OD_CUDA(cudaGetLastError());
    OD_CUDA(cudaMemcpyAsync(P.sc_host, P.sc, sizeof(SolveScalars), cudaMemcpyDeviceToHost, strm));
    OD_CUDA(cudaStreamSynchronize(strm));
    if (P.sc_host->done) break;
  }
  const SolveScalars& h = *P.sc_host;
  // true residual ||b - A x|| / ||b||
  spmv_full_kernel<double><<<g_rows, kThreads, 0, strm>>>(nb, s->bsr.row_ptr, s->bsr.col, s->A64, d_x, P.q);
  OD_CUDA(cudaGetLastError());
  std::vector<double> hb(n), hq(n);
  OD_CUDA(cudaMemcpyAsync(hb.data(), d_b, sizeof(double) * n, cudaMemcpyDeviceToHost, strm));
  OD_CUDA(cudaMemcpyAsync(hq.data(), P.q, sizeof(double) * n, cudaMemcpyDeviceToHost, strm));
  OD_CUDA(cudaStreamSynchronize(strm));
  double num = 0.0, den = 0.0;
  for (int i = 0; i < n; i++) { double d = hb[i] - hq[i]; num += d * d; den += hb[i] * hb[i]; }
  od_status status = (od_status)h.status;
  if (status == OD_OK && h.iter >= h.max_iter && h.rr > h.eps) status = OD_ERR_NOT_CONVERGED;
  if (st) {
    st->iterations = h.iter;
    st->refinements = 0;
    st->rel_residual = den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
    st->ic_shift = shift;
    st->status = status;
  }
  return OD_OK;
}

}  // namespace od
