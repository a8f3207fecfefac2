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
#include <cstdlib>
#include <cstdio>
#include <chrono>
#include <cstring>

#include "od_internal.h"
#include "od_grid.cuh"

namespace od {

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

// Row r of block row (blocks [kb, ke)) of c1 V1 x1 + c2 V2 x2 + c3 V3 x3
// with V* read from the lower layout.  The next block's descriptors are
// loaded with the current block's values (one memory round trip per block
// instead of two); the multiply-adds run in block, column, source order.
template <int NSRC>
__device__ __forceinline__ double lower_row(int kb, int ke, int r, const int* __restrict__ col,
                                            const int* __restrict__ kind, const int* __restrict__ off,
                                            const int* __restrict__ gen, const double* __restrict__ v1, double c1,
                                            const double* __restrict__ x1, const double* __restrict__ v2, double c2,
                                            const double* __restrict__ x2, const double* __restrict__ v3, double c3,
                                            const double* __restrict__ x3) {
  double acc = 0.0;
  if (kb >= ke) return acc;
  int cbn = 3 * col[kb], kdn = kind[kb], ofn = off[kb];
  for (int k = kb; k < ke; k++) {
    const int cb = cbn, kd = kdn, of = ofn;
    if (k + 1 < ke) {
      cbn = 3 * col[k + 1];
      kdn = kind[k + 1];
      ofn = off[k + 1];
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const int src = lower_src(kd, of, r, c, gen);
      if (src >= 0) {
        acc = fma(c1 * v1[src], x1[cb + c], acc);
        if (NSRC >= 2) acc = fma(c2 * v2[src], x2[cb + c], acc);
        if (NSRC >= 3) acc = fma(c3 * v3[src], x3[cb + c], acc);
      } else if (src == -2) {
        acc = fma(c1, x1[cb + c], acc);
      }
    }
  }
  return acc;
}

// y (+)= c1 V1 x1 + c2 V2 x2 + c3 V3 x3 with V* read from the lower layout
// through the full-BSR descriptors (SpMDV semantics, numerMethod.h:134-262).
// Three lanes per block row as in the full-BSR product; absent sources
// (NULL) cost nothing.
template <int NSRC>
__global__ void spmv_lower_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                  const int* __restrict__ kind, const int* __restrict__ off,
                                  const int* __restrict__ gen, const double* __restrict__ v1, double c1,
                                  const double* __restrict__ x1, const double* __restrict__ v2, double c2,
                                  const double* __restrict__ x2, const double* __restrict__ v3, double c3,
                                  const double* __restrict__ x3, double* __restrict__ y, int accumulate) {
  const int lane = threadIdx.x & 31;
  if (lane >= 30) return;
  const int row = (blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5)) * 10 + lane / 3;
  const int r = lane % 3;
  if (row >= nb) return;
  const double acc = lower_row<NSRC>(rp[row], rp[row + 1], r, col, kind, off, gen, v1, c1, x1, v2, c2, x2, v3, c3, x3);
  if (accumulate) y[3 * row + r] += acc;
  else y[3 * row + r] = acc;
}

// ---- several scenes per launch (Newmark system of each scene)
// A = (1 + gamma h alpha_M) M + (gamma h beta_K + beta h^2) K; a tile is
// kExpandTile of one scene's full-BSR values
__global__ void expand_batch_kernel(int n_sc, const int* __restrict__ prefix, const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  const double cK = D.gh * D.beta_k + D.bh2, cM = 1.0 + D.gh * D.alpha_m;
  const int v0 = (blockIdx.x - prefix[s]) * kExpandTile, v1 = min(9 * D.nnzb, v0 + kExpandTile);
  for (int idx = v0 + threadIdx.x; idx < v1; idx += blockDim.x) {
    const int k = idx / 9, e = idx - 9 * k;
    const int src = lower_src(D.desc_kind[k], D.desc_off[k], e / 3, e % 3, D.gen);
    D.A64[idx] = src >= 0 ? cK * D.K[src] + cM * D.M[src] : (src == -2 ? 1.0 : 0.0);
  }
}

// rhs = M tmp + beta_K K tmp2 over kBatchRows block rows of one scene
// (three lanes per block row, ten block rows per warp)
__global__ void spmv_lower_batch_kernel(int n_sc, const int* __restrict__ prefix, const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  const int lane = threadIdx.x & 31;
  if (lane >= 30) return;
  const int row = (blockIdx.x - prefix[s]) * kBatchRows + (threadIdx.x >> 5) * 10 + lane / 3;
  const int r = lane % 3;
  if (row >= D.nb) return;
  // the scene's M tmp + beta_K K tmp2 (c1 = 1: 1.0 * M[src] is M[src])
  D.rhs[3 * row + r] = lower_row<2>(D.row_ptr[row], D.row_ptr[row + 1], r, D.col, D.desc_kind, D.desc_off, D.gen,
                                    D.M, 1.0, D.tmp, D.K, D.beta_k, D.tmp2, nullptr, 0.0, nullptr);
}

// Row-block products of the full BSR.  Three lanes per block row, lane r
// owning row r of the block row: it walks the row's blocks and does three
// FMAs per block with the block's row r (three contiguous values) -- exactly
// one FMA per stored value and no cross-lane reduction, which matters on a
// part whose FP64 rate is low.  Ten block rows per warp (lanes 30, 31 idle).
constexpr int kRowsPerWarp = 10;
constexpr int kWarpRows = (kThreads / 32) * kRowsPerWarp;  // block rows per 256-thread CTA

template <class TA, class TX>
__device__ __forceinline__ double bsr_subrow(int row, int r, const int* __restrict__ rp, const int* __restrict__ col,
                                             const TA* __restrict__ A, const TX* __restrict__ x) {
  double y = 0.0;
  const int kb = rp[row], ke = rp[row + 1];
  // the next block's column is loaded with the current block's x entries
  int cn = kb < ke ? col[kb] : 0;
  for (int k = kb; k < ke; k++) {
    const TA* a = A + (size_t)k * 9 + 3 * r;
    const int c = 3 * cn;
    if (k + 1 < ke) cn = col[k + 1];
    y = fma((double)a[0], (double)x[c], y);
    y = fma((double)a[1], (double)x[c + 1], y);
    y = fma((double)a[2], (double)x[c + 2], y);
  }
  return y;
}

template <class TA>
__global__ void spmv_full_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                 const TA* __restrict__ A, const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  if (lane >= 3 * kRowsPerWarp) return;
  const int row = (blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5)) * kRowsPerWarp + lane / 3;
  const int r = lane % 3;
  if (row < nb) y[3 * row + r] = bsr_subrow<TA, double>(row, r, rp, col, A, x);
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
// Scalars flow through per-CTA partials: a producer kernel writes one
// partial per CTA, and every CTA of the consumer kernel sums all of them in
// the same fixed order (so every CTA sees the identical value, without
// atomics).  The grids are capped at two CTAs per SM with grid-stride loops,
// which keeps the partial count small.  r.z is kept in two parity slots: the
// kernel that reads slot s of iteration k only ever writes slot 1 - s.
constexpr int kUpdThreads = 192;  // multiple of 3 (whole 3x3 blocks) and of 32

// sum of part[0..m) by every thread of the CTA (fixed order), broadcast
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, int m) {
  __shared__ double bc;
  double acc = 0.0;
  for (int j = threadIdx.x; j < m; j += blockDim.x) acc += __ldcg(part + j);
  double t = block_sum(acc);
  if (threadIdx.x == 0) bc = t;
  __syncthreads();
  double v = bc;
  __syncthreads();
  return v;
}

// r = b - A x0; z = M^-1 r; p = z (local preconditioners); partials of r.z,
// b.b and r.r (cgSolver.cpp:20-30)
template <class TA>
__global__ void pcg_init_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                const TA* __restrict__ A, const double* __restrict__ b, const double* __restrict__ x,
                                double* __restrict__ r_out, double* __restrict__ z, double* __restrict__ p, int pkind,
                                const double* __restrict__ pinv, double* __restrict__ part_rz,
                                double* __restrict__ part_bb, double* __restrict__ part_rr) {
  double rz = 0.0, bb = 0.0, rr = 0.0;
  const int lane = threadIdx.x & 31;
  const int warp_global = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  __shared__ double rsh[kThreads];
  for (int wb = warp_global * kRowsPerWarp; wb < nb; wb += gridDim.x * kWarpRows) {
    const int row = wb + lane / 3, r = lane % 3;
    const bool valid = lane < 3 * kRowsPerWarp && row < nb;
    double rv = 0.0, bv = 0.0;
    if (valid) {
      const double qv = bsr_subrow<TA, double>(row, r, rp, col, A, x);
      bv = b[3 * row + r];
      rv = bv - qv;
      r_out[3 * row + r] = rv;
    }
    __syncwarp();
    rsh[threadIdx.x] = rv;
    __syncwarp();
    if (valid) {
      double zv = rv;
      if (pkind == OD_PRECOND_JACOBI) zv = pinv[3 * row + r] * rv;
      else if (pkind == OD_PRECOND_BLOCK_JACOBI) {
        const double* m = pinv + 9 * (size_t)row + 3 * r;
        const int lb = threadIdx.x - r;
        zv = m[0] * rsh[lb] + m[1] * rsh[lb + 1] + m[2] * rsh[lb + 2];
      }
      // (IC(0) and LDL^T are applied by their own sweeps)
      if (pkind < OD_PRECOND_IC0) { z[3 * row + r] = zv; p[3 * row + r] = zv; rz += rv * zv; }
      bb += bv * bv;
      rr += rv * rv;
    }
    __syncwarp();
  }
  double s0 = block_sum(rz), s1 = block_sum(bb), s2 = block_sum(rr);
  if (threadIdx.x == 0) { part_rz[blockIdx.x] = s0; part_bb[blockIdx.x] = s1; part_rr[blockIdx.x] = s2; }
}

// single CTA: rz, b.b, r.r, eps = tol^2 b.b, iteration 0, stop flag
__global__ void pcg_init_finish(const double* __restrict__ part_rz, int g_rz, const double* __restrict__ part_bb,
                                const double* __restrict__ part_rr, int g, double tol, int max_iter,
                                SolveScalars* sc) {
  const double rz = sum_partials(part_rz, g_rz);
  const double bb = sum_partials(part_bb, g);
  const double rr = sum_partials(part_rr, g);
  if (threadIdx.x == 0) {
    sc->rz[0] = rz; sc->rz[1] = rz;
    sc->bb = bb; sc->rr = rr; sc->rr0 = rr;
    sc->eps = bb * tol * tol;
    sc->iter = 0;
    sc->max_iter = max_iter;
    sc->status = isfinite(rr) ? OD_OK : OD_ERR_NAN;
    sc->done = !(0 < max_iter && rr > sc->eps) || !isfinite(rr);
  }
}

// K1: q = A p; partials of p.q
template <class TA>
__global__ void pcg_spmv_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                const TA* __restrict__ A, const double* __restrict__ p, double* __restrict__ q,
                                double* __restrict__ part_pq, const SolveScalars* sc) {
  if (*(volatile const int*)&sc->done) return;
  double pq = 0.0;
  const int lane = threadIdx.x & 31;
  const int warp_global = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  for (int wb = warp_global * kRowsPerWarp; wb < nb; wb += gridDim.x * kWarpRows) {
    const int row = wb + lane / 3, r = lane % 3;
    if (lane < 3 * kRowsPerWarp && row < nb) {
      const double y = bsr_subrow<TA, double>(row, r, rp, col, A, p);
      q[3 * row + r] = y;
      pq = fma(p[3 * row + r], y, pq);
    }
  }
  double t = block_sum(pq);
  if (threadIdx.x == 0) part_pq[blockIdx.x] = t;
}

// K2: alpha = rz / p.q; x += alpha p; r -= alpha q; z = M^-1 r (local
// preconditioners); partials of r.z and r.r.  One thread per DOF; a CTA step
// covers whole 3x3 blocks so block-Jacobi reads its block's residual from
// shared memory.
__global__ void __launch_bounds__(kUpdThreads) pcg_update_kernel(int n, double* __restrict__ x, double* __restrict__ r,
                                                                 double* __restrict__ z, const double* __restrict__ p,
                                                                 const double* __restrict__ q, int pkind,
                                                                 const double* __restrict__ pinv,
                                                                 const double* __restrict__ part_pq, int g_pq,
                                                                 double* __restrict__ part_rz,
                                                                 double* __restrict__ part_rr, SolveScalars* sc,
                                                                 int slot) {
  if (*(volatile int*)&sc->done) return;
  __shared__ double rs[kUpdThreads];
  const double pq = sum_partials(part_pq, g_pq);
  const double alpha = sc->rz[slot] / pq;
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->alpha = alpha;
  double rz = 0.0, rr = 0.0;
  for (int base = blockIdx.x * kUpdThreads; base < n; base += gridDim.x * kUpdThreads) {
    const int i = base + threadIdx.x;
    const bool valid = i < n;
    double rv = 0.0;
    if (valid) {
      x[i] += alpha * p[i];
      rv = r[i] - alpha * q[i];
      r[i] = rv;
    }
    __syncthreads();
    rs[threadIdx.x] = rv;
    __syncthreads();
    rr += rv * rv;
    if (valid && pkind < OD_PRECOND_IC0) {
      double zv;
      if (pkind == OD_PRECOND_JACOBI) {
        zv = pinv[i] * rv;
      } else if (pkind == OD_PRECOND_BLOCK_JACOBI) {
        const int d = i % 3, lb = threadIdx.x - d;
        const double* m = pinv + 3 * (size_t)i;  // row d of block i / 3
        zv = m[0] * rs[lb] + m[1] * rs[lb + 1] + m[2] * rs[lb + 2];
      } else {
        zv = rv;
      }
      z[i] = zv;
      rz += rv * zv;
    }
  }
  double s0 = block_sum(rz), s1 = block_sum(rr);
  if (threadIdx.x == 0) { part_rz[blockIdx.x] = s0; part_rr[blockIdx.x] = s1; }
}

// partials of r.z (IC(0): after the triangular solves)
__global__ void pcg_rz_kernel(int n, const double* __restrict__ r, const double* __restrict__ z,
                              double* __restrict__ part_rz, const SolveScalars* sc) {
  if (sc && *(volatile const int*)&sc->done) return;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += r[i] * z[i];
  double t = block_sum(acc);
  if (threadIdx.x == 0) part_rz[blockIdx.x] = t;
}

// K3: beta = (r.z)_new / (r.z); p = z + beta p; CTA 0 records the new r.z
// in the other slot, r.r, the iteration count and the stop test
// (cgSolver.cpp:32-54)
__global__ void pcg_direction_kernel(int n, const double* __restrict__ z, double* __restrict__ p,
                                     const double* __restrict__ part_rz, int g_rz, const double* __restrict__ part_rr,
                                     int g_rr, SolveScalars* sc, int slot) {
  if (*(volatile int*)&sc->done) return;
  const double rz_new = sum_partials(part_rz, g_rz);
  const double rr = sum_partials(part_rr, g_rr);
  const double beta = rz_new / sc->rz[slot];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = beta * p[i] + z[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rz[1 - slot] = rz_new;
    sc->rr = rr;
    sc->beta = beta;
    const int it = sc->iter + 1;
    sc->iter = it;
    if (!isfinite(rr) || !isfinite(beta)) { sc->status = OD_ERR_NAN; sc->done = 1; }
    else sc->done = !(it < sc->max_iter && rr > sc->eps);
  }
}

// ||b - q||^2 and ||b||^2 (true residual, q = A x); single CTA
__global__ void residual_norm_kernel(int n, const double* __restrict__ b, const double* __restrict__ q,
                                     SolveScalars* sc) {
  double d2 = 0.0, bb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = b[i] - q[i];
    d2 += d * d;
    bb += b[i] * b[i];
  }
  double t0 = block_sum(d2), t1 = block_sum(bb);
  if (threadIdx.x == 0) { sc->tr_num = t0; sc->tr_den = t1; }
}

// ------------------------------------------------------ persistent PCG
// The whole Jacobi / block-Jacobi / unpreconditioned solve in one
// cooperative launch: every CTA is resident (cudaLaunchCooperativeKernel
// refuses grids that are not), the phases of an iteration are separated by a
// grid barrier, and every CTA forms the scalars itself from the per-CTA
// partials in a fixed order, so all CTAs take identical loop decisions.
//
// The barrier is a sense (generation) barrier in global memory.  Its waits
// are bounded: after kSpinLimit polls the waiting CTA records a timeout and
// every CTA leaves the solve at the next barrier, so the kernel always
// returns and the host reports OD_ERR_DEVICE_TIMEOUT.
constexpr int kPThreads = 768;                          // 24 warps; multiple of 3

// sum of part[0..m) by every CTA in the same order, broadcast to the CTA
__device__ __forceinline__ double cta_sum(const double* __restrict__ part, int m) {
  return sum_partials(part, m);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;  // lane 0
}

// Grid-wide sums of NV per-thread values with one grid barrier and two
// CTA barriers.  FP64 arithmetic is scarce on this part (about 1.7 lane
// operations per SM per cycle), so the CTA's threads do none of the
// reduction: they store their values to shared memory, warp 0 sums each
// value's kPThreads entries (four fixed accumulator chains per lane, then
// the lanes by shuffles), lane 0 of warp 0 takes part in the grid barrier,
// then warp 0 sums all CTA partials in a fixed order.  Lane 0 then calls
// fin(sums, extra) once for the CTA (the scalars every thread needs, e.g. a
// step length, computed once instead of by every thread) and everything is
// broadcast through shared memory.  Every CTA obtains bitwise the same sums.
// Returns false after a barrier timeout.
struct NoFinish {
  __device__ void operator()(const double*, double*) const {}
};
constexpr int kSumsMax = 3;   // values per reduction
// one shared block for every instantiation of grid_sums in a kernel (a
// static __shared__ array inside the template would exist once per
// instantiation)
struct SumsShared {
  double vals[kSumsMax][kPThreads];
  double res[kSumsMax + 2];
  int ok;
  unsigned epoch;   // barriers this CTA has passed (thread 0 only)
};
__device__ __forceinline__ SumsShared& sums_shared() {
  __shared__ SumsShared sh;
  return sh;
}
// the plain barrier of the kernels that use grid_sums (same counter)
__device__ __forceinline__ bool grid_barrier_count(GridBarrier* gb) {
  SumsShared& sh = sums_shared();
  __syncthreads();
  if (threadIdx.x == 0) sh.ok = barrier_arrive_wait_count(gb, ++sh.epoch);
  __syncthreads();
  return sh.ok != 0;
}
// loads per lane issued together when a grid sum reads the CTA partials
// (5 x 32 covers one CTA per SM on 152 SMs in one pass)
constexpr int kGridSumLoads = 5;

template <int NV, int NX = 0, class F = NoFinish>
__device__ __forceinline__ bool grid_sums(double (&v)[NV], double* __restrict__ part, GridBarrier* gb,
                                          unsigned long long* __restrict__ work = nullptr,
                                          unsigned long long t0 = 0, double* xout = nullptr, F fin = F()) {
  static_assert(NV <= kSumsMax, "grid_sums: too many values");
  SumsShared& sh = sums_shared();
  auto& vals = sh.vals;
  double* res = sh.res;
  int& ok_s = sh.ok;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int G = gridDim.x;
#pragma unroll
  for (int j = 0; j < NV; j++) vals[j][threadIdx.x] = v[j];
  __syncthreads();
  if (work && threadIdx.x == 0) {  // profiling: this CTA's own share of the phase
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    work[blockIdx.x] += t - t0;
  }
  if (w == 0) {
#pragma unroll
    for (int j = 0; j < NV; j++) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      for (int i = lane; i < (int)blockDim.x; i += 128) {
        a0 += vals[j][i];
        if (i + 32 < (int)blockDim.x) a1 += vals[j][i + 32];
        if (i + 64 < (int)blockDim.x) a2 += vals[j][i + 64];
        if (i + 96 < (int)blockDim.x) a3 += vals[j][i + 96];
      }
      const double t = warp_sum((a0 + a1) + (a2 + a3));
      if (lane == 0) part[(size_t)j * G + blockIdx.x] = t;
    }
    int ok = 1;
    if (lane == 0) ok = barrier_arrive_wait_count(gb, ++sh.epoch);
    __syncwarp();   // orders lane 0's acquire before the other lanes' partial reads
    ok = __shfl_sync(0xffffffffu, ok, 0);
    // every lane's loads of a pass issued before any is used (one L2 round
    // trip per pass); each lane adds its entries in increasing CTA order
    double acc[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) acc[j] = 0.0;
    for (int c0 = 0; c0 < G; c0 += 32 * kGridSumLoads) {
      double ld[NV][kGridSumLoads];
#pragma unroll
      for (int j = 0; j < NV; j++)
#pragma unroll
        for (int q = 0; q < kGridSumLoads; q++) {
          const int c = c0 + lane + 32 * q;
          ld[j][q] = c < G ? __ldcg(part + (size_t)j * G + c) : 0.0;
        }
#pragma unroll
      for (int j = 0; j < NV; j++)
#pragma unroll
        for (int q = 0; q < kGridSumLoads; q++) acc[j] += ld[j][q];
    }
#pragma unroll
    for (int j = 0; j < NV; j++) {
      const double t = warp_sum(acc[j]);
      if (lane == 0) res[j] = t;
    }
    if (lane == 0) {
      ok_s = ok;
      if constexpr (NX > 0) fin(res, res + NV);
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; j++) v[j] = res[j];
  if constexpr (NX > 0) {
#pragma unroll
    for (int j = 0; j < NX; j++) xout[j] = res[NV + j];
  }
  return ok_s != 0;
}

// Work decomposition of the persistent solve: "groups" of 10 block rows
// (30 DOFs, lanes 0..29 of a warp; lane l owns DOF 30 g + l, i.e. row l % 3
// of block row 10 g + l / 3).  Group g goes to warp g / G of CTA g % G, so
// every CTA -- every SM, whose FP64 pipe is the limit -- gets an equal share.
// With GPW > 0 a warp owns at most GPW groups and keeps x, r, z, p and q of
// its DOFs in registers across the grid barriers; only p goes back to memory
// (the SpMV gathers it).  With GPW == 0 the vectors stream from memory.
// Loop over the groups a warp owns.  With GPW > 0 the outer loop is fully
// unrolled (k is a compile-time index into the register arrays) and the
// inner one runs at most once; with GPW == 0 the inner loop strides over all
// groups and the vectors live in memory.
#define OD_GROUP_LOOP(k, g)                                                   \
  _Pragma("unroll") for (int k = 0; k < (GPW > 0 ? NR : 1); k++)              \
    for (int g = g0 + k * gstride; g < ngroups; g += (GPW > 0 ? ngroups : gstride))

// With SMEM (at most two groups per warp) every CTA first copies the
// matrix blocks of its rows (9 values each, then their block columns) and
// its rows of the Jacobi / block-Jacobi inverse into shared memory, one
// segment per (warp, group), and every later product and preconditioner
// apply reads them there: only the gathered vector entries go to L2.  The
// products take the same operations in the same order as bsr_subrow.
constexpr int kSmemGroupsMax = 2;                             // groups per warp of the SMEM variant
constexpr int kSmemSegs = (kPThreads / 32) * kSmemGroupsMax;  // (warp, group) segments per CTA
constexpr int kSmemPinv = 9 * kRowsPerWarp;                   // inverse values per segment

template <class TA, int GPW, bool SMEM>
__global__ void __launch_bounds__(kPThreads, 1) pcg_persistent_kernel(
    int nb, const int* __restrict__ rp, const int* __restrict__ col, const TA* __restrict__ A,
    const double* __restrict__ b, double* __restrict__ x, double* __restrict__ r, double* __restrict__ z,
    double* __restrict__ p, double* __restrict__ q, int pkind, const double* __restrict__ pinv,
    double* __restrict__ part, double tol, int max_iter, SolveScalars* sc, GridBarrier* gb,
    unsigned long long* __restrict__ prof, int recur) {
  constexpr int NR = GPW > 0 ? GPW : 1;
  static_assert(!SMEM || (GPW >= 1 && GPW <= kSmemGroupsMax), "the SMEM variant keeps 1 or 2 groups per warp");
  if (threadIdx.x == 0) sums_shared().epoch = 0;   // the counting barrier's epochs (thread 0 only)
  const int G = gridDim.x;
  double* part_1 = part;          // one-value reductions (p.q, residual)
  double* part_2 = part + G;      // two/three-value reductions (G entries per value)
  const int lane = threadIdx.x & 31;
  const int wpc = kPThreads / 32;
  const int w = threadIdx.x >> 5;
  const int ngroups = (nb + kRowsPerWarp - 1) / kRowsPerWarp;
  const int gstride = G * wpc;
  const int g0 = w * G + blockIdx.x;
  const int rsub = lane % 3;
  const int lbase = lane - rsub;

  double xr[NR], rv[NR], zv[NR], pv[NR], qv[NR];

  // ---- SMEM: stage this CTA's matrix rows and inverse rows
  extern __shared__ __align__(16) unsigned char pcg_dsm[];
  __shared__ int seg_off[SMEM ? kSmemSegs + 1 : 1];
  double* sA = nullptr;   // 9 values per block of the CTA's segments
  int* sC = nullptr;      // their block columns
  double* sP = nullptr;   // kSmemPinv inverse values per segment
  int lb[NR], le[NR];     // this lane's row: its blocks in the CTA's segments
  if constexpr (SMEM) {
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < NR; k++) {
        const int g = g0 + k * gstride;
        int cnt = 0;
        if (g < ngroups) {
          const int r0 = g * kRowsPerWarp, r1 = min(nb, r0 + kRowsPerWarp);
          cnt = rp[r1] - rp[r0];
        }
        seg_off[w * NR + k] = cnt;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int i = 0; i < wpc * NR; i++) {
        const int c = seg_off[i];
        seg_off[i] = acc;
        acc += c;
      }
      seg_off[wpc * NR] = acc;
    }
    __syncthreads();
    sP = reinterpret_cast<double*>(pcg_dsm);
    sA = sP + (size_t)wpc * NR * kSmemPinv;
    sC = reinterpret_cast<int*>(sA + 9 * (size_t)seg_off[wpc * NR]);
#pragma unroll
    for (int k = 0; k < NR; k++) {
      const int g = g0 + k * gstride;
      lb[k] = le[k] = 0;
      if (g >= ngroups) continue;
      const int r0 = g * kRowsPerWarp, r1 = min(nb, r0 + kRowsPerWarp);
      const int base = rp[r0], off = seg_off[w * NR + k], cnt = rp[r1] - base;
      for (int i = lane; i < 9 * cnt; i += 32) sA[9 * (size_t)off + i] = (double)A[9 * (size_t)base + i];
      for (int i = lane; i < cnt; i += 32) sC[off + i] = col[base + i];
      double* dst = sP + (size_t)(w * NR + k) * kSmemPinv;
      if (pkind == OD_PRECOND_BLOCK_JACOBI)
        for (int i = lane; i < 9 * (r1 - r0); i += 32) dst[i] = pinv[9 * (size_t)r0 + i];
      else if (pkind == OD_PRECOND_JACOBI)
        for (int i = lane; i < 3 * (r1 - r0); i += 32) dst[i] = pinv[3 * (size_t)r0 + i];
      const int row = r0 + lane / 3;
      if (lane < 30 && row < nb) {
        lb[k] = off + rp[row] - base;
        le[k] = off + rp[row + 1] - base;
      }
    }
    __syncthreads();
  }
  // row product of this lane's row (group slot k) with v
  auto row_product = [&](int k, int row, const double* __restrict__ v) -> double {
    if constexpr (SMEM) {
      double y = 0.0;
      for (int j = lb[k]; j < le[k]; j++) {
        const double* a = sA + (size_t)j * 9 + 3 * rsub;
        const int c = 3 * sC[j];
        y = fma(a[0], v[c], y);
        y = fma(a[1], v[c + 1], y);
        y = fma(a[2], v[c + 2], y);
      }
      return y;
    } else {
      (void)k;
      return bsr_subrow<TA, double>(row, rsub, rp, col, A, v);
    }
  };

  // z = M^-1 r inside the warp (block-Jacobi through shuffles of the 3 lanes
  // of a block row; every lane takes part in the shuffles)
  auto apply_precond = [&](int k, int row, bool valid, double rl) {
    double r0 = __shfl_sync(0xffffffffu, rl, lbase < 32 ? lbase : 0);
    double r1 = __shfl_sync(0xffffffffu, rl, lbase + 1 < 32 ? lbase + 1 : 0);
    double r2 = __shfl_sync(0xffffffffu, rl, lbase + 2 < 32 ? lbase + 2 : 0);
    if (!valid) return 0.0;
    if constexpr (SMEM) {
      const double* seg = sP + (size_t)(w * NR + k) * kSmemPinv;
      if (pkind == OD_PRECOND_JACOBI) return seg[lane] * rl;
      if (pkind == OD_PRECOND_BLOCK_JACOBI) {
        const double* m = seg + 3 * lane;
        return m[0] * r0 + m[1] * r1 + m[2] * r2;
      }
    } else {
      (void)k;
      if (pkind == OD_PRECOND_JACOBI) return pinv[3 * row + rsub] * rl;
      if (pkind == OD_PRECOND_BLOCK_JACOBI) {
        const double* m = pinv + 9 * (size_t)row + 3 * rsub;
        return m[0] * r0 + m[1] * r1 + m[2] * r2;
      }
    }
    return rl;
  };

  double rz = 0.0, bb = 0.0, rr = 0.0, eps = 0.0;
  int it = 0, status = OD_OK;
  if (GPW > 0 && recur == 2) {
    // ---- pipelined PCG (Ghysels and Vanroose, 2014): u = M^-1 r, w = A u
    // and m = M^-1 w are carried by recurrences, so an iteration's three dot
    // products (r.u, w.u, r.r) and the completion of m, which the product
    // gathers, share one grid-wide sync.  m alternates between two arrays
    // and the sums' partials between two halves by iteration parity: a CTA
    // can only write an array again after the next sync, which every CTA
    // reaches after its last read.  Same iterates as the reference's PCG in
    // exact arithmetic; the stop test is the reference's, on r.r.
    double uv[NR], wv[NR], sv[NR], zr[NR], mv[NR];
    double* const mbuf[2] = {z, q};
    double* const pbuf[2] = {part, part + 3 * (size_t)G};
    double bbl = 0.0;
    OD_GROUP_LOOP(k, g) {
      const int row = g * kRowsPerWarp + lane / 3;
      const bool valid = lane < 30 && row < nb;
      const int i = 3 * row + rsub;
      double bv = 0.0, rl = 0.0;
      if (valid) {
        bv = b[i];
        xr[k] = x[i];
        rl = bv - row_product(k, row, x);
      }
      const double ul = apply_precond(k, row, valid, rl);
      if (valid) {
        rv[k] = rl;
        uv[k] = ul;
        pv[k] = qv[k] = sv[k] = zr[k] = 0.0;
        p[i] = ul;   // gathered by w = A u
        bbl = fma(bv, bv, bbl);
      }
    }
    {
      double v1[1] = {bbl};
      if (!grid_sums<1>(v1, part + 6 * (size_t)G, gb)) return;
      bb = v1[0];
    }
    OD_GROUP_LOOP(k, g) {
      const int row = g * kRowsPerWarp + lane / 3;
      if (lane < 30 && row < nb) wv[k] = row_product(k, row, p);
    }
    eps = bb * tol * tol;
    double gam_prev = 1.0, alpha_prev = 1.0;
    // profiling: CTA 0's clock into the slots of the standard form: the
    // product and recurrences -> [0], the dots and m -> [2], the sum -> [3]
    const bool ptimer = prof && blockIdx.x == 0 && threadIdx.x == 0;
    unsigned long long pt = 0;
    auto pstamp = [&](int slot) {
      if (!ptimer) return;
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (slot >= 0) prof[slot] += t - pt;
      pt = t;
    };
    for (;;) {
      const int par = it & 1;
      pstamp(-1);
      double ga = 0.0, de = 0.0, rrl = 0.0;
      OD_GROUP_LOOP(k, g) {
        const int row = g * kRowsPerWarp + lane / 3;
        const bool valid = lane < 30 && row < nb;
        const int i = 3 * row + rsub;
        const double ml = apply_precond(k, row, valid, valid ? wv[k] : 0.0);
        if (valid) {
          mv[k] = ml;
          mbuf[par][i] = ml;
          ga = fma(rv[k], uv[k], ga);
          de = fma(wv[k], uv[k], de);
          rrl = fma(rv[k], rv[k], rrl);
        }
      }
      pstamp(2);
      double v3[3] = {ga, de, rrl}, ab[2];
      const bool first = it == 0;
      // beta = gamma / gamma_prev, alpha = gamma / (delta - beta gamma / alpha_prev), once per CTA
      if (!grid_sums<3, 2>(v3, pbuf[par], gb, nullptr, 0, ab, [=](const double* sm, double* xo) {
            const double be = first ? 0.0 : sm[0] / gam_prev;
            xo[0] = first ? sm[0] / sm[1] : sm[0] / (sm[1] - be * sm[0] / alpha_prev);
            xo[1] = be;
          }))
        return;
      pstamp(3);
      rz = v3[0];
      rr = v3[2];
      if (!isfinite(rr)) {
        status = OD_ERR_NAN;
        break;
      }
      if (!(rr > eps) || it >= max_iter) break;
      const double alpha = ab[0], beta = ab[1];
      if (!isfinite(alpha) || !isfinite(beta)) {
        status = OD_ERR_NAN;
        break;
      }
      gam_prev = v3[0];
      alpha_prev = alpha;
      OD_GROUP_LOOP(k, g) {
        const int row = g * kRowsPerWarp + lane / 3;
        if (lane < 30 && row < nb) {
          const double nl = row_product(k, row, mbuf[par]);
          zr[k] = fma(beta, zr[k], nl);
          qv[k] = fma(beta, qv[k], mv[k]);
          sv[k] = fma(beta, sv[k], wv[k]);
          pv[k] = fma(beta, pv[k], uv[k]);
          xr[k] = fma(alpha, pv[k], xr[k]);
          rv[k] = fma(-alpha, sv[k], rv[k]);
          uv[k] = fma(-alpha, qv[k], uv[k]);
          wv[k] = fma(-alpha, zr[k], wv[k]);
        }
      }
      pstamp(0);
      if (ptimer) prof[6] += 1;
      it++;
    }
  } else {
  // ---- init: r = b - A x; z = M^-1 r; p = z (cgSolver.cpp:20-30)
  {
    OD_GROUP_LOOP(k, g) {
      const int row = g * kRowsPerWarp + lane / 3;
      const bool valid = lane < 30 && row < nb;
      const int i = 3 * row + rsub;
      double bv = 0.0, xl = 0.0, rl = 0.0;
      if (valid) {
        bv = b[i];
        xl = x[i];
        rl = bv - row_product(k, row, x);
      }
      const double zl = apply_precond(k, row, valid, rl);
      if (valid) {
        rz = fma(rl, zl, rz);
        bb = fma(bv, bv, bb);
        rr = fma(rl, rl, rr);
        if (GPW > 0) { xr[k] = xl; rv[k] = rl; zv[k] = zl; pv[k] = recur ? 0.0 : zl; qv[k] = 0.0; }
        else { r[i] = rl; z[i] = zl; if (recur) q[i] = 0.0; }
        p[i] = recur ? 0.0 : zl;
        if (recur) z[i] = zl;   // the gathered vector of the recurrence form
      }
    }
  }
  {
    double v3[3] = {rz, bb, rr};
    if (!grid_sums<3>(v3, part_2, gb)) return;
    rz = v3[0]; bb = v3[1]; rr = v3[2];
  }
  eps = bb * tol * tol;
  status = isfinite(rr) ? OD_OK : OD_ERR_NAN;

  // profiling (prof != nullptr): CTA 0 stamps the phases of every iteration
  // (its own work, then its wait in the grid-wide sum or barrier that ends
  // the phase) into prof[0..5]; prof[6] counts the iterations; every CTA b
  // adds the time its own warps took for the SpMV, update and direction
  // phases to prof[7 + k G + b], k = 0, 1, 2
  const bool timer = prof && blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long* cta_work = prof ? prof + kPcgProfSlots : nullptr;
  unsigned long long t_prev = 0, t_phase = 0;
  auto stamp = [&](int slot) {
    if (!timer) return;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (slot >= 0) prof[slot] += t - t_prev;
    t_prev = t;
  };
  auto phase_start = [&]() {
    if (prof && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_phase));
  };
  // recurrence form (recur != 0): the product is A z, then q = A z + beta q
  // and p = z + beta p in place (A p = A z + beta A p_prev), so the
  // direction pass and its barrier go; beta_r is the last iteration's beta
  double beta_r = 0.0;
  while (status == OD_OK && it < max_iter && rr > eps) {
    stamp(-1);
    phase_start();
    // ---- q = A p (or A z + beta q); p.q
    double pq = 0.0;
    {
      OD_GROUP_LOOP(k, g) {
        const int row = g * kRowsPerWarp + lane / 3;
        if (lane < 30 && row < nb) {
          const int i = 3 * row + rsub;
          if (!recur) {
            const double y = row_product(k, row, p);
            const double pl = GPW > 0 ? pv[k] : p[i];
            if (GPW > 0) qv[k] = y; else q[i] = y;
            pq = fma(pl, y, pq);
          } else {
            const double y = row_product(k, row, z);
            double pl, ql;
            if (GPW > 0) {
              ql = qv[k] = fma(beta_r, qv[k], y);
              pl = pv[k] = fma(beta_r, pv[k], zv[k]);
            } else {
              ql = q[i] = fma(beta_r, q[i], y);
              pl = p[i] = fma(beta_r, p[i], z[i]);
            }
            pq = fma(pl, ql, pq);
          }
        }
      }
    }
    stamp(0);
    double v1[1] = {pq}, ax[1];
    // alpha = r.z / p.q, formed once per CTA
    if (!grid_sums<1, 1>(v1, part_1, gb, cta_work, t_phase, ax,
                         [rz](const double* sums, double* x) { x[0] = rz / sums[0]; }))
      return;
    stamp(1);
    const double alpha = ax[0];
    phase_start();
    // ---- x += alpha p; r -= alpha q; z = M^-1 r; r.z, r.r
    double rzn = 0.0, rrn = 0.0;
    {
      OD_GROUP_LOOP(k, g) {
        const int row = g * kRowsPerWarp + lane / 3;
        const bool valid = lane < 30 && row < nb;
        const int i = 3 * row + rsub;
        double rl = 0.0;
        if (valid) {
          if (GPW > 0) {
            xr[k] = fma(alpha, pv[k], xr[k]);
            rl = fma(-alpha, qv[k], rv[k]);
            rv[k] = rl;
          } else {
            x[i] = fma(alpha, p[i], x[i]);
            rl = fma(-alpha, q[i], r[i]);
            r[i] = rl;
          }
        }
        const double zl = apply_precond(k, row, valid, rl);
        if (valid) {
          if (GPW > 0) zv[k] = zl; else z[i] = zl;
          if (GPW > 0 && recur) z[i] = zl;   // gathered by the next product
          rzn = fma(rl, zl, rzn);
          rrn = fma(rl, rl, rrn);
        }
      }
    }
    stamp(2);
    double v2[2] = {rzn, rrn}, bx[1];
    // beta = r.z (new) / r.z (old), formed once per CTA
    if (!grid_sums<2, 1>(v2, part_2, gb, cta_work ? cta_work + G : nullptr, t_phase, bx,
                         [rz](const double* sums, double* x) { x[0] = sums[0] / rz; }))
      return;
    stamp(3);
    const double rz_new = v2[0];
    rr = v2[1];
    const double beta = bx[0];
    rz = rz_new;
    it++;
    if (!isfinite(rr) || !isfinite(beta)) status = OD_ERR_NAN;
    if (recur) {
      beta_r = beta;
      if (timer) prof[6] += 1;
      continue;
    }
    phase_start();
    // ---- p = z + beta p
    {
      OD_GROUP_LOOP(k, g) {
        const int row = g * kRowsPerWarp + lane / 3;
        if (lane < 30 && row < nb) {
          const int i = 3 * row + rsub;
          if (GPW > 0) { pv[k] = fma(beta, pv[k], zv[k]); p[i] = pv[k]; }
          else p[i] = fma(beta, p[i], z[i]);
        }
      }
    }
    stamp(4);
    if (cta_work) {  // profiling: this CTA's own share of the direction phase
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        cta_work[2 * G + blockIdx.x] += t - t_phase;
      }
    }
    if (!grid_barrier_count(gb)) return;
    stamp(5);
    if (timer) prof[6] += 1;
  }
  }   // the reference's form and the recurrence form
  // ---- write back x, then the true residual ||b - A x||^2
  if (GPW > 0) {
    OD_GROUP_LOOP(k, g) {
      const int row = g * kRowsPerWarp + lane / 3;
      if (lane < 30 && row < nb) x[3 * row + rsub] = xr[k];
    }
  }
  if (!grid_barrier_count(gb)) return;
  double d2 = 0.0;
  OD_GROUP_LOOP(k, g) {
    const int row = g * kRowsPerWarp + lane / 3;
    if (lane < 30 && row < nb) {
      const double dv = b[3 * row + rsub] - row_product(k, row, x);
      d2 = fma(dv, dv, d2);
    }
  }
  double vr[1] = {d2};
  if (!grid_sums<1>(vr, part_1, gb)) return;
  if (blockIdx.x == 0) {
    const double tr = vr[0];
    if (threadIdx.x == 0) {
      sc->rz[0] = rz;
      sc->rr = rr;
      sc->bb = bb;
      sc->eps = eps;
      sc->iter = it;
      sc->max_iter = max_iter;
      sc->status = status;
      sc->tr_num = tr;
      sc->tr_den = bb;
      sc->done = 1;
    }
  }
}

// --------------------------------------------------- mixed precision
// Inner solve of the iterative refinement: PCG on the FP32 copy of A with
// FP32 vectors, FP32 SpMV with FP32 accumulation and an FP32 block-Jacobi /
// Jacobi apply.  Dot products are accumulated per thread in compensated FP32
// (error-free TwoProduct by FMA and TwoSum, i.e. twice-FP32 accuracy on the
// FP32 units) and reduced across threads and CTAs in FP64.

struct Comp { float s, c; };
__device__ __forceinline__ void comp_add_prod(Comp& a, float x, float y) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);       // x*y = p + e exactly
  const float s = a.s + p;
  const float z = s - a.s;
  const float t = (a.s - (s - z)) + (p - z);  // a.s + p = s + t exactly
  a.s = s;
  a.c += t + e;
}
__device__ __forceinline__ double comp_value(const Comp& a) { return (double)a.s + (double)a.c; }
// Sum of the 32 lanes' compensated partials in compensated FP32 (TwoSum of
// the leading parts, the errors and trailing parts added), so only lane 0
// converts to FP64: the FP64 pipe is far slower than the FP32 one here.
// The sum's relative error stays near 2^-44 for these few levels.
__device__ __forceinline__ double comp_warp_sum(Comp a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float bs = __shfl_down_sync(0xffffffffu, a.s, o);
    const float bc = __shfl_down_sync(0xffffffffu, a.c, o);
    const float s = a.s + bs;
    const float z = s - a.s;
    const float t = (a.s - (s - z)) + (bs - z);
    a.s = s;
    a.c = (a.c + bc) + t;
  }
  return comp_value(a);  // lane 0
}

// ---- sliced FP32 systems of one or more scenes (layout: SliceSys)
// Per-scene arrays are reached through MixDesc; every kernel below is one
// launch for all scenes of a system, a CTA finding its scene in a tile
// directory.
constexpr int kFillSteps = 32;                              // steps per fill tile
constexpr int kResRows = (kThreads / 32) * kRowsPerWarp;    // block rows per residual tile

__device__ __forceinline__ float* mix_pinv(const MixDesc& D) { return D.v32 + 160 * (size_t)D.ns; }
__device__ __forceinline__ float* mix_d(const MixDesc& D) { return D.v32 + 40 * (size_t)D.ns; }

// values of each scene's sliced matrix from its FP64 full BSR
__global__ void mix_fill_kernel(int n_sc, const int* __restrict__ prefix, const MixDesc* __restrict__ desc) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const MixDesc& D = desc[s];
  const int st0 = (blockIdx.x - prefix[s]) * kFillSteps;
  const int nv = (min(D.steps, st0 + kFillSteps) - st0) * 90;
  const double* __restrict__ A = D.A64;
  for (int q = threadIdx.x; q < nv; q += blockDim.x) {
    const int st = st0 + q / 90, rem = q % 90;
    const int j = rem / 30, lane = rem - 30 * j;
    const int blk = D.ssrc[(size_t)st * kSliceRows + lane / 3];
    float v = 0.f;   // padding
    if (blk >= 0) v = (float)A[(size_t)blk * 9 + 3 * (lane % 3) + j];
    else if (blk <= -2) v = (float)(0.5 * A[(size_t)(-blk - 2) * 9 + 3 * (lane % 3) + j]);   // halved diagonal
    D.sval[(size_t)st * 90 + rem] = v;
  }
}

// FP32 Jacobi (30 per slice) or block-Jacobi (90 per slice, [j][lane]) from
// the FP64 diagonal blocks, in slice order; padding rows get zeros
__global__ void mix_precond_kernel(int n_sc, const int* __restrict__ prefix, int kind,
                                   const MixDesc* __restrict__ desc) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const MixDesc& D = desc[s];
  const int rs = (blockIdx.x - prefix[s]) * blockDim.x + threadIdx.x;
  if (rs >= D.ns * kSliceRows) return;
  const int sl = rs / kSliceRows, t = rs - sl * kSliceRows;
  const int row = D.sperm[rs];
  const double* m = row >= 0 ? D.A64 + (size_t)D.diag_pos[row] * 9 : nullptr;
  float* pinv = mix_pinv(D);
  if (kind == OD_PRECOND_JACOBI) {
    for (int d = 0; d < 3; d++) {
      float v = 0.f;
      if (m) v = (float)(m[4 * d] > 0.0 ? 1.0 / m[4 * d] : 1.0);
      pinv[(size_t)30 * sl + 3 * t + d] = v;
    }
    return;
  }
  double o[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (m) {
    const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                       m[2] * (m[3] * m[7] - m[4] * m[6]);
    const double inv = 1.0 / det;
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
  for (int r = 0; r < 3; r++)
    for (int j = 0; j < 3; j++) pinv[(size_t)90 * sl + 30 * j + 3 * t + r] = (float)o[3 * r + j];
}

// r64 = b - A64 x (FP64) over kResRows block rows of a scene (three lanes per
// block row, ten block rows per warp) and the tile's partials of r.r, b.b
// r64 = b - A64 x and the tile partials of r.r, b.b; x_zero: x is known to
// be 0, so r64 = b without the product (b - A 0 is b bit for bit)
__global__ void mix_residual_kernel(int n_sc, const int* __restrict__ prefix, const MixDesc* __restrict__ desc,
                                    double* __restrict__ part, int x_zero) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const MixDesc& D = desc[s];
  const int lane = threadIdx.x & 31;
  const int row = (blockIdx.x - prefix[s]) * kResRows + (threadIdx.x >> 5) * kRowsPerWarp + lane / 3;
  const int rs = lane % 3;
  double rr = 0.0, bb = 0.0;
  if (lane < 30 && row < D.nb) {
    const int i = 3 * row + rs;
    const double bv = D.b[i];
    const double rv = x_zero ? bv : bv - bsr_subrow<double, double>(row, rs, D.row_ptr, D.col, D.A64, D.x);
    D.r64[i] = rv;
    rr = rv * rv;
    bb = bv * bv;
  }
  const double t0 = block_sum(rr), t1 = block_sum(bb);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = t0;
    part[2 * blockIdx.x + 1] = t1;
  }
}

// per scene: r.r and b.b over the scene's residual tiles in a fixed order
__global__ void mix_residual_finish(int n_sc, const int* __restrict__ prefix, const double* __restrict__ part,
                                    double* __restrict__ rrbb) {
  const int s = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= n_sc) return;
  double a = 0.0, b = 0.0;
  for (int k = prefix[s] + lane; k < prefix[s + 1]; k += 32) {
    a += part[2 * k];
    b += part[2 * k + 1];
  }
  a = warp_sum(a);
  b = warp_sum(b);
  if (lane == 0) {
    rrbb[2 * s] = a;
    rrbb[2 * s + 1] = b;
  }
}

// x += ||r64|| d for the scenes of the sweep (slice order back to block rows)
__global__ void mix_update_kernel(int n_sc, const int* __restrict__ prefix, const MixDesc* __restrict__ desc,
                                  const RingScene* __restrict__ ring) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  if (!ring[s].active0) return;
  const MixDesc& D = desc[s];
  const int tid = (blockIdx.x - prefix[s]) * blockDim.x + threadIdx.x;
  if (tid >= 3 * kSliceRows * D.ns) return;
  const int rs = tid / 3, c = tid - 3 * rs;
  const int row = D.sperm[rs];
  if (row < 0) return;
  const int sl = rs / kSliceRows, t = rs - sl * kSliceRows;
  D.x[3 * (size_t)row + c] += ring[s].unscale * (double)mix_d(D)[(size_t)30 * sl + 3 * t + c];
}

// ---- bulk-copy ring of the inner FP32 PCG
// Every CTA owns a contiguous range of slices (of one or more scenes);
// consumer warp w of the CTA takes slices first + w, first + w + NW,
// ...  Producer lane w (of the CTA's last warp) streams warp w's slices, cut
// into pieces of at most PS steps (a template parameter), from global memory into a private
// two-stage ring in shared memory with cp.async.bulk (evict-first in L2, so
// the vectors stay resident), signalling a "full" mbarrier per stage; the
// consumer warp releases a stage through its "empty" mbarrier.  The matrix
// does not change during a solve, so the producer keeps cycling through the
// same pieces: the next iteration's stream overlaps the vector phases and
// grid barriers.  Pieces of a scene that has converged are no longer copied
// (the stage is signalled without data): the producer reads the per-scene
// activity the consumers publish, and may only see it late (it then copies
// data the consumers skip), never early.
// consumer warps per CTA: a template parameter (12 or 15; with the producer
// warp and 128 registers a thread, 15 fill the register file)
constexpr int kRingWarpsMax = 15;
constexpr int kRingWarpsDefault = 12;
// Steps per piece (even; a tile shape the batch autotuner picks): each
// stage holds a piece's values (90 floats per step) then its columns (10
// ints per step); kRingStages stages per consumer warp plus their
// mbarriers.
constexpr int kRingStepsDefault = 20;
__host__ __device__ constexpr int ring_stage_bytes(int ps) { return ps * 400; }
// stages per consumer warp (a third, with pieces of 8 or 10 steps so that
// it fits, let the producer's prefetch slow the update phase more than it
// sped the product)
constexpr int kRingStages = 2;
__host__ __device__ constexpr int ring_smem_bytes(int ps, int nw) {
  return nw * kRingStages * ring_stage_bytes(ps) + nw * kRingStages * 2 * 8;
}
constexpr unsigned long long kMbarSpinLimit = 1ull << 24;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false after kMbarSpinLimit polls
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  for (unsigned long long i = 0; i < kMbarSpinLimit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar,
                                         unsigned long long policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}
// w[0..2] += (a, b, c) as one vector reduction in L2 (w[3] stays zero)
__device__ __forceinline__ void red_add_v4(float4* w, float a, float b, float c) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(w), "f"(a), "f"(b), "f"(c), "f"(0.f)
               : "memory");
}

template <int NT>
__device__ __forceinline__ void named_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
}

// Shared state of one CTA of the ring kernel for the scenes it spans.
struct RingShared {
  double ws[3][kMaxLocalScenes][kRingWarpsMax];  // per-warp partials
  double res[3][kMaxLocalScenes];             // scene sums of the last reduction
  double wg[kRingWarpsMax];
  double g;                                   // grid-wide sum of the last reduction
  double rz[kMaxLocalScenes], rr[kMaxLocalScenes], eps[kMaxLocalScenes];
  double alpha[kMaxLocalScenes], beta[kMaxLocalScenes];   // step lengths of the current iteration
  double scale[kMaxLocalScenes];
  int it[kMaxLocalScenes], status[kMaxLocalScenes], maxit[kMaxLocalScenes];
  MixDesc lp[kMaxLocalScenes];                // the local scenes' arrays
  int c0[kMaxLocalScenes], c1[kMaxLocalScenes];  // CTA range of each local scene
  int lfirst[kMaxLocalScenes + 1];                // first slice of each local scene in the CTA range
  volatile unsigned char act[2][kMaxLocalScenes];  // activity by iteration parity
  unsigned char act_in[kMaxLocalScenes];      // activity given to the launch (before iteration 0)
  unsigned long long tmax;                    // profiling: the last CTA's end of the SpMV phase
  unsigned long long t_phase;                 // start of this CTA's current SpMV phase
  volatile int pub;                           // last iteration whose activity is published
  volatile int stop;
  int ok;
  unsigned epoch;                             // counting-barrier epochs passed (thread 0 only)
};

// local scene of slice sl for a warp walking its slices in increasing order
__device__ __forceinline__ int local_scene(const RingShared& sh, int sl, int& ls) {
  while (sl >= sh.lfirst[ls + 1]) ls++;
  return ls;
}

// Per-scene grid sums: CTA partials per local scene (fixed warp order) ->
// part[j][scene][cta], one grid barrier, then every CTA sums each of its
// scenes over the scene's CTA range in a fixed order (bitwise the same in
// every CTA; entries of CTAs without the scene stay zero); gval is summed
// over all CTAs.  Consumers only.
template <int NV, int NW>
__device__ __forceinline__ bool ring_sums(RingShared& sh, int L, int sc_lo, int n_sc, double gval,
                                          double* __restrict__ part, double* __restrict__ part_g, GridBarrier* gb,
                                          unsigned long long* __restrict__ stamp = nullptr,
                                          unsigned long long* __restrict__ work_ns = nullptr) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int G = gridDim.x, b = blockIdx.x;
  if (lane == 0) sh.wg[w] = gval;
  named_sync<32 * NW>();
  if (work_ns && threadIdx.x == 0) {  // this CTA's share of the phase (its own slot)
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    work_ns[b] += t - sh.t_phase;
  }
  if (stamp && threadIdx.x == 0) {  // profiling: when this CTA's warps finished the phase
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    stamp[b] = t;
  }
  if (w == 0) {
    // the CTA's partials of its scenes (staged in res, whose last values
    // were used before this phase), all stored by lane 0: its release
    // reduction at the barrier then orders them without a separate fence
    if (lane < L) {
#pragma unroll
      for (int j = 0; j < NV; j++) {
        double t = 0.0;
        for (int k = 0; k < NW; k++) t += sh.ws[j][lane][k];
        sh.res[j][lane] = t;
      }
    }
    __syncwarp();
    if (lane == 0) {
      for (int ls = 0; ls < L; ls++)
#pragma unroll
        for (int j = 0; j < NV; j++) part[((size_t)j * n_sc + sc_lo + ls) * G + b] = sh.res[j][ls];
      double t = 0.0;
      for (int k = 0; k < NW; k++) t += sh.wg[k];
      part_g[b] = t;
    }
    int ok = 1;
    if (lane == 0) ok = barrier_arrive_wait_count(gb, ++sh.epoch);
    __syncwarp();   // orders lane 0's acquire before the other lanes' partial reads
    ok = __shfl_sync(0xffffffffu, ok, 0);
    // Every lane's loads of one pass are issued before any is used (one L2
    // round trip per pass rather than one per load); each lane still adds
    // its entries in increasing CTA order, so the sums do not depend on
    // the pass structure.
    if (stamp) {  // profiling: the last CTA's end of the phase
      unsigned long long tmax = 0;
      for (int c0 = 0; c0 < G; c0 += 32 * kGridSumLoads) {
        unsigned long long v[kGridSumLoads];
#pragma unroll
        for (int q = 0; q < kGridSumLoads; q++) {
          const int c = c0 + lane + 32 * q;
          v[q] = c < G ? __ldcg(stamp + c) : 0ull;
        }
#pragma unroll
        for (int q = 0; q < kGridSumLoads; q++) tmax = max(tmax, v[q]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
      if (lane == 0) sh.tmax = tmax;
    }
    double accg = 0.0;
    for (int c0 = 0; c0 < G; c0 += 32 * kGridSumLoads) {
      double v[kGridSumLoads];
#pragma unroll
      for (int q = 0; q < kGridSumLoads; q++) {
        const int c = c0 + lane + 32 * q;
        v[q] = c < G ? __ldcg(part_g + c) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < kGridSumLoads; q++) accg += v[q];
    }
    for (int ls = 0; ls < L; ls++) {
      const int s = sc_lo + ls;
      const int c0 = sh.c0[ls], c1 = sh.c1[ls];
      // a scene that lives in this CTA alone (every local scene but the
      // first and the last can): its sums are the CTA's own partials, which
      // res holds already -- the same values the loads below would add up
      if (c0 == c1) continue;
      double acc[NV];
#pragma unroll
      for (int j = 0; j < NV; j++) acc[j] = 0.0;
      for (int cb = c0; cb <= c1; cb += 32 * kGridSumLoads) {
        double v[NV][kGridSumLoads];
#pragma unroll
        for (int j = 0; j < NV; j++) {
          const double* pp = part + ((size_t)j * n_sc + s) * G;
#pragma unroll
          for (int q = 0; q < kGridSumLoads; q++) {
            const int c = cb + lane + 32 * q;
            v[j][q] = c <= c1 ? __ldcg(pp + c) : 0.0;
          }
        }
#pragma unroll
        for (int j = 0; j < NV; j++)
#pragma unroll
          for (int q = 0; q < kGridSumLoads; q++) acc[j] += v[j][q];
      }
#pragma unroll
      for (int j = 0; j < NV; j++) {
        const double a = warp_sum(acc[j]);
        if (lane == 0) sh.res[j][ls] = a;
      }
    }
    accg = warp_sum(accg);
    if (lane == 0) {
      sh.g = accg;
      sh.ok = ok;
    }
  }
  named_sync<32 * NW>();
  return sh.ok != 0;
}

// the ring kernel's plain barrier (consumer threads; the counting barrier
// that ring_sums also uses, epochs in sh)
template <int NT>
__device__ __forceinline__ bool grid_barrier_named(GridBarrier* gb, RingShared& sh) {
  __shared__ int okb_s;
  named_sync<NT>();
  if (threadIdx.x == 0) okb_s = barrier_arrive_wait_count(gb, ++sh.epoch);
  named_sync<NT>();
  return okb_s != 0;
}

// Inner FP32 PCG of every scene of a sliced system, one cooperative launch
// of 32 (NW + 1) threads per CTA: scene s solves A32 d = rhs_scale * r64 from d = 0
// until ||r_inner|| <= inner_tol ||r_0|| or max_iter, each scene with its own
// step lengths; the loop runs while any scene is active.  Slices are
// numbered through the scenes (scene s owns [slice0, slice0 + ns)); every
// scene's arrays are its own (MixDesc).  Lane l < 30 of a consumer warp owns
// slice element 30*slice + l, i.e. component l%3 of slice row l/3 (lanes
// 30, 31 shadow lane 29 and store nothing).  Dot products accumulate in
// compensated FP32 per lane and are summed in FP64.
template <int PS, int NW>
__global__ void __launch_bounds__(32 * (NW + 1), 1) pcg32_ring_kernel(
    int n_sc, const int* __restrict__ cta_first, const int* __restrict__ cta_sc_lo, const int* __restrict__ sc_cta,
    const int* __restrict__ sc_slice, const MixDesc* __restrict__ desc, RingScene* __restrict__ ring, int pkind,
    double* __restrict__ part, GridBarrier* gb, unsigned long long* __restrict__ prof,
    unsigned long long* __restrict__ cta_ns) {
  constexpr int ST = kRingStages;
  extern __shared__ __align__(128) unsigned char ring_smem[];
  unsigned long long* full = reinterpret_cast<unsigned long long*>(ring_smem + NW * ST * ring_stage_bytes(PS));
  unsigned long long* empty = full + ST * NW;
  __shared__ RingShared sh;
  const int G = gridDim.x;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int sfirst = cta_first[blockIdx.x], send = cta_first[blockIdx.x + 1];
  const int sc_lo = cta_sc_lo[blockIdx.x];
  int L = 0;
  if (send > sfirst) {
    int hi = n_sc;  // scene of slice send - 1: largest s with sc_slice[s] <= send - 1
    int lo = sc_lo;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (sc_slice[mid] <= send - 1) lo = mid;
      else hi = mid;
    }
    L = lo - sc_lo + 1;
  }
  if (threadIdx.x == 0) {
    sh.stop = 0;
    sh.pub = -1;
    sh.epoch = 0;
  }
  if (threadIdx.x < ST * NW) {
    mbar_init(full + threadIdx.x, 1);
    mbar_init(empty + threadIdx.x, 1);
  }
  if (threadIdx.x < L) {
    const int s = sc_lo + threadIdx.x;
    sh.scale[threadIdx.x] = ring[s].rhs_scale;
    sh.eps[threadIdx.x] = ring[s].itol2;  // relative until the first reduction
    sh.maxit[threadIdx.x] = ring[s].max_iter;
    sh.act[0][threadIdx.x] = (unsigned char)(ring[s].active0 != 0);
    sh.act_in[threadIdx.x] = (unsigned char)(ring[s].active0 != 0);
    sh.lp[threadIdx.x] = desc[s];
    sh.c0[threadIdx.x] = sc_cta[2 * s];
    sh.c1[threadIdx.x] = sc_cta[2 * s + 1];
    sh.lfirst[threadIdx.x] = threadIdx.x == 0 ? sfirst : sc_slice[s];
  }
  if (threadIdx.x == 0) sh.lfirst[L] = send;
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();

  if (w == NW) {
    // ---------------- producer: lane pw feeds consumer warp pw
    const int pw = lane;
    if (pw >= NW || sfirst + pw >= send) return;
    unsigned long long policy;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
    unsigned pc = 0;  // pieces issued
    int kit = 0;      // iteration the pieces belong to
    bool ok = true;
    while (ok && !sh.stop) {  // (when every scene is done, no piece is issued: poll stop here)
      // never more than one iteration ahead of the consumers: the activity of
      // iteration kit - 1 must be published before pass kit (a warp whose
      // scenes have all converged issues nothing and would otherwise run
      // ahead and read another iteration's activity)
      if (kit > 0) {
        unsigned long long spins = 0;
        while (sh.pub < kit - 1 && !sh.stop && ++spins < kMbarSpinLimit) {
        }
        if (sh.pub < kit - 1) break;
      }
      int ls = 0;
      for (int sl = sfirst + pw; sl < send && ok; sl += NW) {
        local_scene(sh, sl, ls);
        // pieces of iteration kit exist for the scenes active in iteration
        // kit - 1 (published before the consumers start iteration kit - 1,
        // hence before the producer reaches iteration kit): consumers apply
        // the same rule, so a converged scene costs nothing after one pass
        __threadfence_block();
        if (!(kit == 0 ? sh.act_in[ls] : sh.act[(kit - 1) & 1][ls])) continue;
        bool copy = true;
        if (sh.pub >= kit) {
          __threadfence_block();
          copy = sh.act[kit & 1][ls] != 0;
        }
        const MixDesc& P = sh.lp[ls];
        const int lsl = sl - P.slice0;
        const int k1 = P.soff[lsl + 1];
        for (int k = P.soff[lsl]; k < k1; k += PS) {
          const int n = min(PS, k1 - k);
          const int j = (int)(pc % ST);
          const unsigned par = ((pc / ST) & 1) ^ 1;
          bool got = false;
          for (unsigned long long i = 0; i < kMbarSpinLimit; i++) {
            if (mbar_try_wait(empty + ST * pw + j, par)) { got = true; break; }
            if (sh.stop) break;
          }
          if (!got) { ok = false; break; }
          if (copy) {
            unsigned char* st = ring_smem + (size_t)(ST * pw + j) * ring_stage_bytes(PS);
            mbar_expect_tx(full + ST * pw + j, (unsigned)n * 400u);
            bulk_g2s(st, P.sval + (size_t)k * 90, (unsigned)n * 360u, full + ST * pw + j, policy);
            bulk_g2s(st + PS * 360, P.scol + (size_t)k * kSliceRows, (unsigned)n * 40u, full + ST * pw + j,
                     policy);
          } else {
            mbar_arrive(full + ST * pw + j);
          }
          pc++;
        }
      }
      kit++;
    }
    // drain: the last arming of each stage must complete before the CTA exits
    for (unsigned u = 0; u < (unsigned)ST && u < pc; u++) {
      const unsigned last = pc - 1 - u;
      mbar_wait(full + ST * pw + (last % ST), (last / ST) & 1);
    }
    return;
  }

  // ---------------- consumers
  // Chronopoulos-Gear PCG: one grid-wide sum per iteration.  Roles of the
  // FP32 vectors: u = M^-1 r is the one the SpMV gathers (float4 layout),
  // w = A u, p and s = A p are the directions, d the solution.  Iteration k:
  //   w = A u, (w, u)  -> one sum with the (r, u), (r, r) of the last update
  //   k = 0: alpha = (r,u) / (w,u), beta = 0
  //   k > 0: beta = (r,u) / (r,u)_prev, alpha = (r,u) / ((w,u) - beta (r,u) / alpha_prev)
  //   p = u + beta p, s = w + beta s, d += alpha p, r -= alpha s, u = M^-1 r,
  //   partial (r, u), (r, r); grid barrier (u complete for the next gathers)
  double* part_3 = part;                                    // [3][n_sc][G]
  double* part_g = part + (size_t)3 * n_sc * G;             // [G]
  const bool act_l = lane < 30;
  const int ln = act_l ? lane : 29;
  const int t = ln / 3, rsub = ln - 3 * t, lbase = 3 * t;
  unsigned pc = 0;  // pieces consumed
  bool alive = true;

  // a warp's slices of local scene ls: first_slice(ls), + NW, ... < lfirst[ls + 1]
  auto first_slice = [&](int ls) {
    const int dlt = sh.lfirst[ls] - sfirst - w;
    return dlt <= 0 ? sfirst + w : sfirst + w + ((dlt + NW - 1) / NW) * NW;
  };
  auto zero_ws = [&](int nv) {
    if (lane < L)
      for (int j = 0; j < nv; j++) sh.ws[j][lane][w] = 0.0;
    __syncwarp();
  };
  auto flush = [&](int j, int ls, const Comp& c) {
    const double tv = comp_warp_sum(c);
    if (lane == 0) sh.ws[j][ls][w] = tv;
  };
  // the scene's vectors, indexed by the scene-local slice
  struct Vecs {
    float4* u4;
    float *uf, *d, *r, *p, *w, *pinv, *s;
    float4* w4;   // lower storage: w = A u as float4 rows, accumulated by reductions
    int s0;
  };
  auto vecs = [&](int ls) {
    const MixDesc& P = sh.lp[ls];
    Vecs v;
    const size_t ns = (size_t)P.ns;
    v.u4 = reinterpret_cast<float4*>(P.v32);
    v.uf = P.v32;
    v.d = P.v32 + 40 * ns;
    v.r = v.d + 30 * ns;
    v.p = v.r + 30 * ns;
    v.w = v.p + 30 * ns;
    v.pinv = v.w + 30 * ns;
    v.s = v.pinv + 90 * ns;
    v.w4 = reinterpret_cast<float4*>(v.s + 30 * ns);
    v.s0 = P.slice0;
    return v;
  };

  // init: d = p = s = 0, r = rhs, u = M^-1 r; partials (r, u), (r, r)
  zero_ws(3);
  for (int ls = 0; ls < L; ls++) {
    const bool a0 = sh.act[0][ls] != 0;
    const double scale = sh.scale[ls];
    const Vecs V = vecs(ls);
    const int* __restrict__ perm = sh.lp[ls].sperm;
    const double* __restrict__ r64 = sh.lp[ls].r64;
    Comp cru{0.f, 0.f}, crr{0.f, 0.f};
    for (int sl = first_slice(ls); sl < sh.lfirst[ls + 1]; sl += NW) {
      const int lsl = sl - V.s0;
      const int rs = lsl * kSliceRows + t;
      const int row = perm[rs];
      const float rl = (a0 && row >= 0) ? (float)(r64[3 * (size_t)row + rsub] * scale) : 0.f;
      const float r0 = __shfl_sync(0xffffffffu, rl, lbase);
      const float r1 = __shfl_sync(0xffffffffu, rl, lbase + 1);
      const float r2 = __shfl_sync(0xffffffffu, rl, lbase + 2);
      float ul = rl;
      if (pkind == OD_PRECOND_JACOBI) ul = V.pinv[(size_t)30 * lsl + ln] * rl;
      else if (pkind == OD_PRECOND_BLOCK_JACOBI) {
        const float* m = V.pinv + (size_t)90 * lsl + ln;
        ul = fmaf(m[0], r0, fmaf(m[30], r1, m[60] * r2));
      }
      if (act_l) {
        const size_t i = (size_t)30 * lsl + lane;
        V.r[i] = rl;
        V.d[i] = 0.f;
        V.p[i] = 0.f;
        V.s[i] = 0.f;
        V.uf[4 * (size_t)rs + rsub] = ul;
        if (sh.lp[ls].lower) reinterpret_cast<float*>(V.w4)[4 * (size_t)rs + rsub] = 0.f;
        comp_add_prod(cru, rl, ul);
        comp_add_prod(crr, rl, rl);
      }
    }
    flush(1, ls, cru);
    flush(2, ls, crr);
  }
  if (w == 0 && lane < L) {
    sh.it[lane] = 0;
    sh.status[lane] = OD_OK;
  }
  __threadfence_block();
  if (threadIdx.x == 0) sh.pub = 0;   // act[0] (= the launch's activity) is final
  // u complete everywhere before the first gathers
  if (!grid_barrier_named<(32 * NW)>(gb, sh)) alive = false;

  // profiling (prof != nullptr): CTA 0 times each SpMV + sum phase up to the
  // end of its grid-wide sum, i.e. including the slowest CTA
  const bool timer = prof && blockIdx.x == 0 && threadIdx.x == 0;
  for (int k = 0; alive; k++) {
    const int kp = k & 1;
    unsigned long long t_a = 0;
    if (timer) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_a));
    if (cta_ns && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(sh.t_phase));
    // ---- w = A u (pieces from the ring), (w, u)
    {
      for (int ls = 0; ls < L && alive; ls++) {
        if (!(k == 0 ? sh.act_in[ls] : sh.act[kp ^ 1][ls])) continue;  // no pieces this iteration
        const bool on = sh.act[kp][ls] != 0;
        const bool lower = sh.lp[ls].lower != 0;   // scene-uniform
        const Vecs V = vecs(ls);
        const int* __restrict__ soff = sh.lp[ls].soff;
        Comp cwu{0.f, 0.f};
        // a slice's step range and the u of its own block row (the
        // transposed products and (w, u)) are loaded while the warp's
        // previous slice is processed: the loads cannot move across the
        // mbarrier waits, so each would otherwise be a memory round trip
        // of its own per slice
        const int sl_end = sh.lfirst[ls + 1];
        int ka = 0, kb = 0;
        float4 un = make_float4(0.f, 0.f, 0.f, 0.f);
        auto fetch = [&](int sl) {
          const int l = sl - V.s0;
          ka = soff[l];
          kb = soff[l + 1];
          if (on) un = V.u4[(size_t)l * kSliceRows + t];
        };
        if (first_slice(ls) < sl_end) fetch(first_slice(ls));
        for (int sl = first_slice(ls); sl < sl_end && alive; sl += NW) {
          const int lsl = sl - V.s0;
          const int k0 = ka, k1 = kb;
          const float4 uo = un;
          if (sl + NW < sl_end) fetch(sl + NW);
          float y0 = 0.f, y1 = 0.f, y2 = 0.f;  // partial rows 0, 1, 2 of block row t
          for (int kk = k0; kk < k1; kk += PS) {
            const int n = min(PS, k1 - kk);
            const int j = (int)(pc % ST);
            if (!__all_sync(0xffffffffu, mbar_wait(full + ST * w + j, (pc / ST) & 1))) {
              atomicExch(&gb->timeout, 1);
              alive = false;
              break;
            }
            if (on) {
              const unsigned char* stg = ring_smem + (size_t)(ST * w + j) * ring_stage_bytes(PS);
              const float* sv = reinterpret_cast<const float*>(stg);
              const int* scol = reinterpret_cast<const int*>(stg + PS * 360);
              // lane (t, rsub) takes steps rsub, rsub + 3, ... of the piece
              // for all three rows of block row t: every gather is issued first
              constexpr int kPer = (PS + 2) / 3;
              float4 x[kPer];
#pragma unroll
              for (int u = 0; u < kPer; u++) {
                const int st = rsub + 3 * u;
                x[u] = st < n ? V.u4[scol[st * kSliceRows + t]] : make_float4(0.f, 0.f, 0.f, 0.f);
              }
#pragma unroll
              for (int u = 0; u < kPer; u++) {
                const int st = rsub + 3 * u;
                if (st < n) {
                  const float* a = sv + st * 90 + lbase;  // a[30 j + r] = A[r][j]
                  y0 = fmaf(a[0], x[u].x, y0);
                  y0 = fmaf(a[30], x[u].y, y0);
                  y0 = fmaf(a[60], x[u].z, y0);
                  y1 = fmaf(a[1], x[u].x, y1);
                  y1 = fmaf(a[31], x[u].y, y1);
                  y1 = fmaf(a[61], x[u].z, y1);
                  y2 = fmaf(a[2], x[u].x, y2);
                  y2 = fmaf(a[32], x[u].y, y2);
                  y2 = fmaf(a[62], x[u].z, y2);
                  if (lower && act_l) {
                    // the block's transpose: B^T u_t into the column's row of w
                    const float t0 = fmaf(a[0], uo.x, fmaf(a[1], uo.y, a[2] * uo.z));
                    const float t1 = fmaf(a[30], uo.x, fmaf(a[31], uo.y, a[32] * uo.z));
                    const float t2 = fmaf(a[60], uo.x, fmaf(a[61], uo.y, a[62] * uo.z));
                    red_add_v4(V.w4 + scol[st * kSliceRows + t], t0, t1, t2);
                  }
                }
              }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + ST * w + j);
            pc++;
          }
          if (on) {
            // row rsub of block row t: own partial + the two neighbours' (fixed order)
            const int l1 = lbase + (rsub == 2 ? 0 : rsub + 1), l2 = lbase + (rsub == 0 ? 2 : rsub - 1);
            const float a0 = __shfl_sync(0xffffffffu, y0, l1), b0 = __shfl_sync(0xffffffffu, y0, l2);
            const float a1 = __shfl_sync(0xffffffffu, y1, l1), b1 = __shfl_sync(0xffffffffu, y1, l2);
            const float a2 = __shfl_sync(0xffffffffu, y2, l1), b2 = __shfl_sync(0xffffffffu, y2, l2);
            const float own = rsub == 0 ? y0 : (rsub == 1 ? y1 : y2);
            const float na = rsub == 0 ? a0 : (rsub == 1 ? a1 : a2);
            const float nb = rsub == 0 ? b0 : (rsub == 1 ? b1 : b2);
            const float y = (own + na) + nb;
            const float uown = rsub == 0 ? uo.x : (rsub == 1 ? uo.y : uo.z);   // u of row rsub of block row t
            if (lower) {
              // w of the own row takes the gathered half by one reduction;
              // (w, u) = 2 sum_rows u . (gathered half) (the scattered half
              // carries the same products transposed)
              const float yb = __shfl_sync(0xffffffffu, y, lbase + 1);
              const float yc = __shfl_sync(0xffffffffu, y, lbase + 2);
              if (act_l) {
                comp_add_prod(cwu, 2.f * uown, y);
                if (rsub == 0) red_add_v4(V.w4 + (size_t)lsl * kSliceRows + t, y, yb, yc);
              }
            } else if (act_l) {
              V.w[(size_t)30 * lsl + lane] = y;
              comp_add_prod(cwu, uown, y);
            }
          }
        }
        if (on) flush(0, ls, cwu);
      }
      // active scenes of this CTA at iteration k (grid-wide sum: 0 ends the loop)
      double na = 0.0;
      if (w == 0 && lane == 0)
        for (int ls = 0; ls < L; ls++) na += sh.act[kp][ls] ? 1.0 : 0.0;
      if (!ring_sums<3, NW>(sh, L, sc_lo, n_sc, na, part_3, part_g, gb, prof ? prof + 3 : nullptr, cta_ns))
        alive = false;
    }
    if (!alive || sh.g == 0.0) break;
    if (timer) {
      unsigned long long t_b;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_b));
      prof[0] += t_b - t_a;
      prof[1] += 1;
      prof[2] += sh.tmax - t_a;  // up to the last CTA's end of the SpMV work
    }
    // step lengths and the activity of iteration k + 1 (which also gates
    // this iteration's update)
    if (w == 0 && lane < L) {
      const int ls = lane;
      unsigned char na = 0;
      if (sh.act[kp][ls]) {
        const double wu = sh.res[0][ls], ru = sh.res[1][ls], rr = sh.res[2][ls];
        double alpha, beta;
        if (k == 0) {
          sh.eps[ls] = rr * sh.eps[ls];   // relative to the initial residual
          beta = 0.0;
          alpha = ru / wu;
        } else {
          beta = ru / sh.rz[ls];
          alpha = ru / (wu - beta * ru / sh.alpha[ls]);
        }
        sh.rz[ls] = ru;
        sh.rr[ls] = rr;
        sh.alpha[ls] = alpha;
        sh.beta[ls] = beta;
        if (!isfinite(rr) || !isfinite(alpha) || !isfinite(beta)) sh.status[ls] = OD_ERR_NAN;
        na = (unsigned char)(sh.status[ls] == OD_OK && rr > sh.eps[ls] && sh.it[ls] < sh.maxit[ls]);
        if (na) sh.it[ls]++;
      }
      sh.act[kp ^ 1][ls] = na;
    }
    __threadfence_block();
    named_sync<(32 * NW)>();
    if (threadIdx.x == 0) sh.pub = k + 1;
    // ---- p = u + beta p, s = w + beta s, d += alpha p, r -= alpha s,
    // u = M^-1 r, (r, u), (r, r): kUB slices per batch, all loads of a batch
    // issued before any use
    zero_ws(3);
    for (int ls = 0; ls < L; ls++) {
      if (!sh.act[kp ^ 1][ls]) continue;  // warp-uniform; the partials stay zero
      constexpr int kUB = PS <= 12 ? 6 : 4;   // slices per batch (registers allow 6 at the smaller pieces)
      const int hi = sh.lfirst[ls + 1];
      const Vecs V = vecs(ls);
      const bool lower = sh.lp[ls].lower != 0;
      float* w4f = reinterpret_cast<float*>(V.w4);
      const float alpha = (float)sh.alpha[ls], beta = (float)sh.beta[ls];
      Comp cru{0.f, 0.f}, crr{0.f, 0.f};
      for (int sl0 = first_slice(ls); sl0 < hi; sl0 += kUB * NW) {
        float dv[kUB], pv[kUB], sv[kUB], uv[kUB], wv[kUB], rv[kUB], m0[kUB], m1[kUB], m2[kUB];
#pragma unroll
        for (int u = 0; u < kUB; u++) {
          const int sl = sl0 + u * NW;
          if (sl < hi) {
            const int lsl = sl - V.s0;
            const size_t i = (size_t)30 * lsl + ln;
            dv[u] = V.d[i];
            pv[u] = V.p[i];
            sv[u] = V.s[i];
            uv[u] = V.uf[4 * (size_t)(lsl * kSliceRows + t) + rsub];
            // lower storage: w was summed by reductions in L2 (read there)
            wv[u] = lower ? __ldcg(w4f + 4 * (size_t)(lsl * kSliceRows + t) + rsub) : V.w[i];
            rv[u] = V.r[i];
            if (pkind == OD_PRECOND_BLOCK_JACOBI) {
              const float* m = V.pinv + (size_t)90 * lsl + ln;
              m0[u] = m[0];
              m1[u] = m[30];
              m2[u] = m[60];
            } else if (pkind == OD_PRECOND_JACOBI) {
              m0[u] = V.pinv[(size_t)30 * lsl + ln];
            }
          }
        }
#pragma unroll
        for (int u = 0; u < kUB; u++) {
          const int sl = sl0 + u * NW;
          if (sl < hi) {  // warp-uniform
            const int lsl = sl - V.s0;
            const size_t i = (size_t)30 * lsl + ln;
            const float pn = fmaf(beta, pv[u], uv[u]);
            const float sn = fmaf(beta, sv[u], wv[u]);
            const float rl = act_l ? fmaf(-alpha, sn, rv[u]) : 0.f;
            const float r0 = __shfl_sync(0xffffffffu, rl, lbase);
            const float r1 = __shfl_sync(0xffffffffu, rl, lbase + 1);
            const float r2 = __shfl_sync(0xffffffffu, rl, lbase + 2);
            float ul = rl;
            if (pkind == OD_PRECOND_BLOCK_JACOBI) ul = fmaf(m0[u], r0, fmaf(m1[u], r1, m2[u] * r2));
            else if (pkind == OD_PRECOND_JACOBI) ul = m0[u] * rl;
            if (act_l) {
              V.p[i] = pn;
              V.s[i] = sn;
              V.d[i] = fmaf(alpha, pn, dv[u]);
              V.r[i] = rl;
              V.uf[4 * (size_t)(lsl * kSliceRows + t) + rsub] = ul;
              if (lower) w4f[4 * (size_t)(lsl * kSliceRows + t) + rsub] = 0.f;   // for the next SpMV phase
              comp_add_prod(cru, rl, ul);
              comp_add_prod(crr, rl, rl);
            }
          }
        }
      }
      flush(1, ls, cru);
      flush(2, ls, crr);
    }
    // u complete everywhere before the next gathers (also keeps this
    // iteration's sums from being overwritten before every CTA read them)
    if (!grid_barrier_named<(32 * NW)>(gb, sh)) { alive = false; break; }
  }
  named_sync<(32 * NW)>();
  if (threadIdx.x == 0) sh.stop = 1;
  if (alive && w == 0 && lane < L) {
    const int s = sc_lo + lane;
    if (sc_cta[2 * s] == (int)blockIdx.x) {
      ring[s].iters = sh.it[lane];
      ring[s].status = sh.status[lane];
      ring[s].rr = sh.rr[lane];
    }
  }
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

// IC(0) factorisation in one cooperative launch: rows listed by forward
// level, one warp per row.  The warp first reads every value of other rows
// the row needs -- for each off-diagonal entry (i, j) the L_jk paired with
// the row's own L_ik (k < j), and L_jj -- into shared memory, each waited
// for (bounded) until it is no longer the pending pattern.  Then it forms
// the row right-looking: lane q % 32 owns entry q and its running value
// (A_ij, or (1 + shift) A_ii); when entry k is formed,
//   L_ij = running_ij / L_jj,   L_ii = sqrt(running_ii)  (breakdown test of ic0_factor_level)
// it is published (relaxed store; the value is its own ready flag) and
// broadcast, and every later entry paired with it subtracts L_ik L_jk, the
// diagonal L_ik^2 -- the subtractions of each entry in ascending k, as the
// sequential factorisation makes them.  A step of the row is one multiply,
// one shuffle and one FMA.
constexpr int kIcfThreads = 128;
constexpr int kIcfWarps = kIcfThreads / 32;
constexpr unsigned kIcfSpinLimit = 1u << 21;

constexpr unsigned kIcfPollBurst = 1024;

// warp-cooperative bounded read of one value per lane (p null: none): one
// lane polls the first value still pending in the warp, then every lane
// re-reads its own once, so waiting warps send one poll at a time; called
// by all 32 lanes
__device__ __forceinline__ double icf_warp_read(const double* p, int* err) {
  const int lane = threadIdx.x & 31;
  unsigned long long v = p ? ld_relaxed_u64(p) : 0ull;
  for (unsigned round = 1;; round++) {
    const bool pend = p && v == kPending;
    const unsigned ball = __ballot_sync(0xffffffffu, pend);
    if (!ball) break;
    int stop = 0;
    if (lane == __ffs(ball) - 1) {
      unsigned k = 0;
      while (ld_relaxed_u64(p) == kPending && ++k < kIcfPollBurst) {
      }
      stop = round >= kIcfSpinLimit / kIcfPollBurst || *(volatile int*)err;
      if (round >= kIcfSpinLimit / kIcfPollBurst) atomicOr(err, 1);
    }
    if (__any_sync(0xffffffffu, stop)) {
      if (pend) v = 0ull;
      break;
    }
    if (pend) v = ld_relaxed_u64(p);
  }
  return __longlong_as_double((long long)v);
}

constexpr int kIcfSlots = 4;   // entries per lane: rows of up to 128 entries
constexpr int kIcfBatch = 8;   // paired values per lane read before one cooperative wait

// warp-cooperative bounded read of up to kIcfBatch values per lane (null:
// none), all loads issued before the first wait; called by all 32 lanes
__device__ __forceinline__ void icf_warp_read_batch(const double* const (&p)[kIcfBatch], double (&out)[kIcfBatch],
                                                    int* err) {
  const int lane = threadIdx.x & 31;
  unsigned long long v[kIcfBatch];
#pragma unroll
  for (int u = 0; u < kIcfBatch; u++) v[u] = p[u] ? ld_relaxed_u64(p[u]) : 0ull;
  for (unsigned round = 1;; round++) {
    int pu = -1;
#pragma unroll
    for (int u = kIcfBatch - 1; u >= 0; u--)
      if (p[u] && v[u] == kPending) pu = u;
    const unsigned ball = __ballot_sync(0xffffffffu, pu >= 0);
    if (!ball) break;
    int stop = 0;
    if (lane == __ffs(ball) - 1) {
      const double* q = nullptr;
#pragma unroll
      for (int u = 0; u < kIcfBatch; u++)
        if (u == pu) q = p[u];
      unsigned k = 0;
      while (ld_relaxed_u64(q) == kPending && ++k < kIcfPollBurst) {
      }
      stop = round >= kIcfSpinLimit / kIcfPollBurst || *(volatile int*)err;
      if (round >= kIcfSpinLimit / kIcfPollBurst) atomicOr(err, 1);
    }
    if (__any_sync(0xffffffffu, stop)) {
#pragma unroll
      for (int u = 0; u < kIcfBatch; u++)
        if (v[u] == kPending) v[u] = 0ull;
      break;
    }
#pragma unroll
    for (int u = 0; u < kIcfBatch; u++)
      if (p[u] && v[u] == kPending) v[u] = ld_relaxed_u64(p[u]);
  }
#pragma unroll
  for (int u = 0; u < kIcfBatch; u++) out[u] = __longlong_as_double((long long)v[u]);
}

__global__ void __launch_bounds__(kIcfThreads) ic0_factor_coop_kernel(
    int n, const int* __restrict__ rows, const int* __restrict__ rp, const int* __restrict__ ci,
    const int* __restrict__ src, const double* __restrict__ A, const int* __restrict__ pp,
    const int* __restrict__ pa, const int* __restrict__ pb, double* L, double shift, int maxrow, int maxpairs,
    int* __restrict__ bad, int* __restrict__ err) {
  extern __shared__ double icf_s[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* aval = icf_s + (size_t)wib * (2 * maxrow + maxpairs);
  double* dval = aval + maxrow;
  double* pv = dval + maxrow;
  // the pairs' row positions, staged beside the values (ints after all
  // the warps' doubles)
  int* pa_s = reinterpret_cast<int*>(icf_s + (size_t)kIcfWarps * (2 * maxrow + maxpairs)) + (size_t)wib * maxpairs;
  const int W = gridDim.x * kIcfWarps;
  for (int t = blockIdx.x * kIcfWarps + wib; t < n; t += W) {
    const int i = rows[t];
    const int bi = rp[i], m = rp[i + 1] - bi;
    const int p0 = pp[bi], np = pp[bi + m] - p0;
    __syncwarp();
    // 1) the row's A values, the other rows' diagonals and paired values
    for (int q0 = 0; q0 < m; q0 += 32) {
      const int q = q0 + lane;
      const double* dp = nullptr;
      if (q < m) {
        aval[q] = A[src[bi + q]];
        const int j = ci[bi + q];
        if (j < i) dp = L + rp[j + 1] - 1;
      }
      const double d = icf_warp_read(dp, err);
      if (q < m) dval[q] = dp ? d : 1.0;
    }
    for (int b0 = 0; b0 < np; b0 += 32 * kIcfBatch) {
      const double* ptrs[kIcfBatch];
      double vals[kIcfBatch];
#pragma unroll
      for (int u = 0; u < kIcfBatch; u++) {
        const int p = b0 + u * 32 + lane;
        ptrs[u] = p < np ? L + pb[p0 + p] : nullptr;
      }
      icf_warp_read_batch(ptrs, vals, err);
#pragma unroll
      for (int u = 0; u < kIcfBatch; u++) {
        const int p = b0 + u * 32 + lane;
        if (p < np) {
          pv[p] = vals[u];
          pa_s[p] = pa[p0 + p];
        }
      }
    }
    __syncwarp();
    // 2) right-looking over the row's entries
    double sv[kIcfSlots], rinv[kIcfSlots];
    int cur[kIcfSlots], cend[kIcfSlots], nxt[kIcfSlots];
#pragma unroll
    for (int r = 0; r < kIcfSlots; r++) {
      const int q = lane + 32 * r;
      sv[r] = 0.0;
      rinv[r] = 0.0;
      cur[r] = cend[r] = 0;
      nxt[r] = -1;
      if (q < m) {
        sv[r] = q < m - 1 ? aval[q] : aval[q] * (1.0 + shift);
        rinv[r] = 1.0 / dval[q];
        cur[r] = pp[bi + q] - p0;
        cend[r] = pp[bi + q + 1] - p0;
        nxt[r] = cur[r] < cend[r] ? pa_s[cur[r]] : -1;
      }
    }
    for (int k = 0; k < m; k++) {
      const int ko = k & 31, rk = k >> 5;
      double v = 0.0;
      if (lane == ko) {
        double s = 0.0, rv = 0.0;
#pragma unroll
        for (int r = 0; r < kIcfSlots; r++)
          if (r == rk) {
            s = sv[r];
            rv = rinv[r];
          }
        if (k < m - 1) {
          v = s * rv;
        } else {
          const double d = aval[k] * (1.0 + shift);
          if (!(s > 1e-12 * d)) {
            *bad = 1;
            s = d > 0.0 ? d : 1.0;
          }
          v = sqrt(s);
        }
        st_relaxed_f64(L + bi + k, v);
      }
      v = __shfl_sync(0xffffffffu, v, ko);
#pragma unroll
      for (int r = 0; r < kIcfSlots; r++) {
        const int q = lane + 32 * r;
        if (q > k && q < m) {
          if (q == m - 1) {
            sv[r] -= v * v;
          } else if (nxt[r] == k) {
            sv[r] -= v * pv[cur[r]];
            cur[r]++;
            nxt[r] = cur[r] < cend[r] ? pa_s[cur[r]] : -1;
          }
        }
      }
    }
  }
}

// the IC(0) factor (rows, diagonal last) split for the one-launch sweeps:
// strictly lower rows, values in transposed order, reciprocal diagonal
__global__ void ic0_split_kernel(int n, const int* __restrict__ rp, const int* __restrict__ frp,
                                 const double* __restrict__ L, int nt, const int* __restrict__ tpos,
                                 double* __restrict__ fval, double* __restrict__ bval, double* __restrict__ dval) {
  const int stride = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += stride) bval[t] = L[tpos[t]];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int a = rp[i], e = rp[i + 1] - 1, o = frp[i];
    for (int q = a; q < e; q++) fval[o + q - a] = L[q];
    dval[i] = 1.0 / L[e];   // the apply multiplies by 1 / L_ii
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
  if (v3 && !s->has_damping) v3 = nullptr;
  s->lo.v1 = v1; s->lo.c1 = c1;
  s->lo.v2 = v2; s->lo.c2 = c2;
  s->lo.v3 = v3; s->lo.c3 = c3;
  OD_KL(s);
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
  // drop a second / third source that is absent or known to be zero
  if (v3 && !s->has_damping) v3 = nullptr;
  if (v2 && v2 == s->Dm && !s->has_damping) { v2 = v3; c2 = c3; x2 = x3; v3 = nullptr; }
  const int g = nblk(nb, (kThreads / 32) * 10);
  OD_KL(s);
  if (v3)
    spmv_lower_kernel<3><<<g, kThreads, 0, s->ctx->stream>>>(nb, s->bsr.row_ptr, s->bsr.col, s->bsr.desc_kind,
                                                              s->bsr.desc_off, s->bsr.gen, v1, c1, x1, v2, c2, x2, v3,
                                                              c3, x3, y, accumulate ? 1 : 0);
  else if (v2)
    spmv_lower_kernel<2><<<g, kThreads, 0, s->ctx->stream>>>(nb, s->bsr.row_ptr, s->bsr.col, s->bsr.desc_kind,
                                                              s->bsr.desc_off, s->bsr.gen, v1, c1, x1, v2, c2, x2,
                                                              nullptr, 0.0, nullptr, y, accumulate ? 1 : 0);
  else
    spmv_lower_kernel<1><<<g, kThreads, 0, s->ctx->stream>>>(nb, s->bsr.row_ptr, s->bsr.col, s->bsr.desc_kind,
                                                              s->bsr.desc_off, s->bsr.gen, v1, c1, x1, nullptr, 0.0,
                                                              nullptr, nullptr, 0.0, nullptr, y, accumulate ? 1 : 0);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status launch_expand_batch(Ctx* ctx, int n_sc, const SceneDev* sd, const TileDir& dir) {
  if (dir.tiles <= 0) return OD_OK;
  ctx->launches++;
  expand_batch_kernel<<<dir.tiles, kThreads, 0, ctx->stream>>>(n_sc, dir.prefix, sd);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status launch_spmv_lower_batch(Ctx* ctx, int n_sc, const SceneDev* sd, const TileDir& dir) {
  if (dir.tiles <= 0) return OD_OK;
  ctx->launches++;
  spmv_lower_batch_kernel<<<dir.tiles, kThreads, 0, ctx->stream>>>(n_sc, dir.prefix, sd);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status launch_spmv_full(Scene* s, const double* x, double* y) {
  const int nb = s->bsr.nb;
  if (nb == 0) return OD_OK;
  OD_KL(s);
  spmv_full_kernel<double><<<nblk(nb, kWarpRows), kThreads, 0, s->ctx->stream>>>(nb, s->bsr.row_ptr, s->bsr.col,
                                                                                    s->A64, x, y);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

// IC(0) structure: scalar CSR of the padded lower pattern of the full BSR
// (columns sorted, diagonal last), level sets, and the transposed index.
// Greedy colouring of the block graph (block rows coupled by a stored
// block), blocks visited in index order, each taking the lowest colour no
// coloured neighbour has; order[] lists the blocks by colour, then index.
// Returns the number of colours.  The oracle's IC(0) orders the same way.
static int ic0_colour_order(int nb, const std::vector<int>& rp, const std::vector<int>& col, std::vector<int>& order,
                            std::vector<int>& start_out) {
  std::vector<int> colour(nb, -1), mark;
  int nc = 0;
  for (int b = 0; b < nb; b++) {
    for (int k = rp[b]; k < rp[b + 1]; k++) {
      const int c = colour[col[k]];
      if (c >= 0) {
        if ((int)mark.size() <= c) mark.resize(c + 1, -1);
        mark[c] = b;
      }
    }
    int c = 0;
    while (c < (int)mark.size() && mark[c] == b) c++;
    colour[b] = c;
    nc = std::max(nc, c + 1);
  }
  std::vector<int> start(nc + 1, 0);
  for (int b = 0; b < nb; b++) start[colour[b] + 1]++;
  for (int c = 0; c < nc; c++) start[c + 1] += start[c];
  start_out.assign(start.begin(), start.end());
  order.assign(nb, 0);
  for (int b = 0; b < nb; b++) order[start[colour[b]]++] = b;
  return nc;
}

static od_status ic0_build(Scene* s) {
  Pcg& P = s->pcg;
  if (P.ic_rp) return OD_OK;
  // host copies of the BSR structure
  const int nb = s->bsr.nb;
  std::vector<int> rp(nb + 1), col(s->bsr.nnzb);
  OD_CUDA(cudaMemcpy(rp.data(), s->bsr.row_ptr, sizeof(int) * (nb + 1), cudaMemcpyDeviceToHost));
  OD_CUDA(cudaMemcpy(col.data(), s->bsr.col, sizeof(int) * s->bsr.nnzb, cudaMemcpyDeviceToHost));
  const int n = 3 * nb;
  // Node order of the factor.  By default block rows are ordered by colour
  // (ic0_colour_order): no two blocks of a colour are coupled, so a block
  // row depends only on blocks of earlier colours and the two sweeps have
  // as many dependency levels as there are colours.  OD_GB300_IC0_ORDER=natural
  // keeps the system's order (one level per step of the mesh's longest
  // dependency chain).
  std::vector<int> bperm(nb), binv(nb);
  const char* oenv = std::getenv("OD_GB300_IC0_ORDER");
  const bool natural = oenv && std::strcmp(oenv, "natural") == 0;
  P.ic_colours = natural ? 0 : ic0_colour_order(nb, rp, col, bperm, P.ic_cstart);
  if (natural)
    for (int b = 0; b < nb; b++) bperm[b] = b;
  for (int b = 0; b < nb; b++) binv[bperm[b]] = b;
  std::vector<int> srp(n + 1, 0), sci, ssrc;
  sci.reserve((size_t)s->bsr.nnzb * 5);
  ssrc.reserve((size_t)s->bsr.nnzb * 5);
  std::vector<std::pair<int, int>> blk;   // (factor block column, BSR block) of one block row
  for (int R = 0; R < nb; R++) {
    const int br = bperm[R];
    blk.clear();
    for (int k = rp[br]; k < rp[br + 1]; k++)
      if (binv[col[k]] <= R) blk.push_back({binv[col[k]], k});
    std::sort(blk.begin(), blk.end());
    for (int r = 0; r < 3; r++) {
      const int i = 3 * R + r;
      for (const auto& e : blk) {
        const int C = e.first, k = e.second;
        for (int c = 0; c < 3; c++) {
          const int j = 3 * C + c;
          if (j > i) break;
          sci.push_back(j);
          ssrc.push_back(9 * k + 3 * r + c);
        }
      }
      srp[i + 1] = (int)sci.size();
    }
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
  // pair lists of the one-launch factorisation (merge of row i before the
  // entry with row j without its diagonal, as ic0_factor_level walks them)
  std::vector<int> pp(nnz + 1, 0), pa, pb;
  int maxrow = 0, maxpairs = 0;
  for (int i = 0; i < n; i++) {
    const int bi = srp[i], ei = srp[i + 1];
    maxrow = std::max(maxrow, ei - bi);
    const size_t row0 = pa.size();
    for (int q = bi; q < ei; q++) {
      const int j = sci[q];
      if (j < i) {
        int a = bi, b = srp[j];
        const int eb = srp[j + 1] - 1;
        while (a < q && b < eb) {
          if (sci[a] == sci[b]) {
            pa.push_back(a - bi);
            pb.push_back(b);
            a++;
            b++;
          } else if (sci[a] < sci[b]) {
            a++;
          } else {
            b++;
          }
        }
      }
      pp[q + 1] = (int)pa.size();
    }
    maxpairs = std::max(maxpairs, (int)(pa.size() - row0));
  }
  // strictly lower rows for the forward sweep
  std::vector<int> frp(n + 1, 0), fci;
  fci.reserve(nnz);
  for (int i = 0; i < n; i++) {
    for (int q = srp[i]; q < srp[i + 1] - 1; q++) fci.push_back(sci[q]);
    frp[i + 1] = (int)fci.size();
  }
  // row triples by level for the one-launch sweeps
  std::vector<int> gof, gob;
  int gdf = 0, gdb = 0;
  sweep_group_levels(n, frp, fci, trp2, tci2, gof, gob, &gdf, &gdb);
  P.ic_gdepth = gdf + gdb;
  std::vector<int> lrf;
  build_ic_levels(srp, sci, n, lrf, P.lvl_ptr_f, true);
  P.ic_n = n;
  P.ic_nnz = nnz;
  P.n_levels_f = (int)P.lvl_ptr_f.size() - 1;
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
  if ((st = up(&P.icT_rp, trp2)) != OD_OK) return st;
  if ((st = up(&P.icT_ci, tci2)) != OD_OK) return st;
  if ((st = up(&P.icT_pos, tpos2)) != OD_OK) return st;
  if ((st = up(&P.ic_frp, frp)) != OD_OK) return st;
  if ((st = up(&P.ic_fci, fci)) != OD_OK) return st;
  if ((st = up(&P.ic_gord_f, gof)) != OD_OK) return st;
  {
    // one-launch factorisation when a row and its pairs fit the shared memory
    const size_t smem = sizeof(double) * (size_t)kIcfWarps * (2 * (size_t)maxrow + (size_t)maxpairs) +
                        sizeof(int) * (size_t)kIcfWarps * (size_t)maxpairs;
    int dev_coop = 0, per_sm = 0;
    OD_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, s->ctx->device));
    // OD_GB300_IC0_FACTOR=levels keeps the one-launch-per-level factorisation
    // (the path of rows too long for the warp's registers or shared memory)
    const char* fenv = std::getenv("OD_GB300_IC0_FACTOR");
    const bool levels_only = fenv && std::strcmp(fenv, "levels") == 0;
    if (dev_coop && !levels_only && pa.size() < (size_t)INT32_MAX && smem <= 96 * 1024 &&
        maxrow <= 32 * kIcfSlots) {
      OD_CUDA(cudaFuncSetAttribute(ic0_factor_coop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      OD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ic0_factor_coop_kernel, kIcfThreads, smem));
      if (per_sm > 0) {
        if ((st = up(&P.ic_pp, pp)) != OD_OK) return st;
        if ((st = up(&P.ic_pa, pa)) != OD_OK) return st;
        if ((st = up(&P.ic_pb, pb)) != OD_OK) return st;
        // two CTAs (8 warps) per SM: 1,216 warps hold a level's rows (a
        // few hundred on the 98k-tet beam) many times over; more only poll
        P.ic_fgrid = std::min(per_sm, 2) * s->ctx->num_sms;
        P.ic_fmaxrow = maxrow;
        P.ic_fmaxpairs = maxpairs;
        P.ic_fsmem = smem;
      }
    }
  }
  if ((st = up(&P.ic_gord_b, gob)) != OD_OK) return st;
  if (!natural) {
    std::vector<int> pdof(n);
    for (int R = 0; R < nb; R++)
      for (int r = 0; r < 3; r++) pdof[3 * R + r] = 3 * bperm[R] + r;
    if ((st = up(&P.ic_pdof, pdof)) != OD_OK) return st;
    OD_CUDA(cudaMalloc(&P.ic_zp, sizeof(double) * std::max(1, n)));
    s->device_bytes += sizeof(double) * (long long)n;
  }
  OD_CUDA(cudaMalloc(&P.ic_val, sizeof(double) * std::max(1, nnz)));
  const size_t nl = std::max<size_t>(1, fci.size());
  OD_CUDA(cudaMalloc(&P.ic_fval, sizeof(double) * nl));
  OD_CUDA(cudaMalloc(&P.ic_bval, sizeof(double) * nl));
  OD_CUDA(cudaMalloc(&P.ic_dval, sizeof(double) * std::max(1, n)));
  OD_CUDA(cudaMalloc(&P.ic_y, sizeof(double) * std::max(1, n)));
  OD_CUDA(cudaMalloc(&P.ic_bad, sizeof(int)));
  OD_CUDA(cudaMalloc(&P.ic_err, sizeof(int)));
  OD_CUDA(cudaMemset(P.ic_err, 0, sizeof(int)));
  OD_CUDA(cudaMallocHost(&P.ic_err_host, sizeof(int)));
  OD_TRY(sweep_grid(s, n, &P.ic_grid));
  // colours far larger than the one-launch sweep's warps (8 per CTA) go one
  // launch per colour instead
  P.ic_by_colour = false;
  if (!natural && P.ic_cstart.size() > 1) {
    int largest = 0;
    for (size_t c = 0; c + 1 < P.ic_cstart.size(); c++) largest = std::max(largest, P.ic_cstart[c + 1] - P.ic_cstart[c]);
    const char* lenv = std::getenv("OD_GB300_IC0_SWEEP");
    P.ic_by_colour = lenv ? std::strcmp(lenv, "levels") == 0 : largest > 4 * 8 * std::max(1, P.ic_grid);
  }
  s->device_bytes += sizeof(double) * ((long long)nnz + 2LL * (long long)nl + 2LL * n);
  return OD_OK;
}

od_status ic0_check(Scene* s);

// shifted IC(0) factorisation of the current A64 with the Manteuffel retry
od_status ic0_factor(Scene* s) {
  Pcg& P = s->pcg;
  od_status st = ic0_build(s);
  if (st != OD_OK) return st;
  cudaStream_t strm = s->ctx->stream;
  double shift = 0.0;
  for (int attempt = 0; attempt < 40; attempt++) {
    OD_CUDA(cudaMemsetAsync(P.ic_bad, 0, sizeof(int), strm));
    if (P.ic_fgrid > 0) {
      // every value starts "not yet written" (all-ones bytes)
      OD_CUDA(cudaMemsetAsync(P.ic_val, 0xff, sizeof(double) * (size_t)P.ic_nnz, strm));
      int nrow = P.ic_n, mr = P.ic_fmaxrow, mp = P.ic_fmaxpairs;
      const int* rows = P.lvl_rows_f;
      const int* rp = P.ic_rp;
      const int* ci = P.ic_ci;
      const int* src = P.ic_src;
      const double* A = s->A64;
      const int* pp = P.ic_pp;
      const int* pa = P.ic_pa;
      const int* pb = P.ic_pb;
      double* L = P.ic_val;
      int* badp = P.ic_bad;
      int* errp = P.ic_err;
      void* args[] = {(void*)&nrow, (void*)&rows, (void*)&rp,    (void*)&ci, (void*)&src,   (void*)&A,
                      (void*)&pp,   (void*)&pa,   (void*)&pb,    (void*)&L,  (void*)&shift, (void*)&mr,
                      (void*)&mp,   (void*)&badp, (void*)&errp};
      OD_KL(s);
      OD_CUDA(cudaLaunchCooperativeKernel((void*)ic0_factor_coop_kernel, dim3(P.ic_fgrid), dim3(kIcfThreads), args,
                                          P.ic_fsmem, strm));
    } else {
      for (int l = 0; l < P.n_levels_f; l++) {
        int l0 = P.lvl_ptr_f[l], l1 = P.lvl_ptr_f[l + 1];
        OD_KL(s);
        ic0_factor_level<double><<<nblk(l1 - l0, 128), 128, 0, strm>>>(l0, l1, P.lvl_rows_f, P.ic_rp, P.ic_ci,
                                                                        P.ic_src, s->A64, P.ic_val, shift, P.ic_bad);
      }
    }
    OD_CUDA(cudaGetLastError());
    int bad = 0;
    OD_CUDA(cudaMemcpyAsync(&bad, P.ic_bad, sizeof(int), cudaMemcpyDeviceToHost, strm));
    OD_TRY(sync_stream(s));
    if (P.ic_fgrid > 0) OD_TRY(ic0_check(s));
    if (!bad) break;
    shift = shift == 0.0 ? 1e-3 : 2.0 * shift;
  }
  P.ic_shift = shift;
  if (P.ic_n > 0) {
    const int nt = P.ic_nnz - P.ic_n;
    OD_KL(s);
    ic0_split_kernel<<<nblk(std::max(nt, P.ic_n), 256), 256, 0, strm>>>(P.ic_n, P.ic_rp, P.ic_frp, P.ic_val, nt,
                                                                         P.icT_pos, P.ic_fval, P.ic_bval, P.ic_dval);
    OD_CUDA(cudaGetLastError());
  }
  s->ctx->sweep_levels = P.ic_gdepth;
  return OD_OK;
}

// L y = r, L^T z = y in one cooperative launch (rows by dependency level,
// each row's value its own ready flag)
static od_status ic0_apply(Scene* s, const double* r, double* z, const SolveScalars* sc) {
  Pcg& P = s->pcg;
  SweepView v;
  v.n = P.ic_n;
  v.n_pad = P.n_pad;
  v.ic = 1;
  v.grid = P.ic_grid;
  v.nnz = (long long)P.ic_nnz - P.ic_n;
  v.frp = P.ic_frp;
  v.fci = P.ic_fci;
  v.fval = P.ic_fval;
  v.bcp = P.icT_rp;
  v.bri = P.icT_ci;
  v.bval = P.ic_bval;
  v.ord_f = P.ic_gord_f;
  v.ord_b = P.ic_gord_b;
  v.diag = P.ic_dval;
  v.y = P.ic_y;
  v.err = P.ic_err;
  v.perm = P.ic_pdof;
  v.zperm = P.ic_zp;
  if (P.ic_by_colour) v.colour_start = &P.ic_cstart;
  return sweep_launch(s, v, r, z, sc);
}

od_status ic0_check(Scene* s) {
  Pcg& P = s->pcg;
  if (!P.ic_err) return OD_OK;
  cudaStream_t strm = s->ctx->stream;
  OD_CUDA(cudaMemcpyAsync(P.ic_err_host, P.ic_err, sizeof(int), cudaMemcpyDeviceToHost, strm));
  OD_TRY(sync_stream(s));
  if (*P.ic_err_host) {
    OD_CUDA(cudaMemsetAsync(P.ic_err, 0, sizeof(int), strm));
    set_error("IC(0) sweep: a bounded wait on a row value ran out");
    return OD_ERR_DEVICE_TIMEOUT;
  }
  return OD_OK;
}

od_status pcg_alloc(Scene* s) {
  Pcg& P = s->pcg;
  const int n = 3 * s->bsr.nb;
  P.n_pad = n;
  P.grid = std::max(1, 2 * std::max(1, s->ctx->num_sms));  // partial capacity per array
  size_t nv = std::max(1, n);
  for (double** v : {&P.x, &P.r, &P.z, &P.p, &P.q, &P.b}) {
    OD_CUDA(cudaMalloc(v, sizeof(double) * nv));
    OD_CUDA(cudaMemset(*v, 0, sizeof(double) * nv));
  }
  OD_CUDA(cudaMalloc(&P.partial, sizeof(double) * 4 * (size_t)P.grid));
  OD_CUDA(cudaMalloc(&P.sc, sizeof(SolveScalars)));
  OD_CUDA(cudaMemset(P.sc, 0, sizeof(SolveScalars)));
  OD_CUDA(cudaMallocHost(&P.sc_host, sizeof(SolveScalars)));
  OD_CUDA(cudaMalloc(&P.pinv, sizeof(double) * 9 * (size_t)std::max(1, s->bsr.nb)));
  OD_CUDA(cudaMalloc(&P.gbar, sizeof(GridBarrier)));
  OD_CUDA(cudaMemset(P.gbar, 0, sizeof(GridBarrier)));
  OD_CUDA(cudaMallocHost(&P.timeout_host, sizeof(int)));
  // the device counters only grow; the host keeps the last copy read (second
  // half of prof_host) and takes differences
  P.prof_slots = kPcgProfSlots + 3 * P.grid;
  OD_CUDA(cudaMalloc(&P.prof, P.prof_slots * sizeof(unsigned long long)));
  OD_CUDA(cudaMemset(P.prof, 0, P.prof_slots * sizeof(unsigned long long)));
  OD_CUDA(cudaMallocHost(&P.prof_host, 2 * P.prof_slots * sizeof(unsigned long long)));
  std::memset(P.prof_host, 0, 2 * P.prof_slots * sizeof(unsigned long long));
  // co-resident CTAs for the cooperative solve: one 768-thread CTA per SM
  // (fewest arrivals per grid barrier; the round-robin group mapping keeps
  // every SM's FP64 pipe equally loaded)
  int coop = 0, bps = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, s->ctx->device);
  if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pcg_persistent_kernel<double, 4, false>, kPThreads, 0) ==
                  cudaSuccess && bps > 0) {
    P.coop_grid = std::min(bps, 1) * std::max(1, s->ctx->num_sms);
    P.grid = std::max(P.grid, P.coop_grid);
  }
  // shared memory of the staged variant: the largest CTA share of matrix
  // blocks (72 B values + 4 B column each) plus the inverse rows of every
  // (warp, group) segment; 0 when it does not fit one CTA's shared memory or
  // a warp would own more than two groups (OD_GB300_PCG_SMEM=0 disables it)
  P.smem_bytes = 0;
  // the one-launch PCG's form: -1 by size and tolerance (at the launch);
  // OD_GB300_PCG_FORM=standard, =recur or =pipelined forces one
  P.recur = -1;
  if (const char* f = std::getenv("OD_GB300_PCG_FORM"))
    P.recur = std::strcmp(f, "pipelined") == 0 ? 2 : (std::strcmp(f, "recur") == 0 ? 1 : 0);
  const char* smem_env = std::getenv("OD_GB300_PCG_SMEM");
  const int nb = s->bsr.nb;
  if (P.coop_grid > 0 && nb > 0 && !(smem_env && smem_env[0] == '0') && (int)s->hbsr_rp.size() == nb + 1) {
    const int G = P.coop_grid, wpc = kPThreads / 32;
    const int ngroups = (nb + kRowsPerWarp - 1) / kRowsPerWarp;
    const int need = (ngroups + G * wpc - 1) / (G * wpc);
    if (need <= kSmemGroupsMax) {
      std::vector<long long> cta((size_t)G, 0);
      for (int g = 0; g < ngroups; g++) {
        const int r0 = g * kRowsPerWarp, r1 = std::min(nb, r0 + kRowsPerWarp);
        cta[(size_t)(g % G)] += s->hbsr_rp[r1] - s->hbsr_rp[r0];
      }
      const long long mx = *std::max_element(cta.begin(), cta.end());
      const long long bytes = 8LL * wpc * need * kSmemPinv + 76LL * mx;
      int dev_max = 0;
      cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->ctx->device);
      const void* fn = need <= 1 ? (const void*)pcg_persistent_kernel<double, 1, true>
                                 : (const void*)pcg_persistent_kernel<double, 2, true>;
      // the attribute is per function, shared by every scene: set it to the
      // most the device allows, never to one scene's size
      cudaFuncAttributes fa{};
      const long long cap = (long long)dev_max - 1024;
      if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess && bytes + (long long)fa.sharedSizeBytes <= cap &&
          cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(cap - (long long)fa.sharedSizeBytes)) == cudaSuccess) {
        int bps2 = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps2, fn, kPThreads, (size_t)bytes) == cudaSuccess &&
            bps2 >= 1)
          P.smem_bytes = (int)bytes;
      }
      cudaGetLastError();   // a refused attribute is not an error of the scene
    }
  }
  OD_CUDA(cudaFree(P.partial));
  OD_CUDA(cudaMalloc(&P.partial, sizeof(double) * 4 * (size_t)P.grid));
  s->device_bytes += (long long)sizeof(double) * (6 * nv + 9 * (size_t)s->bsr.nb + 4 * (size_t)P.grid);
  return OD_OK;
}

void pcg_free(Scene* s) {
  Pcg& P = s->pcg;
  for (double* v : {P.x, P.r, P.z, P.p, P.q, P.b, P.partial, P.pinv, P.ic_val, P.ic_fval, P.ic_bval, P.ic_dval, P.ic_y,
                    P.ic_zp})
    cudaFree(v);
  if (P.ic_err_host) cudaFreeHost(P.ic_err_host);
  for (int* v : {P.ic_rp, P.ic_ci, P.ic_src, P.lvl_rows_f, P.icT_rp, P.icT_ci, P.icT_pos, P.ic_bad,
                 P.ic_frp, P.ic_fci, P.ic_err, P.ic_gord_f, P.ic_gord_b, P.ic_pp, P.ic_pa, P.ic_pb, P.ic_pdof})
    cudaFree(v);
  cudaFree(P.sc);
  cudaFree(P.gbar);
  mixed_free(P.mix);
  mixed_ic0_free(P.mic);
  slice_free(P.slice);
  sweep_free(P.sweep);
  if (P.sc_host) cudaFreeHost(P.sc_host);
  if (P.timeout_host) cudaFreeHost(P.timeout_host);
  cudaFree(P.prof);
  if (P.prof_host) cudaFreeHost(P.prof_host);
  P = Pcg();
}

// true residual ||b - A x|| / ||b|| on the device, then the statistics
static od_status pcg_finish(Scene* s, const double* d_b, double* d_x, double shift, od_solve_stats* st,
                            bool persistent, bool timed_persistent, bool phases = false) {
  Pcg& P = s->pcg;
  cudaStream_t strm = s->ctx->stream;
  const int nb = s->bsr.nb, n = P.n_pad;
  if (!persistent) {
    OD_KL(s);
    spmv_full_kernel<double><<<nblk(nb, kWarpRows), kThreads, 0, strm>>>(nb, s->bsr.row_ptr, s->bsr.col, s->A64,
                                                                         d_x, P.q);
    OD_KL(s);
    residual_norm_kernel<<<1, 1024, 0, strm>>>(n, d_b, P.q, P.sc);
    OD_CUDA(cudaGetLastError());
  }
  OD_CUDA(cudaMemcpyAsync(P.sc_host, P.sc, sizeof(SolveScalars), cudaMemcpyDeviceToHost, strm));
  if (phases)
    OD_CUDA(cudaMemcpyAsync(P.prof_host, P.prof, P.prof_slots * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            strm));
  int timeout = 0;
  if (P.gbar) OD_CUDA(cudaMemcpyAsync(P.timeout_host, &((GridBarrier*)P.gbar)->timeout, sizeof(int),
                                      cudaMemcpyDeviceToHost, strm));
  OD_TRY(sync_stream(s));
  if (P.gbar) timeout = *P.timeout_host;
  const SolveScalars& h = *P.sc_host;
  if (timed_persistent) {
    float ms = 0.f;
    OD_CUDA(cudaEventElapsedTime(&ms, s->ctx->ev_pool[0], s->ctx->ev_pool[1]));
    s->ctx->pcg_kernel_ms += ms;
    s->ctx->pcg_kernel_launches++;
    s->ctx->pcg_kernel_iters += h.iter;
  }
  if (phases) {
    unsigned long long* last = P.prof_host + P.prof_slots;
    for (int k = 0; k < kPcgPhases; k++) s->ctx->pcg_phase_ms[k] += 1e-6 * (double)(P.prof_host[k] - last[k]);
    s->ctx->pcg_phase_iters += (long long)(P.prof_host[kPcgPhases] - last[kPcgPhases]);
    // per-CTA own work of this solve: the slowest CTA and the mean
    const int G2 = P.coop_grid;
    for (int k = 0; k < 3 && G2 > 0; k++) {
      double mx = 0.0, sum = 0.0;
      for (int b = 0; b < G2; b++) {
        const size_t i = kPcgProfSlots + (size_t)k * G2 + b;
        const double d = 1e-6 * (double)(P.prof_host[i] - last[i]);
        mx = std::max(mx, d);
        sum += d;
      }
      s->ctx->pcg_work_max_ms[k] += mx;
      s->ctx->pcg_work_mean_ms[k] += sum / G2;
    }
    for (int k = 0; k < P.prof_slots; k++) last[k] = P.prof_host[k];
  }
  od_status status = (od_status)h.status;
  if (timeout) { status = OD_ERR_DEVICE_TIMEOUT; set_error("PCG grid barrier timed out"); }
  if (status == OD_OK && h.iter >= h.max_iter && h.rr > h.eps) status = OD_ERR_NOT_CONVERGED;
  if (st) {
    st->iterations = h.iter;
    st->refinements = 0;
    st->rel_residual = h.tr_den > 0.0 ? std::sqrt(h.tr_num / h.tr_den) : std::sqrt(h.tr_num);
    st->ic_shift = shift;
    st->status = status;
  }
  return status == OD_ERR_DEVICE_TIMEOUT ? OD_ERR_DEVICE_TIMEOUT : OD_OK;
}

// ---- mixed-precision systems: build, partition, solve

// the ring kernel of a tile shape: piece size (12, 16 or 20 steps) x
// consumer warps (12, or 15 with pieces of 12 or 16 steps: 15 warps of
// 20-step rings exceed the shared memory)
static const void* ring_kernel(int ps, int nw) {
  if (nw == 15) return ps == 12 ? (const void*)pcg32_ring_kernel<12, 15> : (const void*)pcg32_ring_kernel<16, 15>;
  switch (ps) {
    case 12: return (const void*)pcg32_ring_kernel<12, 12>;
    case 16: return (const void*)pcg32_ring_kernel<16, 12>;
    default: return (const void*)pcg32_ring_kernel<20, 12>;
  }
}

bool ring_shape_supported(int ps, int nw) {
  return (nw == 12 && (ps == 12 || ps == 16 || ps == 20)) || (nw == 15 && (ps == 12 || ps == 16));
}

static const int kRingShapes[5][2] = {{12, 12}, {16, 12}, {20, 12}, {12, 15}, {16, 15}};

// co-resident CTAs of the ring kernel: one per SM for every tile shape
static int ring_kernel_ctas(const Ctx* ctx) {
  int per_sm = 1;
  for (const auto& sh : kRingShapes) {
    const int ps = sh[0], nw = sh[1];
    int p = 0;
    if (cudaFuncSetAttribute(ring_kernel(ps, nw), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             ring_smem_bytes(ps, nw)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, ring_kernel(ps, nw), 32 * (nw + 1),
                                                      ring_smem_bytes(ps, nw)) != cudaSuccess)
      return 0;
    per_sm = std::min(per_sm, p);
  }
  return per_sm * ctx->num_sms;
}

void slice_free(SliceSys* sl) {
  if (!sl) return;
  for (int* v : {sl->perm, sl->off, sl->col, sl->src}) cudaFree(v);
  cudaFree(sl->val);
  cudaFree(sl->v32);
  cudaFree(sl->r64);
  delete sl;
}

template <class T>
static od_status dev_upload(T** dst, const T* src, size_t n, long long& bytes) {
  OD_CUDA(cudaMalloc((void**)dst, sizeof(T) * std::max<size_t>(1, n)));
  if (n) OD_CUDA(cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  bytes += (long long)(sizeof(T) * n);
  return OD_OK;
}

od_status slice_build(Scene* s) {
  Pcg& P = s->pcg;
  if (P.slice) return OD_OK;
  SliceSys* sl = new SliceSys();
  HostSliced hs;
  // the symmetric (lower-triangle) operator halves the matrix stream of
  // every inner iteration; OD_GB300_MIXED_SPMV=full keeps both triangles
  // (deterministic: no atomic accumulation)
  const char* menv = std::getenv("OD_GB300_MIXED_SPMV");
  const bool lower = !(menv && std::strcmp(menv, "full") == 0);
  build_sliced(s->hbsr_rp, s->hbsr_col, s->bsr.nb, hs, lower);
  sl->lower = lower ? 1 : 0;
  sl->ns = hs.ns;
  sl->steps = hs.off[hs.ns];
  sl->off_host = hs.off;
  long long stored = 0;
  for (int r = 0; r < s->bsr.nb; r++)
    for (int k = s->hbsr_rp[r]; k < s->hbsr_rp[r + 1]; k++) stored += (!lower || s->hbsr_col[k] <= r) ? 1 : 0;
  sl->bytes = 40.0 * (double)stored + 24.0 * s->bsr.nb;
  auto fail = [&](od_status st) { slice_free(sl); return st; };
  od_status st;
  if ((st = dev_upload(&sl->perm, hs.perm.data(), hs.perm.size(), sl->device_bytes)) != OD_OK) return fail(st);
  if ((st = dev_upload(&sl->off, hs.off.data(), hs.off.size(), sl->device_bytes)) != OD_OK) return fail(st);
  if ((st = dev_upload(&sl->col, hs.col.data(), hs.col.size(), sl->device_bytes)) != OD_OK) return fail(st);
  if ((st = dev_upload(&sl->src, hs.src.data(), hs.src.size(), sl->device_bytes)) != OD_OK) return fail(st);
  const size_t ns = (size_t)std::max(1, sl->ns);
  const size_t nval = (size_t)std::max<long long>(1, sl->steps) * 90;
  // u (float4 rows), d, r, p, w, preconditioner, s; lower storage adds w as float4 rows
  const size_t nvec = (40 + 4 * 30 + 90 + 30 + (lower ? 40 : 0)) * ns;
  cudaError_t e = cudaMalloc(&sl->val, sizeof(float) * nval);
  if (e == cudaSuccess) e = cudaMalloc(&sl->v32, sizeof(float) * nvec);
  if (e == cudaSuccess) e = cudaMemset(sl->v32, 0, sizeof(float) * nvec);
  if (e == cudaSuccess) e = cudaMalloc(&sl->r64, sizeof(double) * std::max(1, P.n_pad));
  if (e != cudaSuccess) return fail(cuda_fail(e, "slice_build"));
  sl->device_bytes += (long long)(sizeof(float) * (nval + nvec) + sizeof(double) * P.n_pad);
  s->device_bytes += sl->device_bytes;
  P.slice = sl;
  return OD_OK;
}

void mixed_free(MixedSys* m) {
  if (!m) return;
  for (int* v : {m->sc_slice_dev, m->dirs, m->cta_first, m->cta_sc_lo, m->sc_cta}) cudaFree(v);
  cudaFree(m->desc);
  cudaFree(m->ring);
  cudaFree(m->rrbb);
  cudaFree(m->res_part);
  cudaFree(m->part);
  cudaFree(m->cta_ns);
  if (m->cta_ns_host) cudaFreeHost(m->cta_ns_host);
  cudaFree(m->gbar);
  cudaFree(m->prof);
  if (m->ring_host) cudaFreeHost(m->ring_host);
  if (m->rrbb_host) cudaFreeHost(m->rrbb_host);
  if (m->timeout_host) cudaFreeHost(m->timeout_host);
  if (m->prof_host) cudaFreeHost(m->prof_host);
  delete m;
}

// Contiguous slice ranges per CTA with about equal cost and at most
// kMaxLocalScenes scenes each.  Cost of a slice = its steps + kSliceCost
// (the fixed work of a slice: ring hand-offs, shuffles, the q store), so
// regions of short rows (boundary layers) do not make their CTAs the last to
// finish.  OD_GB300_SLICE_COST overrides the constant.
constexpr double kSliceCost = 8.0;
// Contiguous slice ranges of equal total weight, one per CTA (at most
// kMaxLocalScenes scenes per CTA).  The weight of a slice is its steps plus a
// per-slice cost at first; measured times refine it (mixed_rebalance).
static od_status mixed_partition(MixedSys* m, int G) {
  const int ns = m->ns;
  if ((int)m->slice_w.size() != ns) {
    const double c_slice = m->slice_cost;
    m->slice_w.resize(ns);
    for (int k = 0; k < ns; k++) m->slice_w[k] = (double)(m->off_host[k + 1] - m->off_host[k]) + c_slice;
  }
  std::vector<int> sc_of(ns);
  for (int s = 0; s < m->n_sc; s++)
    for (int k = m->sc_slice[s]; k < m->sc_slice[s + 1]; k++) sc_of[k] = s;
  std::vector<double> cum(ns + 1, 0.0);
  for (int k = 0; k < ns; k++) cum[k + 1] = cum[k] + m->slice_w[k];
  std::vector<int> first(G + 1, ns), sc_lo(G, 0);
  std::vector<int> sc_cta(2 * std::max(1, m->n_sc), -1);
  for (int s = 0; s < m->n_sc; s++) sc_cta[2 * s + 1] = -2;  // empty range for scenes without slices
  // Each CTA takes slices up to an equal share of the remaining weight; it
  // takes more when the scenes left after it would not fit the remaining
  // CTAs at kMaxLocalScenes each (many small scenes), and it never spans more
  // than kMaxLocalScenes scenes.
  int sl = 0;
  for (int b = 0; b < G; b++) {
    first[b] = sl;
    sc_lo[b] = sl < ns ? sc_of[sl] : 0;
    const double target = cum[sl] + (cum[ns] - cum[sl]) / (G - b);
    const long long room_after = (long long)kMaxLocalScenes * (G - b - 1);
    while (sl < ns) {
      if (sc_of[sl] - sc_lo[b] >= kMaxLocalScenes) break;
      const bool share = cum[sl] < target || b == G - 1;
      const bool crowded = (long long)(m->n_sc - sc_of[sl]) > room_after;
      if (!share && !crowded) break;
      sl++;
    }
  }
  first[G] = sl;
  if (sl < ns) {
    set_error("mixed solve: too many small scenes for one grid (at most " + std::to_string(kMaxLocalScenes) +
              " per multiprocessor)");
    return OD_ERR_UNSUPPORTED;
  }
  for (int b = 0; b < G; b++) {
    if (first[b + 1] <= first[b]) continue;
    for (int s = sc_of[first[b]]; s <= sc_of[first[b + 1] - 1]; s++) {
      if (sc_cta[2 * s] < 0) sc_cta[2 * s] = b;
      sc_cta[2 * s + 1] = b;
    }
  }
  m->first_host = first;
  const size_t npart = (size_t)3 * std::max(1, m->n_sc) * G + 2 * (size_t)G;
  if (!m->cta_first) {
    long long scratch = 0;
    OD_TRY(dev_upload(&m->cta_first, first.data(), first.size(), scratch));
    OD_TRY(dev_upload(&m->cta_sc_lo, sc_lo.data(), sc_lo.size(), scratch));
    OD_TRY(dev_upload(&m->sc_cta, sc_cta.data(), sc_cta.size(), scratch));
    OD_CUDA(cudaMalloc(&m->part, sizeof(double) * npart));
    OD_CUDA(cudaMalloc(&m->cta_ns, sizeof(unsigned long long) * G));
    OD_CUDA(cudaMallocHost(&m->cta_ns_host, sizeof(unsigned long long) * G));
  } else {
    OD_CUDA(cudaMemcpy(m->cta_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice));
    OD_CUDA(cudaMemcpy(m->cta_sc_lo, sc_lo.data(), sizeof(int) * sc_lo.size(), cudaMemcpyHostToDevice));
    OD_CUDA(cudaMemcpy(m->sc_cta, sc_cta.data(), sizeof(int) * sc_cta.size(), cudaMemcpyHostToDevice));
  }
  OD_CUDA(cudaMemset(m->part, 0, sizeof(double) * npart));
  OD_CUDA(cudaMemset(m->cta_ns, 0, sizeof(unsigned long long) * G));
  m->cta_grid = G;
  return OD_OK;
}

// Weights of a multi-scene system's slices: the slice's steps plus the
// per-slice cost, times its scene's expected inner iterations relative to
// the median (those of the scene's last mixed solve; the median for a scene
// without one; clamped to [1/16, 256] x the median), so that each scene's
// share of the CTAs follows its work and the scenes finish together rather
// than the slowest one running its last iterations on the few CTAs a
// size-proportional share gives it.  Leaves the weights alone when no scene
// has a history.
static void mixed_work_weights(MixedSys* m) {
  std::vector<double> known;
  for (Scene* s : m->scenes)
    if (s->mix_iters_last > 0.0) known.push_back(s->mix_iters_last);
  if (known.empty()) return;
  std::nth_element(known.begin(), known.begin() + known.size() / 2, known.end());
  const double med = std::max(1.0, known[known.size() / 2]);
  const double c_slice = m->slice_cost;
  m->slice_w.resize(m->ns);
  for (int s = 0; s < m->n_sc; s++) {
    const double it = m->scenes[s]->mix_iters_last > 0.0 ? m->scenes[s]->mix_iters_last : med;
    const double f = std::min(256.0, std::max(1.0 / 16.0, it / med));
    for (int k = m->sc_slice[s]; k < m->sc_slice[s + 1]; k++)
      m->slice_w[k] = ((double)(m->off_host[k + 1] - m->off_host[k]) + c_slice) * f;
  }
}

// the partition with the work weights, else (too many scenes for a CTA)
// with the size weights
static od_status mixed_partition_work(MixedSys* m, int G) {
  mixed_work_weights(m);
  if (mixed_partition(m, G) == OD_OK) return OD_OK;
  m->slice_w.clear();
  return mixed_partition(m, G);
}

// new tile shapes for a built system: piece size of the ring kernel and the
// per-slice cost of the partition (the slices are re-partitioned)
od_status mixed_retune(MixedSys* m, int piece_steps, int ring_warps, double slice_cost) {
  if (!ring_shape_supported(piece_steps, ring_warps) || !(slice_cost >= 0.0)) {
    set_error("mixed tuning: piece steps 12, 16 or 20 with 12 consumer warps, or 12 or 16 with 15, and a slice "
              "cost >= 0");
    return OD_ERR_INVALID_ARG;
  }
  m->piece_steps = piece_steps;
  m->ring_warps = ring_warps;
  m->slice_cost = slice_cost;
  m->slice_w.clear();
  return m->n_sc > 1 ? mixed_partition_work(m, m->cta_grid) : mixed_partition(m, m->cta_grid);
}

// After a solve of a one-scene system: scale the weights of each CTA's
// slices by the CTA's measured SpMV time per weight (relative to the
// median) and re-partition, while the slowest CTA is more than 3% behind
// the median (at most three times per system).  The slowness is a property
// of the slices (boundary layers: short rows, padding) and moves with them.
static od_status mixed_rebalance(Ctx* ctx, MixedSys* m) {
  const int G = m->cta_grid;
  OD_CUDA(cudaMemcpyAsync(m->cta_ns_host, m->cta_ns, sizeof(unsigned long long) * G, cudaMemcpyDeviceToHost,
                          ctx->stream));
  OD_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<double> t(G), rate(G, 0.0);
  for (int b = 0; b < G; b++) t[b] = (double)m->cta_ns_host[b];
  std::vector<double> sorted = t;
  std::sort(sorted.begin(), sorted.end());
  const double median = sorted[G / 2], worst = sorted[G - 1];
  OD_CUDA(cudaMemsetAsync(m->cta_ns, 0, sizeof(unsigned long long) * G, ctx->stream));
  if (m->n_sc != 1 || m->rebalances >= 3 || median <= 0.0 || worst < 1.03 * median) return OD_OK;
  std::vector<double> rates;
  for (int b = 0; b < G; b++) {
    double w = 0.0;
    for (int k = m->first_host[b]; k < m->first_host[b + 1]; k++) w += m->slice_w[k];
    if (w > 0.0 && t[b] > 0.0) {
      rate[b] = t[b] / w;
      rates.push_back(rate[b]);
    }
  }
  if (rates.empty()) return OD_OK;
  std::sort(rates.begin(), rates.end());
  const double mid = rates[rates.size() / 2];
  for (int b = 0; b < G; b++) {
    if (rate[b] <= 0.0) continue;
    const double f = std::min(2.0, std::max(0.5, rate[b] / mid));
    for (int k = m->first_host[b]; k < m->first_host[b + 1]; k++) m->slice_w[k] *= f;
  }
  m->rebalances++;
  return mixed_partition(m, G);
}

od_status mixed_build(Ctx* ctx, const std::vector<Scene*>& scenes, const std::vector<const double*>& b,
                      const std::vector<double*>& x, MixedSys** out) {
  for (Scene* s : scenes) OD_TRY(slice_build(s));
  const int G = ring_kernel_ctas(ctx);
  if (G <= 0) {
    set_error("mixed precision needs a cooperative launch of the ring kernel");
    return OD_ERR_UNSUPPORTED;
  }
  MixedSys* m = new MixedSys();
  // default tile shape by layout (measured on the 2.6M-tet block: lower
  // storage 47.7 ms per step with 12-step pieces and 15 consumer warps
  // against 51.5 with 20 and 12; both triangles best with 20 and 12)
  if (!scenes.empty() && scenes[0]->pcg.slice && scenes[0]->pcg.slice->lower) {
    m->piece_steps = 12;
    m->ring_warps = 15;
  }
  if (const char* e = std::getenv("OD_GB300_SLICE_COST")) m->slice_cost = std::atof(e);
  {
    int ps = m->piece_steps, nw = m->ring_warps;
    if (const char* e = std::getenv("OD_GB300_RING_PIECE")) ps = std::atoi(e);
    if (const char* e = std::getenv("OD_GB300_RING_WARPS")) nw = std::atoi(e);
    if (ring_shape_supported(ps, nw)) {
      m->piece_steps = ps;
      m->ring_warps = nw;
    }
  }
  const int n = (int)scenes.size();
  m->n_sc = n;
  m->scenes = scenes;
  m->sc_slice.assign(1, 0);
  m->off_host.assign(1, 0);
  std::vector<int> dirs(4 * (n + 1), 0);
  int* pres = dirs.data();
  int* pfill = pres + (n + 1);
  int* ppre = pfill + (n + 1);
  int* pupd = ppre + (n + 1);
  for (int i = 0; i < n; i++) {
    Scene* s = scenes[i];
    const SliceSys* sl = s->pcg.slice;
    const int step0 = m->off_host.back();
    for (int k = 1; k <= sl->ns; k++) m->off_host.push_back(step0 + sl->off_host[k]);
    MixDesc d{};
    d.row_ptr = s->bsr.row_ptr;
    d.col = s->bsr.col;
    d.diag_pos = s->bsr.diag_pos;
    d.A64 = s->A64;
    d.b = i < (int)b.size() ? b[i] : nullptr;
    d.x = i < (int)x.size() ? x[i] : nullptr;
    d.nb = s->bsr.nb;
    d.ns = sl->ns;
    d.steps = (int)sl->steps;
    d.slice0 = m->sc_slice.back();
    d.sperm = sl->perm;
    d.soff = sl->off;
    d.scol = sl->col;
    d.ssrc = sl->src;
    d.sval = sl->val;
    d.v32 = sl->v32;
    d.r64 = sl->r64;
    d.lower = sl->lower;
    m->desc_host.push_back(d);
    m->sc_slice.push_back(d.slice0 + sl->ns);
    m->sc_nb.push_back(s->bsr.nb);
    m->sc_bytes.push_back(sl->bytes);
    pres[i + 1] = pres[i] + (d.nb + kResRows - 1) / kResRows;
    pfill[i + 1] = pfill[i] + (d.steps + kFillSteps - 1) / kFillSteps;
    ppre[i + 1] = ppre[i] + (d.ns * kSliceRows + kThreads - 1) / kThreads;
    pupd[i + 1] = pupd[i] + (3 * kSliceRows * d.ns + kThreads - 1) / kThreads;
  }
  m->ns = m->sc_slice.back();
  auto fail = [&](od_status st) { mixed_free(m); return st; };
  long long scratch = 0;
  od_status st;
  if ((st = dev_upload(&m->sc_slice_dev, m->sc_slice.data(), m->sc_slice.size(), scratch)) != OD_OK) return fail(st);
  if ((st = dev_upload(&m->desc, m->desc_host.data(), m->desc_host.size(), scratch)) != OD_OK) return fail(st);
  if ((st = dev_upload(&m->dirs, dirs.data(), dirs.size(), scratch)) != OD_OK) return fail(st);
  m->res_dir = TileDir{m->dirs, pres[n], kResRows};
  m->fill_dir = TileDir{m->dirs + (n + 1), pfill[n], kFillSteps};
  m->pre_dir = TileDir{m->dirs + 2 * (n + 1), ppre[n], kThreads};
  m->upd_dir = TileDir{m->dirs + 3 * (n + 1), pupd[n], kThreads};
  cudaError_t e = cudaMalloc(&m->ring, sizeof(RingScene) * std::max(1, n));
  if (e == cudaSuccess) e = cudaMallocHost(&m->ring_host, sizeof(RingScene) * std::max(1, n));
  if (e == cudaSuccess) e = cudaMalloc(&m->rrbb, sizeof(double) * 2 * std::max(1, n));
  if (e == cudaSuccess) e = cudaMallocHost(&m->rrbb_host, sizeof(double) * 2 * std::max(1, n));
  if (e == cudaSuccess) e = cudaMalloc(&m->res_part, sizeof(double) * 2 * std::max(1, pres[n]));
  if (e == cudaSuccess) e = cudaMalloc(&m->gbar, sizeof(GridBarrier));
  if (e == cudaSuccess) e = cudaMallocHost(&m->timeout_host, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&m->prof, (3 + (size_t)ctx->num_sms) * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMallocHost(&m->prof_host, 3 * sizeof(unsigned long long));
  if (e != cudaSuccess) return fail(cuda_fail(e, "mixed_build"));
  if ((st = n > 1 ? mixed_partition_work(m, G) : mixed_partition(m, G)) != OD_OK) return fail(st);
  *out = m;
  return OD_OK;
}

// FP64 residual of every scene and its norms; brings rrbb (and the ring
// outputs) back to the host
static od_status mixed_residual(Ctx* ctx, MixedSys* m, bool with_ring, bool x_zero = false) {
  cudaStream_t strm = ctx->stream;
  if (m->res_dir.tiles > 0) {
    ctx->launches += 2;
    mix_residual_kernel<<<m->res_dir.tiles, kThreads, 0, strm>>>(m->n_sc, m->res_dir.prefix, m->desc, m->res_part,
                                                                  x_zero ? 1 : 0);
    mix_residual_finish<<<nblk(m->n_sc, kThreads / 32), kThreads, 0, strm>>>(m->n_sc, m->res_dir.prefix, m->res_part,
                                                                             m->rrbb);
    OD_CUDA(cudaGetLastError());
  } else {
    OD_CUDA(cudaMemsetAsync(m->rrbb, 0, sizeof(double) * 2 * m->n_sc, strm));
  }
  OD_CUDA(cudaMemcpyAsync(m->rrbb_host, m->rrbb, sizeof(double) * 2 * m->n_sc, cudaMemcpyDeviceToHost, strm));
  if (with_ring)
    OD_CUDA(cudaMemcpyAsync(m->ring_host, m->ring, sizeof(RingScene) * m->n_sc, cudaMemcpyDeviceToHost, strm));
  ctx->host_syncs++;
  OD_CUDA(cudaStreamSynchronize(strm));
  return OD_OK;
}

od_status mixed_solve(Ctx* ctx, MixedSys* m, int pk, const std::vector<od_solver_params>& prm,
                      std::vector<od_solve_stats>& st, bool x_zero) {
  cudaStream_t strm = ctx->stream;
  const int n_sc = m->n_sc;
  st.assign(n_sc, od_solve_stats{});
  if (pk < 0 || pk >= OD_PRECOND_IC0) {
    set_error("the multi-scene mixed solve supports the none, Jacobi and block-Jacobi preconditioners "
              "(mixed IC(0) solves one scene at a time)");
    return OD_ERR_UNSUPPORTED;
  }
  if (m->fill_dir.tiles > 0) {
    ctx->launches++;
    mix_fill_kernel<<<m->fill_dir.tiles, kThreads, 0, strm>>>(n_sc, m->fill_dir.prefix, m->desc);
  }
  if (pk != OD_PRECOND_NONE && m->pre_dir.tiles > 0) {
    ctx->launches++;
    mix_precond_kernel<<<m->pre_dir.tiles, kThreads, 0, strm>>>(n_sc, m->pre_dir.prefix, pk, m->desc);
  }
  OD_TRY(mixed_residual(ctx, m, false, x_zero));
  std::vector<double> eps(n_sc), rr(n_sc), bb(n_sc);
  std::vector<int> total(n_sc, 0), sweeps(n_sc, 0), need(n_sc, 0), status(n_sc, OD_OK);
  for (int s = 0; s < n_sc; s++) {
    rr[s] = m->rrbb_host[2 * s];
    bb[s] = m->rrbb_host[2 * s + 1];
    eps[s] = bb[s] * prm[s].tol * prm[s].tol;
    if (!std::isfinite(rr[s])) status[s] = OD_ERR_NAN;
    need[s] = status[s] == OD_OK && rr[s] > eps[s] && prm[s].max_iter > 0 && m->sc_nb[s] > 0;
  }
  const bool prof = ctx->profiling && ctx->ev_pool.size() >= 2;
  od_status rc = OD_OK;
  for (int sweep = 0;; sweep++) {
    bool any = false;
    for (int s = 0; s < n_sc; s++) {
      const int max_refine = prm[s].max_refine > 0 ? prm[s].max_refine : 20;
      if (need[s] && (sweeps[s] >= max_refine || total[s] >= prm[s].max_iter)) need[s] = 0;
      RingScene& R = m->ring_host[s];
      R = RingScene{};
      R.active0 = need[s];
      if (need[s]) {
        any = true;
        const double rn = std::sqrt(rr[s]);
        const double inner_tol = prm[s].inner_tol > 0.0 ? prm[s].inner_tol : 1e-4;
        // a sweep reduces the residual no further than the outer target needs
        // (with a 0.3 margin), and at least by inner_tol
        const double itol = std::max(inner_tol, std::min(0.5, 0.3 * std::sqrt(eps[s] / rr[s])));
        R.rhs_scale = rn > 0.0 ? 1.0 / rn : 1.0;
        R.unscale = rn > 0.0 ? rn : 1.0;
        R.itol2 = itol * itol;
        R.max_iter = prm[s].max_iter - total[s];
      }
    }
    if (!any) break;
    OD_CUDA(cudaMemcpyAsync(m->ring, m->ring_host, sizeof(RingScene) * n_sc, cudaMemcpyHostToDevice, strm));
    OD_CUDA(cudaMemsetAsync(m->gbar, 0, sizeof(GridBarrier), strm));
    GridBarrier* gbp = (GridBarrier*)m->gbar;
    unsigned long long* profp = prof ? m->prof : nullptr;
    if (prof) OD_CUDA(cudaMemsetAsync(m->prof, 0, 3 * sizeof(unsigned long long), strm));
    int pkv = pk, nsc = n_sc;
    void* args[] = {(void*)&nsc,       (void*)&m->cta_first, (void*)&m->cta_sc_lo, (void*)&m->sc_cta,
                    (void*)&m->sc_slice_dev, (void*)&m->desc, (void*)&m->ring,    (void*)&pkv,
                    (void*)&m->part,   (void*)&gbp,          (void*)&profp,       (void*)&m->cta_ns};
    if (prof) OD_CUDA(cudaEventRecord(ctx->ev_pool[0], strm));
    ctx->launches++;
    OD_CUDA(cudaLaunchCooperativeKernel(ring_kernel(m->piece_steps, m->ring_warps), dim3(m->cta_grid),
                                        dim3(32 * (m->ring_warps + 1)), args,
                                        ring_smem_bytes(m->piece_steps, m->ring_warps), strm));
    if (prof) OD_CUDA(cudaEventRecord(ctx->ev_pool[1], strm));
    if (m->upd_dir.tiles > 0) {
      ctx->launches++;
      mix_update_kernel<<<m->upd_dir.tiles, kThreads, 0, strm>>>(n_sc, m->upd_dir.prefix, m->desc, m->ring);
    }
    OD_CUDA(cudaMemcpyAsync(m->timeout_host, &gbp->timeout, sizeof(int), cudaMemcpyDeviceToHost, strm));
    OD_TRY(mixed_residual(ctx, m, true));
    if (*m->timeout_host) {
      set_error("PCG grid barrier timed out");
      rc = OD_ERR_DEVICE_TIMEOUT;
      for (int s = 0; s < n_sc; s++)
        if (need[s]) status[s] = OD_ERR_DEVICE_TIMEOUT;
      break;
    }
    if (prof) {
      float ms = 0.f;
      OD_CUDA(cudaEventElapsedTime(&ms, ctx->ev_pool[0], ctx->ev_pool[1]));
      ctx->pcg_kernel_ms += ms;
      ctx->pcg_kernel_launches++;
      OD_CUDA(cudaMemcpy(m->prof_host, m->prof, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
      ctx->mix_spmv_ms += 1e-6 * (double)m->prof_host[0];
      ctx->mix_spmv_work_ms += 1e-6 * (double)m->prof_host[2];
      ctx->mix_iters += (long long)m->prof_host[1];
      for (int s = 0; s < n_sc; s++)
        if (need[s]) ctx->mix_spmv_bytes += (double)m->ring_host[s].iters * m->sc_bytes[s];
    }
    for (int s = 0; s < n_sc; s++) {
      if (!need[s]) continue;
      const RingScene& R = m->ring_host[s];
      total[s] += R.iters;
      if (prof) ctx->pcg_kernel_iters += R.iters;
      sweeps[s]++;
      rr[s] = m->rrbb_host[2 * s];
      if (!std::isfinite(rr[s]) || R.status == OD_ERR_NAN) { status[s] = OD_ERR_NAN; need[s] = 0; continue; }
      need[s] = rr[s] > eps[s] && R.iters > 0;  // no progress possible without an inner iteration
    }
  }
  if (rc == OD_OK) OD_TRY(mixed_rebalance(ctx, m));
  for (int s = 0; s < n_sc; s++) {
    if (status[s] == OD_OK && rr[s] > eps[s] && m->sc_nb[s] > 0) status[s] = OD_ERR_NOT_CONVERGED;
    if ((status[s] == OD_ERR_NOT_CONVERGED || status[s] == OD_ERR_NAN) && rc == OD_OK) {
      // the FP32 inner solve could not carry the refinement (FP32 operator too
      // far from the FP64 one for this system): finish with the FP64 PCG from
      // the current iterate, same tolerance and preconditioner
      od_solver_params p64 = prm[s];
      p64.precision = OD_PRECISION_FP64;
      p64.max_iter = std::max(1, prm[s].max_iter);
      const MixDesc& D = m->desc_host[s];
      od_solve_stats s64{};
      if (!std::isfinite(rr[s])) OD_CUDA(cudaMemsetAsync(D.x, 0, sizeof(double) * 3 * (size_t)D.nb, strm));
      const auto tf0 = std::chrono::steady_clock::now();
      const od_status rc64 = pcg_solve(m->scenes[s], D.b, D.x, &p64, &s64);
      ctx->mix_fallback_ms +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tf0).count();
      ctx->mix_fallbacks++;
      if (rc64 == OD_OK) {
        total[s] += s64.iterations;
        status[s] = s64.status;
        rr[s] = s64.rel_residual * s64.rel_residual * (bb[s] > 0.0 ? bb[s] : 1.0);
      }
    }
    st[s].iterations = total[s];
    m->scenes[s]->mix_iters_last = (double)total[s];
    st[s].refinements = sweeps[s];
    st[s].rel_residual = bb[s] > 0.0 ? std::sqrt(rr[s] / bb[s]) : std::sqrt(rr[s]);
    st[s].ic_shift = 0.0;
    st[s].status = status[s];
  }
  // a multi-scene system solved again (a reused batch) starts from the
  // partition its scenes' iterations ask for
  if (rc == OD_OK && n_sc > 1) OD_TRY(mixed_partition_work(m, m->cta_grid));
  return rc;
}

// single-scene mixed solve: the scene's own one-scene system
static od_status pcg_solve_mixed(Scene* s, const double* d_b, double* d_x, const od_solver_params* prm,
                                 od_solve_stats* st, bool x_zero) {
  Pcg& P = s->pcg;
  if (prm->precond == OD_PRECOND_IC0) return mixed_ic0_solve(s, d_b, d_x, prm, st);
  if (!P.mix) OD_TRY(mixed_build(s->ctx, {s}, {d_b}, {d_x}, &P.mix));
  MixedSys* m = P.mix;
  if (m->desc_host[0].b != d_b || m->desc_host[0].x != d_x) {
    m->desc_host[0].b = d_b;
    m->desc_host[0].x = d_x;
    OD_CUDA(cudaMemcpyAsync(m->desc, m->desc_host.data(), sizeof(MixDesc), cudaMemcpyHostToDevice, s->ctx->stream));
  }
  std::vector<od_solve_stats> out;
  od_status rc = mixed_solve(s->ctx, m, prm->precond, {*prm}, out, x_zero);
  if (st) *st = out[0];
  return rc;
}

// Solve A64 x = b (device vectors of length n_pad; padding entries zero).
// The preconditioner is rebuilt from A64 first, as CGSolver does on every
// solve (cgSolver.cpp:23).
od_status pcg_solve(Scene* s, const double* d_b, double* d_x, const od_solver_params* prm, od_solve_stats* st) {
  Pcg& P = s->pcg;
  const bool x_zero = P.x_zero;   // one solve only
  P.x_zero = false;
  cudaStream_t strm = s->ctx->stream;
  const int nb = s->bsr.nb, n = P.n_pad;
  const int pk = prm->precond;
  if (pk < 0 || pk > OD_PRECOND_IC) { set_error("unknown preconditioner"); return OD_ERR_INVALID_ARG; }
  if (nb == 0) {
    if (st) *st = od_solve_stats{};
    return OD_OK;
  }
  if (prm->precision == OD_PRECISION_MIXED) return pcg_solve_mixed(s, d_b, d_x, prm, st, x_zero);
  const int G = P.grid;
  const int g_rows = std::min(G, nblk(nb, kWarpRows));
  const int g_upd = std::min(G, nblk(n, kUpdThreads));
  const int g_vec = std::min(G, nblk(n, kThreads));
  double* part_a = P.partial;           // p.q / init r.z
  double* part_b = P.partial + G;       // r.r
  double* part_c = P.partial + 2 * G;   // r.z
  double* part_d = P.partial + 3 * G;   // init b.b
  double shift = 0.0;
  if (pk == OD_PRECOND_JACOBI || pk == OD_PRECOND_BLOCK_JACOBI) {
    OD_KL(s);
    precond_setup_kernel<double><<<nblk(nb, kThreads), kThreads, 0, strm>>>(nb, pk, s->bsr.diag_pos, s->A64, P.pinv);
  } else if (pk == OD_PRECOND_IC0) {
    od_status e = ic0_factor(s);
    if (e != OD_OK) return e;
    shift = P.ic_shift;
  } else if (pk == OD_PRECOND_LDLT) {
    // Preconditioner::Preprocess runs inside every solve (cgSolver.cpp:23)
    od_status e = ldlt_factor(s, nullptr, prm->sainv_eps > 0.0 ? prm->sainv_eps : kLdltSainvDefault,
                              prm->ldlt_eps > 0.0 ? prm->ldlt_eps : kLdltDropDefault);
    if (e != OD_OK) return e;
  } else if (pk == OD_PRECOND_IC) {
    if (s->dofs < 2) {
      set_error("the incomplete Cholesky preconditioner needs at least 2 DOFs");
      return OD_ERR_INVALID_ARG;
    }
    od_status e = ic_factor(s, nullptr, prm->ic_eps > 0.0 ? prm->ic_eps : kIcEpsDefault, prm->ic_relax);
    if (e != OD_OK) return e;
  }
  // applied by triangular sweeps
  const bool swept = pk == OD_PRECOND_IC0 || pk == OD_PRECOND_LDLT || pk == OD_PRECOND_IC;
  if (!swept && P.coop_grid > 0 && !P.disable_persistent) {
    // one cooperative launch for the whole solve
    OD_CUDA(cudaMemsetAsync(P.gbar, 0, sizeof(GridBarrier), strm));
    const int G2 = P.coop_grid;
    const int ngroups = (nb + kRowsPerWarp - 1) / kRowsPerWarp;
    const int warps = G2 * (kPThreads / 32);
    const int need = (ngroups + warps - 1) / warps;   // groups per warp
    const double tol = prm->tol;
    const int maxit = prm->max_iter;
    GridBarrier* gbp = (GridBarrier*)P.gbar;
    const int* rpp = s->bsr.row_ptr;
    const int* colp = s->bsr.col;
    const double* Ap = s->A64;
    double* xp = d_x;
    int pkv = pk;
    void* args[] = {(void*)&nb, (void*)&rpp, (void*)&colp, (void*)&Ap, (void*)&d_b, (void*)&xp, (void*)&P.r,
                    (void*)&P.z, (void*)&P.p, (void*)&P.q, (void*)&pkv, (void*)&P.pinv, (void*)&P.partial,
                    (void*)&tol, (void*)&maxit, (void*)&P.sc, (void*)&gbp, nullptr, (void*)&P.recur};
    // the shared-memory variant when every CTA's rows fit (P.smem_bytes)
    const bool smem = P.smem_bytes > 0 && need <= kSmemGroupsMax;
    void* fn = smem ? (need <= 1 ? (void*)pcg_persistent_kernel<double, 1, true>
                                 : (void*)pcg_persistent_kernel<double, 2, true>)
             : need <= 1 ? (void*)pcg_persistent_kernel<double, 1, false>
             : need <= 2 ? (void*)pcg_persistent_kernel<double, 2, false>
             : need <= 4 ? (void*)pcg_persistent_kernel<double, 4, false>
                         : (void*)pcg_persistent_kernel<double, 0, false>;
    const size_t dyn = smem ? (size_t)P.smem_bytes : 0;
    // The form: pipelined (one grid sync per iteration; its vectors live in
    // registers, so at most two groups per warp) for tolerances down to 1e-9;
    // the recurrence form (q = A z + beta q: two syncs) down to 1e-10; below,
    // cgSolver.cpp's q = A p (three), so no recurrence drift can hold the
    // residual above a very small target
    int recur = P.recur >= 0 ? P.recur
                             : (need <= 2 && prm->tol >= 1e-9 ? 2 : (prm->tol >= 1e-10 ? 1 : 0));
    if (recur == 2 && need > 2) recur = 1;
    args[18] = (void*)&recur;
    const bool prof = s->ctx->profiling && s->ctx->ev_pool.size() >= 2;
    const bool phases = prof && s->ctx->profiling >= 2;
    unsigned long long* profp = phases ? P.prof : nullptr;
    args[17] = (void*)&profp;
    if (prof) OD_CUDA(cudaEventRecord(s->ctx->ev_pool[0], strm));
    OD_KL(s);
    OD_CUDA(cudaLaunchCooperativeKernel(fn, dim3(G2), dim3(kPThreads), args, dyn, strm));
    if (prof) OD_CUDA(cudaEventRecord(s->ctx->ev_pool[1], strm));
    return pcg_finish(s, d_b, d_x, shift, st, true, prof, phases);
  }
  OD_KL(s);
  pcg_init_kernel<double><<<g_rows, kThreads, 0, strm>>>(nb, s->bsr.row_ptr, s->bsr.col, s->A64, d_b, d_x, P.r, P.z,
                                                          P.p, pk, P.pinv, part_c, part_d, part_b);
  int g_rz0 = g_rows;
  if (swept) {
    if (pk == OD_PRECOND_IC0) OD_TRY(ic0_apply(s, P.r, P.z, nullptr));
    else OD_TRY(sweep_apply(s, P.r, P.z, nullptr));
    OD_KL(s);
    pcg_rz_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.r, P.z, part_c, nullptr);
    g_rz0 = g_vec;
    OD_KL(s);
    copy_kernel<<<nblk(n, kThreads), kThreads, 0, strm>>>(n, P.z, P.p);
  }
  OD_KL(s);
  pcg_init_finish<<<1, kThreads, 0, strm>>>(part_c, g_rz0, part_d, part_b, g_rows, prm->tol, prm->max_iter, P.sc);
  OD_CUDA(cudaGetLastError());
  // iterations are queued in chunks; every kernel returns at once after the
  // stop flag is set, and the host reads the flag between chunks
  const int chunk = 16;
  int ev_used = 0, spmv_seen = 0;
  long long launched = 0;
  for (;;) {
    for (int k = 0; k < chunk; k++, launched++) {
      const int slot = (int)(launched & 1);
      const bool prof = s->ctx->profiling && ev_used + 2 <= (int)s->ctx->ev_pool.size();
      if (prof) OD_CUDA(cudaEventRecord(s->ctx->ev_pool[ev_used], strm));
      OD_KL(s);
      pcg_spmv_kernel<double><<<g_rows, kThreads, 0, strm>>>(nb, s->bsr.row_ptr, s->bsr.col, s->A64, P.p, P.q,
                                                              part_a, P.sc);
      if (prof) { OD_CUDA(cudaEventRecord(s->ctx->ev_pool[ev_used + 1], strm)); ev_used += 2; }
      OD_KL(s);
      pcg_update_kernel<<<g_upd, kUpdThreads, 0, strm>>>(n, d_x, P.r, P.z, P.p, P.q, pk, P.pinv, part_a, g_rows,
                                                         part_c, part_b, P.sc, slot);
      int g_rz = g_upd;
      if (swept) {
        if (pk == OD_PRECOND_IC0) OD_TRY(ic0_apply(s, P.r, P.z, P.sc));
        else OD_TRY(sweep_apply(s, P.r, P.z, P.sc));
        OD_KL(s);
        pcg_rz_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.r, P.z, part_c, P.sc);
        g_rz = g_vec;
      }
      OD_KL(s);
      pcg_direction_kernel<<<g_vec, kThreads, 0, strm>>>(n, P.z, P.p, part_c, g_rz, part_b, g_upd, P.sc, slot);
    }
    OD_CUDA(cudaGetLastError());
    OD_CUDA(cudaMemcpyAsync(P.sc_host, P.sc, sizeof(SolveScalars), cudaMemcpyDeviceToHost, strm));
    OD_TRY(sync_stream(s));
    // SpMV launches that did work (the ones after the stop flag returned at
    // once and are not counted)
    for (int k = 0; k + 1 < ev_used; k += 2) {
      float ms = 0.f;
      OD_CUDA(cudaEventElapsedTime(&ms, s->ctx->ev_pool[k], s->ctx->ev_pool[k + 1]));
      if (k / 2 < P.sc_host->iter - spmv_seen) { s->ctx->spmv_ms += ms; s->ctx->spmv_launches++; }
    }
    spmv_seen = P.sc_host->iter;
    ev_used = 0;
    if (P.sc_host->done) break;
  }
  if (pk == OD_PRECOND_LDLT || pk == OD_PRECOND_IC) OD_TRY(sweep_check(s));
  if (pk == OD_PRECOND_IC0) OD_TRY(ic0_check(s));
  return pcg_finish(s, d_b, d_x, shift, st, false, false);
}

// Self-test of the bounded grid barrier: a cooperative launch of two CTAs
// in which CTA 0 never arrives, so the other's wait runs out (kSpinLimit
// polls) and it leaves with the barrier's timeout flag set -- the path every
// persistent kernel takes when a CTA stops answering.
__global__ void selftest_barrier_kernel(GridBarrier* gb, GridBarrier* gb_count, int* failed) {
  if (blockIdx.x == 0) return;
  // the counting barrier of the one-launch PCG, then the generation barrier
  if (threadIdx.x == 0 && !barrier_arrive_wait_count(gb_count, 1)) atomicAdd(failed + 1, 1);
  __syncthreads();
  if (!grid_barrier(gb) && threadIdx.x == 0) atomicAdd(failed, 1);
}

od_status selftest_barrier_timeout(Ctx* c, int* timed_out) {
  *timed_out = 0;
  int dev_coop = 0;
  OD_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, c->device));
  if (!dev_coop) return OD_OK;
  DeviceTemps tmp;
  GridBarrier* gb = nullptr;    // [0] generation barrier, [1] counting barrier
  int* failed = nullptr;
  OD_CUDA(tmp.alloc(&gb, 2 * sizeof(GridBarrier)));
  OD_CUDA(tmp.alloc(&failed, 2 * sizeof(int)));
  OD_CUDA(cudaMemsetAsync(gb, 0, 2 * sizeof(GridBarrier), c->stream));
  OD_CUDA(cudaMemsetAsync(failed, 0, 2 * sizeof(int), c->stream));
  GridBarrier* gb_count = gb + 1;
  void* args[] = {(void*)&gb, (void*)&gb_count, (void*)&failed};
  cudaError_t e = cudaLaunchCooperativeKernel((void*)selftest_barrier_kernel, dim3(2), dim3(32), args, 0, c->stream);
  GridBarrier h[2]{};
  int hf[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, gb, 2 * sizeof(GridBarrier), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hf, failed, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "barrier self-test");
  *timed_out = h[0].timeout == 1 && hf[0] == 1 && h[1].timeout == 1 && hf[1] == 1;
  return OD_OK;
}

}  // namespace od
