// Mixed-precision solve with the IC(0) preconditioner (OD_PRECOND_IC0 with
// OD_PRECISION_MIXED; no reference counterpart).
//
// FP64 outer iterative refinement: r64 = b - A64 x (FP64), the inner solve
// A32 d = r64 / ||r64|| to a relative tolerance, x += ||r64|| d (FP64),
// until ||b - A64 x|| <= tol ||b||.  The inner PCG runs on FP32 data with
// FP32 accumulation -- the SpMV over an FP32 copy of the full block-CSR
// matrix and the IC(0) triangular sweeps over an FP32 copy of the factor --
// while its dot products are accumulated in FP64.  The IC(0) factor itself
// is made in FP64 (the shifted IC(0) of A64 in colour order, exactly as the
// FP64 solve makes it) and rounded to FP32 once per solve.  The inner loop
// is one launch per kernel and iteration (SpMV, update, the one-launch
// sweep, r.z, direction), queued in chunks with the stop flag on the
// device, like the FP64 multi-kernel PCG.
#include <algorithm>
#include <cmath>
#include <vector>

#include "od_grid.cuh"
#include "od_internal.h"

namespace od {

namespace {

constexpr int kT = 256;
constexpr int kRows = 10;   // block rows per warp (3 lanes each)

__device__ __forceinline__ double block_total(double v) {
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;
}

// sum of part[0..m) in a fixed order, the same in every CTA
__device__ __forceinline__ double parts_total(const double* __restrict__ part, int m) {
  __shared__ double bc;
  double acc = 0.0;
  for (int j = threadIdx.x; j < m; j += blockDim.x) acc += __ldcg(part + j);
  const double t = block_total(acc);
  if (threadIdx.x == 0) bc = t;
  __syncthreads();
  const double v = bc;
  __syncthreads();
  return v;
}

__global__ void to_f32_kernel(long long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// r64 = b - q (q = A64 x) and per-CTA partials of r.r, b.b
__global__ void residual64_kernel(int n, const double* __restrict__ b, const double* __restrict__ q,
                                  double* __restrict__ r64, double* __restrict__ part) {
  double rr = 0.0, bb = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double r = b[i] - q[i];
    r64[i] = r;
    rr = fma(r, r, rr);
    bb = fma(b[i], b[i], bb);
  }
  const double t0 = block_total(rr), t1 = block_total(bb);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = t0;
    part[2 * blockIdx.x + 1] = t1;
  }
}

// x += unscale d (FP64)
__global__ void refine_kernel(int n, double unscale, const float* __restrict__ d, double* __restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = fma(unscale, (double)d[i], x[i]);
}

// r = scale r64 (FP32), d = 0; partial r.r
__global__ void inner_init_kernel(int n, double scale, const double* __restrict__ r64, float* __restrict__ r,
                                  float* __restrict__ d, double* __restrict__ part_rr) {
  double rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float v = (float)(scale * r64[i]);
    r[i] = v;
    d[i] = 0.f;
    rr = fma((double)v, (double)v, rr);
  }
  const double t = block_total(rr);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = t;
}

// p = z; partial r.z
__global__ void inner_start_kernel(int n, const float* __restrict__ r, const float* __restrict__ z,
                                   float* __restrict__ p, double* __restrict__ part_rz) {
  double rz = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    p[i] = z[i];
    rz = fma((double)r[i], (double)z[i], rz);
  }
  const double t = block_total(rz);
  if (threadIdx.x == 0) part_rz[blockIdx.x] = t;
}

__global__ void inner_start_finish(int g, const double* __restrict__ part_rz, const double* __restrict__ part_rr,
                                   double itol, int max_iter, SolveScalars* __restrict__ sc) {
  const double rz = parts_total(part_rz, g), rr = parts_total(part_rr, g);
  if (threadIdx.x == 0) {
    sc->rz[0] = sc->rz[1] = rz;
    sc->rr = rr;
    sc->rr0 = rr;
    sc->eps = rr * itol * itol;
    sc->iter = 0;
    sc->max_iter = max_iter;
    sc->status = isfinite(rr) && isfinite(rz) ? OD_OK : OD_ERR_NAN;
    sc->done = !(max_iter > 0 && rr > sc->eps) || sc->status != OD_OK;
  }
}

// q = A32 p with FP32 accumulation (three lanes per block row, one FMA per
// stored value); partial p.q in FP64
__global__ void inner_spmv_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                  const float* __restrict__ A, const float* __restrict__ p, float* __restrict__ q,
                                  double* __restrict__ part_pq, const SolveScalars* __restrict__ sc) {
  if (*(volatile const int*)&sc->done) return;
  const int lane = threadIdx.x & 31;
  double pq = 0.0;
  const int rows_per_cta = (blockDim.x >> 5) * kRows;
  for (int row0 = blockIdx.x * rows_per_cta; row0 < nb; row0 += gridDim.x * rows_per_cta) {
    const int row = row0 + (threadIdx.x >> 5) * kRows + lane / 3;
    const int r = lane % 3;
    if (lane < 3 * kRows && row < nb) {
      float y = 0.f;
      for (int k = rp[row]; k < rp[row + 1]; k++) {
        const float* a = A + (size_t)k * 9 + 3 * r;
        const float* x = p + 3 * (size_t)col[k];
        y = fmaf(a[0], x[0], y);
        y = fmaf(a[1], x[1], y);
        y = fmaf(a[2], x[2], y);
      }
      q[3 * (size_t)row + r] = y;
      pq = fma((double)p[3 * (size_t)row + r], (double)y, pq);
    }
  }
  const double t = block_total(pq);
  if (threadIdx.x == 0) part_pq[blockIdx.x] = t;
}

// alpha = r.z / p.q; d += alpha p; r -= alpha q; partial r.r
__global__ void inner_update_kernel(int n, int g, int slot, const float* __restrict__ p, const float* __restrict__ q,
                                    float* __restrict__ d, float* __restrict__ r, const double* __restrict__ part_pq,
                                    double* __restrict__ part_rr, SolveScalars* __restrict__ sc) {
  if (*(volatile const int*)&sc->done) return;
  const double pq = parts_total(part_pq, g);
  const float alpha = (float)(sc->rz[slot] / pq);
  double rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    d[i] = fmaf(alpha, p[i], d[i]);
    const float v = fmaf(-alpha, q[i], r[i]);
    r[i] = v;
    rr = fma((double)v, (double)v, rr);
  }
  const double t = block_total(rr);
  if (threadIdx.x == 0) {
    part_rr[blockIdx.x] = t;
    if (blockIdx.x == 0 && !(isfinite(pq) && pq != 0.0)) sc->status = OD_ERR_NAN;
  }
}

// partial r.z after the preconditioner apply
__global__ void inner_rz_kernel(int n, const float* __restrict__ r, const float* __restrict__ z,
                                double* __restrict__ part_rz, const SolveScalars* __restrict__ sc) {
  if (*(volatile const int*)&sc->done) return;
  double rz = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    rz = fma((double)r[i], (double)z[i], rz);
  const double t = block_total(rz);
  if (threadIdx.x == 0) part_rz[blockIdx.x] = t;
}

// beta = r.z_new / r.z; p = z + beta p; CTA 0 records the iteration and the stop test
__global__ void inner_direction_kernel(int n, int g, int slot, const float* __restrict__ z, float* __restrict__ p,
                                       const double* __restrict__ part_rz, const double* __restrict__ part_rr,
                                       SolveScalars* __restrict__ sc) {
  if (*(volatile const int*)&sc->done) return;
  const double rz_new = parts_total(part_rz, g), rr = parts_total(part_rr, g);
  const double beta = rz_new / sc->rz[slot];
  const float fb = (float)beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = fmaf(fb, p[i], z[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rz[1 - slot] = rz_new;
    sc->rr = rr;
    const int it = sc->iter + 1;
    sc->iter = it;
    if (!isfinite(rr) || !isfinite(beta) || sc->status != OD_OK) {
      sc->status = OD_ERR_NAN;
      sc->done = 1;
    } else {
      sc->done = !(it < sc->max_iter && rr > sc->eps);
    }
  }
}

int nblocks(long long n) { return (int)std::max(1LL, std::min(4096LL, (n + kT - 1) / kT)); }

}  // namespace

struct MixIc0 {
  int n = 0;
  long long nnz9 = 0, nl = 0;
  float *A32 = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *d = nullptr;
  float *fval = nullptr, *bval = nullptr, *dval = nullptr, *y = nullptr, *zp = nullptr;
  double *r64 = nullptr, *q64 = nullptr, *part = nullptr;
  SolveScalars* sc = nullptr;
  SolveScalars* sc_host = nullptr;
  int g = 0;
  long long bytes = 0;
};

void mixed_ic0_free(MixIc0* m) {
  if (!m) return;
  for (float* v : {m->A32, m->r, m->z, m->p, m->q, m->d, m->fval, m->bval, m->dval, m->y, m->zp}) cudaFree(v);
  for (double* v : {m->r64, m->q64, m->part}) cudaFree(v);
  cudaFree(m->sc);
  if (m->sc_host) cudaFreeHost(m->sc_host);
  delete m;
}

static od_status mixed_ic0_alloc(Scene* s) {
  Pcg& P = s->pcg;
  const int n = P.n_pad;
  const long long nnz9 = 9LL * s->bsr.nnzb, nl = std::max(1LL, (long long)P.ic_nnz - P.ic_n);
  if (P.mic && P.mic->n == n && P.mic->nnz9 == nnz9 && P.mic->nl == nl) return OD_OK;
  mixed_ic0_free(P.mic);
  MixIc0* m = new MixIc0();
  P.mic = m;
  m->n = n;
  m->nnz9 = nnz9;
  m->nl = nl;
  m->g = std::min(nblocks(n), 2 * std::max(1, s->ctx->num_sms));
  auto f = [&](float** v, long long k) {
    m->bytes += 4 * k;
    return cudaMalloc(v, sizeof(float) * (size_t)std::max(1LL, k));
  };
  cudaError_t e = f(&m->A32, nnz9);
  for (float** v : {&m->r, &m->z, &m->p, &m->q, &m->d, &m->dval, &m->y, &m->zp})
    if (e == cudaSuccess) e = f(v, n);
  if (e == cudaSuccess) e = f(&m->fval, nl);
  if (e == cudaSuccess) e = f(&m->bval, nl);
  if (e == cudaSuccess) e = cudaMalloc(&m->r64, sizeof(double) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&m->q64, sizeof(double) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&m->part, sizeof(double) * 4 * (size_t)std::max(m->g, nblocks(n)));
  if (e == cudaSuccess) e = cudaMalloc(&m->sc, sizeof(SolveScalars));
  if (e == cudaSuccess) e = cudaMallocHost(&m->sc_host, sizeof(SolveScalars));
  if (e != cudaSuccess) return cuda_fail(e, "mixed IC(0) buffers");
  m->bytes += 8 * (2LL * n + 4LL * std::max(m->g, nblocks(n)));
  s->device_bytes += m->bytes;
  return OD_OK;
}

od_status mixed_ic0_solve(Scene* s, const double* d_b, double* d_x, const od_solver_params* prm,
                          od_solve_stats* st) {
  Pcg& P = s->pcg;
  Ctx* ctx = s->ctx;
  cudaStream_t strm = ctx->stream;
  // the FP64 factor (colour order), as the FP64 solve makes it
  OD_TRY(ic0_factor(s));
  OD_TRY(mixed_ic0_alloc(s));
  MixIc0* m = P.mic;
  const int n = m->n, nb = s->bsr.nb, g = m->g, gr = nblocks(n);
  ctx->launches += 4;
  to_f32_kernel<<<nblocks(m->nnz9), kT, 0, strm>>>(m->nnz9, s->A64, m->A32);
  to_f32_kernel<<<nblocks(m->nl), kT, 0, strm>>>((long long)P.ic_nnz - P.ic_n, P.ic_fval, m->fval);
  to_f32_kernel<<<nblocks(m->nl), kT, 0, strm>>>((long long)P.ic_nnz - P.ic_n, P.ic_bval, m->bval);
  to_f32_kernel<<<nblocks(P.ic_n), kT, 0, strm>>>(P.ic_n, P.ic_dval, m->dval);
  OD_CUDA(cudaGetLastError());
  SweepView v;
  v.n = P.ic_n;
  v.n_pad = P.n_pad;
  v.ic = 1;
  v.grid = P.ic_grid;
  v.nnz = (long long)P.ic_nnz - P.ic_n;
  v.frp = P.ic_frp;
  v.fci = P.ic_fci;
  v.bcp = P.icT_rp;
  v.bri = P.icT_ci;
  v.ord_f = P.ic_gord_f;
  v.ord_b = P.ic_gord_b;
  v.err = P.ic_err;
  v.perm = P.ic_pdof;
  if (P.ic_by_colour) v.colour_start = &P.ic_cstart;
  const double inner_tol = prm->inner_tol > 0.0 ? prm->inner_tol : 1e-4;
  const int max_refine = prm->max_refine > 0 ? prm->max_refine : 20;
  double* part_a = m->part;           // p.q
  double* part_b = m->part + gr;      // r.r
  double* part_c = m->part + 2 * gr;  // r.z
  int total = 0, sweeps = 0;
  double rr = 0.0, bb = 0.0;
  od_status status = OD_OK;
  for (;;) {
    // FP64 true residual
    OD_TRY(launch_spmv_full(s, d_x, m->q64));
    ctx->launches++;
    residual64_kernel<<<gr, kT, 0, strm>>>(n, d_b, m->q64, m->r64, part_a);
    OD_CUDA(cudaGetLastError());
    std::vector<double> h(2 * (size_t)gr);
    OD_CUDA(cudaMemcpyAsync(h.data(), part_a, sizeof(double) * 2 * gr, cudaMemcpyDeviceToHost, strm));
    OD_TRY(sync_stream(s));
    rr = bb = 0.0;
    for (int k = 0; k < gr; k++) {
      rr += h[2 * k];
      bb += h[2 * k + 1];
    }
    const double eps = bb * prm->tol * prm->tol;
    if (!std::isfinite(rr)) { status = OD_ERR_NAN; break; }
    if (rr <= eps || sweeps >= max_refine || total >= prm->max_iter) break;
    const double rn = std::sqrt(rr);
    const double itol = std::max(inner_tol, std::min(0.5, 0.3 * std::sqrt(eps / rr)));
    // inner FP32 PCG from d = 0 on r = r64 / ||r64||
    ctx->launches += 3;
    inner_init_kernel<<<gr, kT, 0, strm>>>(n, 1.0 / rn, m->r64, m->r, m->d, part_b);
    OD_TRY(sweep_launch_f32(s, v, m->fval, m->bval, m->dval, m->r, m->y, m->z, m->zp, nullptr));
    inner_start_kernel<<<gr, kT, 0, strm>>>(n, m->r, m->z, m->p, part_c);
    inner_start_finish<<<1, kT, 0, strm>>>(gr, part_c, part_b, itol, prm->max_iter - total, m->sc);
    OD_CUDA(cudaGetLastError());
    long long launched = 0;
    for (;;) {
      for (int k = 0; k < 16; k++, launched++) {
        const int slot = (int)(launched & 1);
        ctx->launches += 4;
        inner_spmv_kernel<<<g, kT, 0, strm>>>(nb, s->bsr.row_ptr, s->bsr.col, m->A32, m->p, m->q, part_a, m->sc);
        inner_update_kernel<<<gr, kT, 0, strm>>>(n, g, slot, m->p, m->q, m->d, m->r, part_a, part_b, m->sc);
        OD_TRY(sweep_launch_f32(s, v, m->fval, m->bval, m->dval, m->r, m->y, m->z, m->zp, m->sc));
        inner_rz_kernel<<<gr, kT, 0, strm>>>(n, m->r, m->z, part_c, m->sc);
        inner_direction_kernel<<<gr, kT, 0, strm>>>(n, gr, slot, m->z, m->p, part_c, part_b, m->sc);
      }
      OD_CUDA(cudaGetLastError());
      OD_CUDA(cudaMemcpyAsync(m->sc_host, m->sc, sizeof(SolveScalars), cudaMemcpyDeviceToHost, strm));
      OD_TRY(sync_stream(s));
      if (m->sc_host->done) break;
    }
    OD_TRY(ic0_check(s));
    total += m->sc_host->iter;
    sweeps++;
    if (m->sc_host->status != OD_OK) { status = (od_status)m->sc_host->status; break; }
    ctx->launches++;
    refine_kernel<<<gr, kT, 0, strm>>>(n, rn, m->d, d_x);
    OD_CUDA(cudaGetLastError());
    if (m->sc_host->iter == 0) break;   // no progress possible
  }
  if (status == OD_OK && rr > bb * prm->tol * prm->tol) status = OD_ERR_NOT_CONVERGED;
  if (st) {
    st->iterations = total;
    st->refinements = sweeps;
    st->rel_residual = bb > 0.0 ? std::sqrt(rr / bb) : std::sqrt(rr);
    st->ic_shift = P.ic_shift;
    st->status = status;
  }
  return status == OD_ERR_NAN ? OD_ERR_NAN : OD_OK;
}

}  // namespace od
