// Allocation-free PCG entry point (od_bsr_pcg_noalloc, include/od_gb300.h).
//
// For callers that must not allocate device memory themselves or through
// this library -- a host application whose own allocator owns every byte of
// the GPU, or a plugin whose host forbids allocation after start-up -- this
// entry point solves A x = b for a full block-CSR matrix the caller already
// holds on the device, with every work vector kept in one file-scope device
// array (g_pcg_scratch) of fixed size.  It calls no cudaMalloc, cudaFree or
// allocating library routine.  The call is synchronous: it waits on the
// caller's stream every 16 iterations to read the convergence test, and
// returns when the solve has finished.
//
// The array is shared by every call on a device and keeps the contents of
// the last call; the scalars and counters that must start at zero are reset
// on the caller's stream at the start of each call.  Calls that overlap on
// the GPU (different streams, or another thread) race on the array: callers
// serialise them.
//
// Host code must not pass g_pcg_scratch itself to a kernel (in host code the
// name is a host-side stand-in, not a device address).  The device address
// is looked up with cudaGetSymbolAddress once per device, on the first call
// made with that device current, and kept for the life of the process: a
// cudaDeviceReset of that device after the first call is not supported.
//
// The matrix comes from the caller, so the first kernel checks it before
// any other reads it: a row pointer that does not start at 0 or decreases,
// or a block column outside 0..nb-1, stops the solve with
// OD_ERR_INVALID_ARG (d_row_ptr[nb] must be the length of d_col).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "od_internal.h"

namespace od {
namespace noalloc {

constexpr int kMaxBlockRows = OD_NOALLOC_MAX_BLOCK_ROWS;
constexpr int kMaxN = 3 * kMaxBlockRows;
constexpr int kMaxGrid = 1024;
constexpr int kT = 256;

// scratch layout (doubles)
constexpr size_t kOffR = 0;
constexpr size_t kOffZ = kOffR + kMaxN;
constexpr size_t kOffP = kOffZ + kMaxN;
constexpr size_t kOffQ = kOffP + kMaxN;
constexpr size_t kOffPinv = kOffQ + kMaxN;                 // 9 per block row
constexpr size_t kOffPart = kOffPinv + 9 * (size_t)kMaxBlockRows;  // 3 arrays of kMaxGrid
constexpr size_t kOffScal = kOffPart + 3 * (size_t)kMaxGrid;
constexpr size_t kScratchDoubles = kOffScal + 16;

struct Scal {  // lives at kOffScal (16 doubles)
  double rz[2], rr, bb, eps, tr_num, tr_den;
  int iter, max_iter, done, status;
};
static_assert(sizeof(Scal) <= 16 * sizeof(double), "scalar block too large");

static __device__ __align__(256) double g_pcg_scratch[kScratchDoubles];

__device__ __forceinline__ double block_sum_na(double v) {
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
  return t;
}

// sum of part[0..m) in a fixed order, broadcast to the CTA
__device__ __forceinline__ double sum_parts(const double* part, int m) {
  __shared__ double bc;
  double acc = 0.0;
  for (int j = threadIdx.x; j < m; j += blockDim.x) acc += __ldcg(part + j);
  double t = block_sum_na(acc);
  if (threadIdx.x == 0) bc = t;
  __syncthreads();
  double v = bc;
  __syncthreads();
  return v;
}

// y_row = (A x)_row for one DOF (row of a block row), one thread per DOF
__device__ __forceinline__ double row_dot(int i, const int* __restrict__ rp, const int* __restrict__ col,
                                          const double* __restrict__ A, const double* __restrict__ x) {
  const int br = i / 3, r = i - 3 * br;
  double y = 0.0;
  for (int k = rp[br]; k < rp[br + 1]; k++) {
    const double* a = A + (size_t)k * 9 + 3 * r;
    const int c = 3 * col[k];
    y = fma(a[0], x[c], y);
    y = fma(a[1], x[c + 1], y);
    y = fma(a[2], x[c + 2], y);
  }
  return y;
}

__device__ __forceinline__ double precond_row(int pk, int i, const double* __restrict__ pinv, const double* r) {
  if (pk == OD_PRECOND_JACOBI) return pinv[i] * r[i];
  if (pk == OD_PRECOND_BLOCK_JACOBI) {
    const int br = i / 3, d = i - 3 * br;
    const double* m = pinv + 9 * (size_t)br + 3 * d;
    return m[0] * r[3 * br] + m[1] * r[3 * br + 1] + m[2] * r[3 * br + 2];
  }
  return r[i];
}

// Structure check, before any kernel reads x through the columns: row
// pointers start at 0 and never decrease, every block column lies in
// 0..nb-1.  A violation stops the solve with OD_ERR_INVALID_ARG (the rows
// are not walked further).
__global__ void validate_kernel(int nb, const int* __restrict__ rp, const int* __restrict__ col,
                                double* __restrict__ scratch) {
  Scal* sc = reinterpret_cast<Scal*>(scratch + kOffScal);
  const int br = blockIdx.x * blockDim.x + threadIdx.x;
  if (br >= nb) return;
  const int k0 = rp[br], k1 = rp[br + 1];
  bool bad = (br == 0 && k0 != 0) || k1 < k0;
  for (int k = k0; !bad && k < k1; k++) bad = col[k] < 0 || col[k] >= nb;
  if (bad) {
    sc->status = OD_ERR_INVALID_ARG;
    sc->done = 1;
  }
}

__device__ __forceinline__ bool stopped(const double* scratch) {
  return *(volatile const int*)&reinterpret_cast<const Scal*>(scratch + kOffScal)->done != 0;
}

// Jacobi (1/d, or 1 when d <= 0) or inverse 3x3 diagonal blocks
__global__ void setup_kernel(int nb, int pk, const int* __restrict__ rp, const int* __restrict__ col,
                             const double* __restrict__ A, double* __restrict__ scratch) {
  int br = blockIdx.x * blockDim.x + threadIdx.x;
  if (br >= nb || stopped(scratch)) return;
  double* pinv = scratch + kOffPinv;
  const double* a = nullptr;
  for (int k = rp[br]; k < rp[br + 1]; k++)
    if (col[k] == br) { a = A + (size_t)k * 9; break; }
  double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (a)
    for (int k = 0; k < 9; k++) m[k] = a[k];
  if (pk == OD_PRECOND_JACOBI) {
    for (int d = 0; d < 3; d++) pinv[3 * br + d] = m[4 * d] > 0.0 ? 1.0 / m[4 * d] : 1.0;
  } else {
    const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                       m[2] * (m[3] * m[7] - m[4] * m[6]);
    const double inv = 1.0 / det;
    double* o = pinv + 9 * (size_t)br;
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

// r = b - A x and partial b.b, r.r (the preconditioned pass follows)
__global__ void init_r_kernel(int n, const int* __restrict__ rp, const int* __restrict__ col,
                              const double* __restrict__ A, const double* __restrict__ b,
                              const double* __restrict__ x, double* __restrict__ scratch) {
  if (stopped(scratch)) return;  // CTA-uniform
  double* r = scratch + kOffR;
  double* part = scratch + kOffPart;
  double bb = 0.0, rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double rv = b[i] - row_dot(i, rp, col, A, x);
    r[i] = rv;
    bb = fma(b[i], b[i], bb);
    rr = fma(rv, rv, rr);
  }
  double t0 = block_sum_na(bb), t1 = block_sum_na(rr);
  if (threadIdx.x == 0) { part[blockIdx.x] = t0; part[kMaxGrid + blockIdx.x] = t1; }
}

// z = M^-1 r; p = z; partial r.z
__global__ void init_z_kernel(int n, int pk, double* __restrict__ scratch) {
  if (stopped(scratch)) return;
  const double* r = scratch + kOffR;
  double* z = scratch + kOffZ;
  double* p = scratch + kOffP;
  const double* pinv = scratch + kOffPinv;
  double* part = scratch + kOffPart;
  double rz = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double zv = precond_row(pk, i, pinv, r);
    z[i] = zv;
    p[i] = zv;
    rz = fma(r[i], zv, rz);
  }
  double t = block_sum_na(rz);
  if (threadIdx.x == 0) part[2 * kMaxGrid + blockIdx.x] = t;
}

__global__ void init_finish_kernel(int g, double tol, int max_iter, double* __restrict__ scratch) {
  if (stopped(scratch)) return;  // the structure check failed: its status stands
  const double* part = scratch + kOffPart;
  Scal* sc = reinterpret_cast<Scal*>(scratch + kOffScal);
  const double bb = sum_parts(part, g), rr = sum_parts(part + kMaxGrid, g), rz = sum_parts(part + 2 * kMaxGrid, g);
  if (threadIdx.x == 0) {
    sc->rz[0] = sc->rz[1] = rz;
    sc->bb = bb;
    sc->rr = rr;
    sc->eps = bb * tol * tol;
    sc->iter = 0;
    sc->max_iter = max_iter;
    sc->status = isfinite(rr) ? OD_OK : OD_ERR_NAN;
    sc->done = !(0 < max_iter && rr > sc->eps) || !isfinite(rr);
  }
}

// q = A p; partial p.q
__global__ void spmv_kernel(int n, const int* __restrict__ rp, const int* __restrict__ col,
                            const double* __restrict__ A, double* __restrict__ scratch) {
  const Scal* sc = reinterpret_cast<const Scal*>(scratch + kOffScal);
  if (*(volatile const int*)&sc->done) return;
  const double* p = scratch + kOffP;
  double* q = scratch + kOffQ;
  double* part = scratch + kOffPart;
  double pq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double y = row_dot(i, rp, col, A, p);
    q[i] = y;
    pq = fma(p[i], y, pq);
  }
  double t = block_sum_na(pq);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// alpha = rz / p.q; x += alpha p; r -= alpha q; partial r.r (z follows)
__global__ void update_kernel(int n, int g, int slot, double* __restrict__ x, double* __restrict__ scratch) {
  const Scal* sc = reinterpret_cast<const Scal*>(scratch + kOffScal);
  if (*(volatile const int*)&sc->done) return;
  const double* p = scratch + kOffP;
  const double* q = scratch + kOffQ;
  double* r = scratch + kOffR;
  double* part = scratch + kOffPart;
  const double alpha = sc->rz[slot] / sum_parts(part, g);
  double rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const double rv = fma(-alpha, q[i], r[i]);
    r[i] = rv;
    rr = fma(rv, rv, rr);
  }
  double t = block_sum_na(rr);
  if (threadIdx.x == 0) part[kMaxGrid + blockIdx.x] = t;
}

// z = M^-1 r; partial r.z
__global__ void precond_kernel(int n, int pk, double* __restrict__ scratch) {
  const Scal* sc = reinterpret_cast<const Scal*>(scratch + kOffScal);
  if (*(volatile const int*)&sc->done) return;
  const double* r = scratch + kOffR;
  double* z = scratch + kOffZ;
  const double* pinv = scratch + kOffPinv;
  double* part = scratch + kOffPart;
  double rz = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double zv = precond_row(pk, i, pinv, r);
    z[i] = zv;
    rz = fma(r[i], zv, rz);
  }
  double t = block_sum_na(rz);
  if (threadIdx.x == 0) part[2 * kMaxGrid + blockIdx.x] = t;
}

// beta = rz_new / rz; p = z + beta p; CTA 0 records the iteration
__global__ void direction_kernel(int n, int g, int slot, double* __restrict__ scratch) {
  Scal* sc = reinterpret_cast<Scal*>(scratch + kOffScal);
  if (*(volatile int*)&sc->done) return;
  const double* z = scratch + kOffZ;
  double* p = scratch + kOffP;
  double* part = scratch + kOffPart;
  const double rr = sum_parts(part + kMaxGrid, g);
  const double rz_new = sum_parts(part + 2 * kMaxGrid, g);
  const double beta = rz_new / sc->rz[slot];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = fma(beta, p[i], z[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rz[1 - slot] = rz_new;
    sc->rr = rr;
    const int it = sc->iter + 1;
    sc->iter = it;
    if (!isfinite(rr) || !isfinite(beta)) { sc->status = OD_ERR_NAN; sc->done = 1; }
    else sc->done = !(it < sc->max_iter && rr > sc->eps);
  }
}

// true residual: partials of ||b - A x||^2 and ||b||^2 per CTA (skipped when
// the structure check failed)
__global__ void residual_kernel(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                const double* __restrict__ A, const double* __restrict__ b,
                                const double* __restrict__ x, double* __restrict__ scratch) {
  const Scal* sc = reinterpret_cast<const Scal*>(scratch + kOffScal);
  if (sc->status == OD_ERR_INVALID_ARG) return;
  double* part = scratch + kOffPart;
  double d2 = 0.0, bb = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = b[i] - row_dot(i, rp, col, A, x);
    d2 = fma(d, d, d2);
    bb = fma(b[i], b[i], bb);
  }
  double t0 = block_sum_na(d2), t1 = block_sum_na(bb);
  if (threadIdx.x == 0) { part[blockIdx.x] = t0; part[kMaxGrid + blockIdx.x] = t1; }
}

__global__ void residual_finish_kernel(int g, double* __restrict__ scratch) {
  Scal* sc = reinterpret_cast<Scal*>(scratch + kOffScal);
  if (sc->status == OD_ERR_INVALID_ARG) return;
  const double* part = scratch + kOffPart;
  const double d2 = sum_parts(part, g), bb = sum_parts(part + kMaxGrid, g);
  if (threadIdx.x == 0) { sc->tr_num = d2; sc->tr_den = bb; }
}

// device address of g_pcg_scratch, looked up once per device
constexpr int kMaxDevices = 64;
static double* s_scratch[kMaxDevices];
static std::mutex s_mutex;

static od_status scratch_for_current_device(double** out) {
  int dev = 0;
  OD_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) { set_error("od_bsr_pcg_noalloc: device index out of range"); return OD_ERR_UNSUPPORTED; }
  std::lock_guard<std::mutex> lock(s_mutex);
  if (!s_scratch[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_pcg_scratch);
    if (e != cudaSuccess || !ptr) return cuda_fail(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress");
    s_scratch[dev] = (double*)ptr;
  }
  *out = s_scratch[dev];
  return OD_OK;
}

}  // namespace noalloc
}  // namespace od

using namespace od;
using namespace od::noalloc;

extern "C" od_status od_bsr_pcg_noalloc(int nb, const int* d_row_ptr, const int* d_col, const double* d_values,
                                        const double* d_b, double* d_x, const od_solver_params* params,
                                        void* stream, od_solve_stats* stats) {
  if (!params || !d_row_ptr || !d_col || !d_values || !d_b || !d_x) {
    set_error("od_bsr_pcg_noalloc: NULL argument");
    return OD_ERR_INVALID_ARG;
  }
  if (nb < 1 || nb > kMaxBlockRows) {
    set_error("od_bsr_pcg_noalloc: block row count must be in 1.." + std::to_string(kMaxBlockRows) +
              " (OD_NOALLOC_MAX_BLOCK_ROWS); use od_scene_pcg for larger systems");
    return OD_ERR_INVALID_ARG;
  }
  if (params->precond != OD_PRECOND_NONE && params->precond != OD_PRECOND_JACOBI &&
      params->precond != OD_PRECOND_BLOCK_JACOBI) {
    set_error("od_bsr_pcg_noalloc: only the none, Jacobi and block-Jacobi preconditioners need no allocation");
    return OD_ERR_UNSUPPORTED;
  }
  if (params->precision != OD_PRECISION_FP64 || params->tol < 0.0 || params->max_iter < 0) {
    set_error("od_bsr_pcg_noalloc: FP64 precision, tol >= 0 and max_iter >= 0 required");
    return OD_ERR_INVALID_ARG;
  }
  double* scratch = nullptr;
  od_status st = scratch_for_current_device(&scratch);
  if (st != OD_OK) return st;
  cudaStream_t strm = (cudaStream_t)stream;
  const int n = 3 * nb;
  const int g = std::min(kMaxGrid, std::max(1, (n + kT - 1) / kT));
  const int pk = params->precond;
  // scalars start from zero on every call (the array keeps the last call's contents)
  OD_CUDA(cudaMemsetAsync(scratch + kOffScal, 0, 16 * sizeof(double), strm));
  validate_kernel<<<(nb + kT - 1) / kT, kT, 0, strm>>>(nb, d_row_ptr, d_col, scratch);
  if (pk != OD_PRECOND_NONE) setup_kernel<<<(nb + kT - 1) / kT, kT, 0, strm>>>(nb, pk, d_row_ptr, d_col, d_values, scratch);
  init_r_kernel<<<g, kT, 0, strm>>>(n, d_row_ptr, d_col, d_values, d_b, d_x, scratch);
  init_z_kernel<<<g, kT, 0, strm>>>(n, pk, scratch);
  init_finish_kernel<<<1, kT, 0, strm>>>(g, params->tol, params->max_iter, scratch);
  OD_CUDA(cudaGetLastError());
  Scal h{};
  const Scal* dsc = reinterpret_cast<const Scal*>(scratch + kOffScal);
  long long launched = 0;
  for (;;) {
    for (int k = 0; k < 16; k++, launched++) {
      const int slot = (int)(launched & 1);
      spmv_kernel<<<g, kT, 0, strm>>>(n, d_row_ptr, d_col, d_values, scratch);
      update_kernel<<<g, kT, 0, strm>>>(n, g, slot, d_x, scratch);
      precond_kernel<<<g, kT, 0, strm>>>(n, pk, scratch);
      direction_kernel<<<g, kT, 0, strm>>>(n, g, slot, scratch);
    }
    OD_CUDA(cudaGetLastError());
    OD_CUDA(cudaMemcpyAsync(&h, dsc, sizeof(Scal), cudaMemcpyDeviceToHost, strm));
    OD_CUDA(cudaStreamSynchronize(strm));
    if (h.done) break;
  }
  residual_kernel<<<g, kT, 0, strm>>>(n, d_row_ptr, d_col, d_values, d_b, d_x, scratch);
  residual_finish_kernel<<<1, kT, 0, strm>>>(g, scratch);
  OD_CUDA(cudaGetLastError());
  OD_CUDA(cudaMemcpyAsync(&h, dsc, sizeof(Scal), cudaMemcpyDeviceToHost, strm));
  OD_CUDA(cudaStreamSynchronize(strm));
  od_status status = (od_status)h.status;
  if (status == OD_ERR_INVALID_ARG) {
    set_error("od_bsr_pcg_noalloc: row pointers must start at 0 and not decrease, and every block column "
              "must lie in 0..nb-1");
    if (stats) {
      *stats = od_solve_stats{};
      stats->status = status;
    }
    return status;
  }
  if (status == OD_OK && h.iter >= h.max_iter && h.rr > h.eps) status = OD_ERR_NOT_CONVERGED;
  if (stats) {
    stats->iterations = h.iter;
    stats->refinements = 0;
    stats->rel_residual = h.tr_den > 0.0 ? std::sqrt(h.tr_num / h.tr_den) : std::sqrt(h.tr_num);
    stats->ic_shift = 0.0;
    stats->status = status;
  }
  return status == OD_ERR_NAN ? OD_ERR_NAN : OD_OK;
}
