// Arithmetic-throughput measurement of the device (od_measure_fma_rate).
//
// The FP64 kernels of the step (element evaluation, the FP64 SpMV and PCG)
// are bound by the FP64 pipe on GB300, not by HBM, so their roofline needs
// the device's FP64 multiply-add rate.  This kernel runs a fixed count of
// independent multiply-add chains on every SM at full occupancy and is timed
// with CUDA events on the context stream; the rate is multiply-adds per
// second (one multiply-add = two floating-point operations).  The FP32 rate
// is measured the same way, for the FP32 kernels of the mixed solve.
#include <algorithm>

#include "od_internal.h"

namespace od {

constexpr int kPeakThreads = 256;
constexpr int kPeakChains = 8;  // independent chains per thread

template <class T>
__global__ void __launch_bounds__(kPeakThreads) fma_rate_kernel(int iters, T a, T b, T* __restrict__ out) {
  T x[kPeakChains];
#pragma unroll
  for (int c = 0; c < kPeakChains; c++) x[c] = (T)(threadIdx.x + c) * (T)1e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kPeakChains; c++) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < kPeakChains; c++) s += x[c];
  // a, b come from the host, so the chains cannot be folded; the store keeps them
  if (s == (T)-1.2345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T>
static od_status fma_rate(Ctx* c, int iters, double* fma_per_s, double* ms) {
  int per_sm = 0;
  OD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_rate_kernel<T>, kPeakThreads, 0));
  const int grid = c->num_sms * std::max(1, per_sm);
  DeviceTemps tmp;
  T* out = nullptr;
  OD_CUDA(tmp.alloc(&out, sizeof(T) * (size_t)grid * kPeakThreads));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  OD_CUDA(cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; e == cudaSuccess && rep < 4; rep++) {  // the first launch warms the clocks
    e = cudaEventRecord(e0, c->stream);
    if (e == cudaSuccess) {
      fma_rate_kernel<T><<<grid, kPeakThreads, 0, c->stream>>>(iters, (T)0.999999, (T)1e-7, out);
      c->launches++;
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.f || t < best)) best = t;
  }
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(e, "multiply-add rate kernel");
  const double fmas = (double)grid * kPeakThreads * kPeakChains * (double)iters;
  *ms = best;
  *fma_per_s = best > 0.f ? fmas / (best * 1e-3) : 0.0;
  return OD_OK;
}

}  // namespace od

using namespace od;

extern "C" od_status od_measure_fma_rate(od_ctx* ctx, int fp64, int iters, double* fma_per_s, double* ms) {
  OD_CHECK_ARG(ctx && fma_per_s && ms, "od_measure_fma_rate: NULL argument");
  OD_CHECK_ARG(iters >= 1 && iters <= (1 << 24), "od_measure_fma_rate: iters must be in 1..2^24");
  OD_CUDA(cudaSetDevice(ctx->c.device));
  return fp64 ? fma_rate<double>(&ctx->c, iters, fma_per_s, ms) : fma_rate<float>(&ctx->c, iters, fma_per_s, ms);
}
