// Modal (reduced) linear Newmark: the path of intergrator/linearNewmark.cpp.
//
// Setup (LinearNewmark::LinearNewmark, linearNewmark.cpp:8-50): the Hooke
// stiffness K (material/hooke.cpp:18-60, assembled on the device by the
// element gather) and the scene's consistent mass M; then the n_modes
// eigenpairs of K phi = lambda M phi nearest zero.  The reference obtains
// them from ARPACK in shift-invert mode at 0 with a SuperLU factorisation
// of K (core/eigensolver.cpp:8-13).  Here the same spectral transformation,
// OP = K^-1 M (self-adjoint in the M inner product, its largest eigenvalues
// theta = 1 / lambda), runs as a thick-restart Lanczos iteration on the
// device: every OP apply is one FP64 block-Jacobi PCG solve with K (the
// persistent cooperative solver), the basis Q and Y = M Q live in HBM, each
// new vector is M-orthogonalised against the whole basis twice (classical
// Gram-Schmidt, the inner products as one multi-dot launch), and the small
// projected matrix T = Q^T M OP Q is diagonalised on the host (cyclic
// Jacobi).  At a restart the wanted Ritz vectors and the last basis vector
// are kept (T becomes an arrow matrix).  A Ritz pair (theta, Q s) has the
// residual |beta_m s_m| in the M norm; it has converged when that is below
// tol * theta.
//
// Steps (runOneTimeStep, linearNewmark.cpp:57-79) update every mode's
// (d, v, a) with the reference's predictor-corrector; one launch runs any
// number of steps (the modes are independent).  Displacements and
// velocities are sum_i d_i phi_i (getFullOrderProperties, :81-92) on the
// device, then scattered to the node layout.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "od_internal.h"

namespace od {
namespace {

constexpr int kMT = 256;           // threads of the vector kernels
constexpr int kDotChunk = 16384;   // DOFs per partial sum of the multi-dot

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[kMT / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < kMT / 32; k++) t += ws[k];
  return t;  // thread 0
}

// part[i * nch + c] = sum over chunk c of V[i][t] w[t], for i < nv
__global__ void __launch_bounds__(kMT) mdot_partial_kernel(int n, long long ld, const double* __restrict__ V,
                                                           const double* __restrict__ w, int nch,
                                                           double* __restrict__ part) {
  const int i = blockIdx.y, c = blockIdx.x;
  const double* v = V + (size_t)i * ld;
  const int t1 = min(n, (c + 1) * kDotChunk);
  double acc = 0.0;
  for (int t = c * kDotChunk + threadIdx.x; t < t1; t += kMT) acc = fma(v[t], w[t], acc);
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[(size_t)i * nch + c] = acc;
}

// h[i] = sum of the chunk partials of vector i, in chunk order
__global__ void mdot_finish_kernel(int nv, int nch, const double* __restrict__ part, double* __restrict__ h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  double acc = 0.0;
  for (int c = 0; c < nch; c++) acc += part[(size_t)i * nch + c];
  h[i] = acc;
}

// w[t] -= sum_i Q[i][t] h[i] (i < nv, in order)
__global__ void __launch_bounds__(kMT) reorth_kernel(int n, int nv, long long ld, const double* __restrict__ Q,
                                                     const double* __restrict__ h, double* __restrict__ w) {
  const int t = blockIdx.x * kMT + threadIdx.x;
  if (t >= n) return;
  double acc = w[t];
  for (int i = 0; i < nv; i++) acc = fma(-Q[(size_t)i * ld + t], h[i], acc);
  w[t] = acc;
}

__global__ void scale_kernel(int n, const double* __restrict__ a, double sc, double* __restrict__ x) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) x[t] = a[t] * sc;
}

// out[c][t] = sum_i V[i][t] S[i * k + c] for c < k (i < m, in order)
__global__ void __launch_bounds__(kMT) combine_kernel(int n, int m, int k, long long ld, const double* __restrict__ V,
                                                      const double* __restrict__ S, double* __restrict__ out) {
  const int t = blockIdx.x * kMT + threadIdx.x;
  const int c = blockIdx.y;
  if (t >= n) return;
  double acc = 0.0;
  for (int i = 0; i < m; i++) acc = fma(V[(size_t)i * ld + t], S[(size_t)i * k + c], acc);
  out[(size_t)c * ld + t] = acc;
}

// seeded start vector on the free DOFs (splitmix64 of the index), zero on
// the padding
__global__ void random_kernel(int n, int dofs, unsigned long long seed, double* __restrict__ x) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(t + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  x[t] = t < dofs ? (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5 : 0.0;
}

// runOneTimeStep of every mode, steps times (linearNewmark.cpp:57-79);
// st = [d | v | a | f | lambda], n_modes each
__global__ void modal_step_kernel(int r, int steps, double* __restrict__ st, double h, double betaDeltaT2,
                                  double gammaDeltaT, double minusBetaDeltaT2, double minusGammaDeltaT,
                                  double alpha_m, double beta_k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r) return;
  double d = st[i], v = st[r + i], a = st[2 * r + i];
  const double f = st[3 * r + i], w2 = st[4 * r + i];
  for (int k = 0; k < steps; k++) {
    const double d_predict = d + h * v + minusBetaDeltaT2 * a;
    const double v_predict = v + minusGammaDeltaT * a;
    const double xi = alpha_m + beta_k * w2;
    const double righthand = f - xi * v_predict - w2 * d_predict;
    const double lefthand = 1.0 + gammaDeltaT * xi + betaDeltaT2 * w2;
    a = righthand / lefthand;
    v = v_predict + gammaDeltaT * a;
    d = d_predict + betaDeltaT2 * a;
  }
  st[i] = d;
  st[r + i] = v;
  st[2 * r + i] = a;
}

// full-order values of the reduced vector c: sum_i c_i phi_i (i in order),
// written to the node layout (constrained entries: base, or zero)
__global__ void __launch_bounds__(kMT) full_order_kernel(int n3, int r, long long ld, const int* __restrict__ node_dof,
                                                         const double* __restrict__ Phi,
                                                         const double* __restrict__ c,
                                                         const double* __restrict__ base, double* __restrict__ out) {
  const int p = blockIdx.x * kMT + threadIdx.x;
  if (p >= n3) return;
  const int t = node_dof[p];
  if (t < 0) {
    out[p] = base ? base[p] : 0.0;
    return;
  }
  double acc = 0.0;
  for (int i = 0; i < r; i++) acc += c[i] * Phi[(size_t)i * ld + t];
  out[p] = acc;
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// eigen-decomposition of the symmetric n x n matrix A (row-major, destroyed):
// cyclic Jacobi rotations until the off-diagonal mass is negligible; w the
// eigenvalues, V (row-major, column j the eigenvector of w[j])
void sym_eig(int n, std::vector<double>& A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) V[(size_t)i * n + i] = 1.0;
  auto at = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; i++) {
      diag += at(i, i) * at(i, i);
      for (int j = i + 1; j < n; j++) off += at(i, j) * at(i, j);
    }
    if (off <= 1e-32 * diag || off == 0.0) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = at(p, q);
        if (apq == 0.0) continue;
        // rotation that zeroes A[p][q] (Golub and Van Loan, symmetric Schur 2x2)
        const double tau = (at(q, q) - at(p, p)) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; k++) {
          const double akp = at(k, p), akq = at(k, q);
          at(k, p) = c * akp - s * akq;
          at(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          const double apk = at(p, k), aqk = at(q, k);
          at(p, k) = c * apk - s * aqk;
          at(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; i++) w[i] = at(i, i);
}

}  // namespace

struct ModalSys {
  Scene* s = nullptr;
  od_modal_params p{};
  int r = 0, m = 0, n = 0, np = 0;
  long long ld = 0;
  double* Kh = nullptr;       // Hooke stiffness, reference value layout
  double* Q = nullptr;        // (m + 1) x ld Lanczos basis
  double* Y = nullptr;        // (m + 1) x ld, M Q
  double* Q2 = nullptr;       // restart targets
  double* Y2 = nullptr;
  double* w = nullptr;        // new direction, M w
  double* sv = nullptr;
  double* part = nullptr;     // multi-dot partials
  double* h = nullptr;        // multi-dot results (m + 1)
  double* S = nullptr;        // Ritz coefficients on the device (m x m)
  double* phi = nullptr;      // r x ld modes
  double* st = nullptr;       // reduced state [d | v | a | f | lambda]
  double* full = nullptr;     // node-layout output (3 n_nodes)
  int nch = 0;
  std::vector<double> lambda;
  od_modal_info info{};
  ~ModalSys() {
    for (double* v : {Kh, Q, Y, Q2, Y2, w, sv, part, h, S, phi, st, full}) cudaFree(v);
  }
};

namespace {

// h[0..nv) = V[0..nv)^T x on the device
od_status mdot(ModalSys& M, const double* V, int nv, const double* x) {
  cudaStream_t strm = M.s->ctx->stream;
  OD_KL(M.s);
  mdot_partial_kernel<<<dim3(M.nch, nv), kMT, 0, strm>>>(M.n, M.ld, V, x, M.nch, M.part);
  OD_KL(M.s);
  mdot_finish_kernel<<<nblk(nv, 128), 128, 0, strm>>>(nv, M.nch, M.part, M.h);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status mass_apply(ModalSys& M, const double* x, double* y) {
  return launch_spmv_lower(M.s, M.s->M, 1.0, x, nullptr, 0.0, nullptr, nullptr, 0.0, nullptr, y, false);
}

// M-normalise x into Q[j] / Y[j]; returns its M norm in *nrm
od_status normalise_into(ModalSys& M, double* x, int j, double* nrm) {
  cudaStream_t strm = M.s->ctx->stream;
  OD_TRY(mass_apply(M, x, M.sv));
  OD_TRY(mdot(M, x, 1, M.sv));
  double hh = 0.0;
  OD_CUDA(cudaMemcpyAsync(&hh, M.h, sizeof(double), cudaMemcpyDeviceToHost, strm));
  OD_TRY(sync_stream(M.s));
  *nrm = std::sqrt(std::max(hh, 0.0));
  if (!(*nrm > 0.0) || !std::isfinite(*nrm)) return OD_OK;
  OD_KL(M.s);
  scale_kernel<<<nblk(M.np, kMT), kMT, 0, strm>>>(M.np, x, 1.0 / *nrm, M.Q + (size_t)j * M.ld);
  OD_KL(M.s);
  scale_kernel<<<nblk(M.np, kMT), kMT, 0, strm>>>(M.np, M.sv, 1.0 / *nrm, M.Y + (size_t)j * M.ld);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

// two classical Gram-Schmidt passes of w against Q[0..nv) in the M inner
// product; hsum receives the summed coefficients
od_status orthogonalise(ModalSys& M, int nv, std::vector<double>& hsum) {
  cudaStream_t strm = M.s->ctx->stream;
  hsum.assign(nv, 0.0);
  std::vector<double> hh(nv);
  for (int pass = 0; pass < 2; pass++) {
    OD_TRY(mdot(M, M.Y, nv, M.w));
    OD_KL(M.s);
    reorth_kernel<<<nblk(M.n, kMT), kMT, 0, strm>>>(M.n, nv, M.ld, M.Q, M.h, M.w);
    OD_CUDA(cudaGetLastError());
    OD_CUDA(cudaMemcpyAsync(hh.data(), M.h, sizeof(double) * nv, cudaMemcpyDeviceToHost, strm));
    OD_TRY(sync_stream(M.s));
    for (int i = 0; i < nv; i++) hsum[i] += hh[i];
  }
  return OD_OK;
}

od_status modal_setup(ModalSys& M) {
  Scene* s = M.s;
  cudaStream_t strm = s->ctx->stream;
  const od_modal_params& p = M.p;
  // K (Hooke) into the scene's working matrix
  OD_TRY(launch_hooke(s, p.youngs, p.poisson, M.Kh));
  OD_TRY(launch_expand(s, M.Kh, 1.0, nullptr, 0.0, nullptr, 0.0));
  od_solver_params sp{};
  sp.tol = p.inner_tol;
  sp.max_iter = p.inner_max_iter;
  sp.precond = OD_PRECOND_BLOCK_JACOBI;
  sp.precision = OD_PRECISION_FP64;

  const int m = M.m, r = M.r;
  std::vector<double> T((size_t)(m + 1) * (m + 1), 0.0), hs, theta, Sv;
  auto Tat = [&](int i, int j) -> double& { return T[(size_t)i * (m + 1) + j]; };
  // start vector
  OD_KL(s);
  random_kernel<<<nblk(M.np, kMT), kMT, 0, strm>>>(M.np, M.n, 0x0DDEF0E5ull, M.w);
  OD_CUDA(cudaGetLastError());
  double nrm = 0.0;
  OD_TRY(normalise_into(M, M.w, 0, &nrm));
  if (!(nrm > 0.0)) {
    set_error("od_modal_create: the mass matrix gives the start vector no norm");
    return OD_ERR_INVALID_ARG;
  }
  int k = 0;  // vectors kept by the last restart
  std::vector<int> order(m);
  for (int restart = 0;; restart++) {
    for (int j = k; j < m; j++) {
      // w = K^-1 M q_j
      OD_CUDA(cudaMemsetAsync(M.w, 0, sizeof(double) * M.np, strm));
      od_solve_stats ss{};
      OD_TRY(pcg_solve(s, M.Y + (size_t)j * M.ld, M.w, &sp, &ss));
      M.info.pcg_iterations += ss.iterations;
      M.info.lanczos_steps++;
      if (ss.status != OD_OK) {
        set_error("od_modal_create: a shift-invert PCG solve with the Hooke stiffness did not converge");
        return ss.status == OD_ERR_NOT_CONVERGED ? OD_ERR_NOT_CONVERGED : (od_status)ss.status;
      }
      OD_TRY(orthogonalise(M, j + 1, hs));
      for (int i = 0; i <= j; i++) Tat(i, j) = Tat(j, i) = hs[i];
      double beta = 0.0;
      OD_TRY(normalise_into(M, M.w, j + 1, &beta));
      if (!(beta > 1e-300) || !std::isfinite(beta)) {
        // invariant subspace: continue with a fresh random direction
        OD_KL(s);
        random_kernel<<<nblk(M.np, kMT), kMT, 0, strm>>>(M.np, M.n, 0x5EEDull + (unsigned long long)j, M.w);
        OD_CUDA(cudaGetLastError());
        OD_TRY(mass_apply(M, M.w, M.sv));
        OD_TRY(orthogonalise(M, j + 1, hs));
        double nn = 0.0;
        OD_TRY(normalise_into(M, M.w, j + 1, &nn));
        if (!(nn > 0.0)) {
          set_error("od_modal_create: the Lanczos basis lost rank");
          return OD_ERR_NAN;
        }
        beta = 0.0;
      }
      Tat(j + 1, j) = Tat(j, j + 1) = beta;
    }
    // Ritz pairs of the m x m projection, largest theta first
    std::vector<double> A((size_t)m * m);
    for (int i = 0; i < m; i++)
      for (int j = 0; j < m; j++) A[(size_t)i * m + j] = Tat(i, j);
    sym_eig(m, A, theta, Sv);
    for (int i = 0; i < m; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return theta[a] > theta[b]; });
    const double beta_m = Tat(m, m - 1);
    double worst = 0.0;
    bool ok = true;
    for (int c = 0; c < r; c++) {
      const int o = order[c];
      const double th = theta[o];
      const double res = std::fabs(beta_m * Sv[(size_t)(m - 1) * m + o]);
      const double rel = th > 0.0 ? res / th : INFINITY;
      worst = std::max(worst, rel);
      if (!(th > 0.0) || !(rel <= p.tol)) ok = false;
    }
    M.info.max_residual = worst;
    M.info.restarts = restart;
    const bool last = ok || restart >= p.max_restarts;
    const int keep = last ? r : r + (m - r) / 2;
    // Ritz coefficients of the kept pairs, m x keep
    std::vector<double> Sk((size_t)m * keep);
    for (int i = 0; i < m; i++)
      for (int c = 0; c < keep; c++) Sk[(size_t)i * keep + c] = Sv[(size_t)i * m + order[c]];
    OD_CUDA(cudaMemcpyAsync(M.S, Sk.data(), sizeof(double) * Sk.size(), cudaMemcpyHostToDevice, strm));
    if (last) {
      if (!ok) {
        set_error("od_modal_create: the Lanczos iteration did not converge within max_restarts");
        return OD_ERR_NOT_CONVERGED;
      }
      OD_KL(s);
      combine_kernel<<<dim3(nblk(M.n, kMT), r), kMT, 0, strm>>>(M.n, m, r, M.ld, M.Q, M.S, M.phi);
      OD_CUDA(cudaGetLastError());
      // M-normalise each mode (Ritz vectors of an M-orthonormal basis are
      // M-orthonormal up to rounding)
      M.lambda.resize(r);
      for (int c = 0; c < r; c++) {
        double* ph = M.phi + (size_t)c * M.ld;
        OD_TRY(mass_apply(M, ph, M.sv));
        OD_TRY(mdot(M, ph, 1, M.sv));
        double hh = 0.0;
        OD_CUDA(cudaMemcpyAsync(&hh, M.h, sizeof(double), cudaMemcpyDeviceToHost, strm));
        OD_TRY(sync_stream(s));
        OD_KL(s);
        scale_kernel<<<nblk(M.n, kMT), kMT, 0, strm>>>(M.n, ph, 1.0 / std::sqrt(hh), ph);
        M.lambda[c] = 1.0 / theta[order[c]];
      }
      OD_CUDA(cudaGetLastError());
      return OD_OK;
    }
    // thick restart: Q <- [Q S_keep, q_m], T <- arrow(theta, beta_m s_m)
    OD_KL(s);
    combine_kernel<<<dim3(nblk(M.n, kMT), keep), kMT, 0, strm>>>(M.n, m, keep, M.ld, M.Q, M.S, M.Q2);
    OD_KL(s);
    combine_kernel<<<dim3(nblk(M.n, kMT), keep), kMT, 0, strm>>>(M.n, m, keep, M.ld, M.Y, M.S, M.Y2);
    OD_CUDA(cudaGetLastError());
    OD_CUDA(cudaMemcpyAsync(M.Q2 + (size_t)keep * M.ld, M.Q + (size_t)m * M.ld, sizeof(double) * M.ld,
                            cudaMemcpyDeviceToDevice, strm));
    OD_CUDA(cudaMemcpyAsync(M.Y2 + (size_t)keep * M.ld, M.Y + (size_t)m * M.ld, sizeof(double) * M.ld,
                            cudaMemcpyDeviceToDevice, strm));
    std::swap(M.Q, M.Q2);
    std::swap(M.Y, M.Y2);
    std::fill(T.begin(), T.end(), 0.0);
    for (int c = 0; c < keep; c++) {
      Tat(c, c) = theta[order[c]];
      Tat(keep, c) = Tat(c, keep) = beta_m * Sv[(size_t)(m - 1) * m + order[c]];
    }
    k = keep;
  }
}

}  // namespace
}  // namespace od

struct od_modal {
  od::ModalSys m;
};

using namespace od;

od_status od_modal_create(od_scene* scene, const od_modal_params* params, od_modal** out) {
  OD_CHECK_ARG(scene && params && out, "od_modal_create: NULL argument");
  *out = nullptr;
  Scene* s = &scene->s;
  const od_modal_params& q = *params;
  OD_CHECK_ARG(q.n_modes >= 1 && q.n_modes < s->dofs, "od_modal_create: need 1 <= n_modes < scene dofs");
  OD_CHECK_ARG(q.dt > 0.0 && std::isfinite(q.dt), "od_modal_create: dt must be positive");
  OD_CHECK_ARG(q.youngs > 0.0 && q.poisson > -1.0 && q.poisson < 0.5,
               "od_modal_create: need youngs > 0 and -1 < poisson < 0.5");
  OD_CHECK_ARG(q.krylov == 0 || (q.krylov > q.n_modes + 1 && q.krylov <= s->dofs),
               "od_modal_create: krylov must exceed n_modes + 1 and not exceed the scene dofs");
  OD_CHECK_ARG(q.tol >= 0.0 && q.inner_tol >= 0.0 && q.inner_max_iter >= 0 && q.max_restarts >= 0,
               "od_modal_create: negative tolerance or limit");
  OD_CUDA(cudaSetDevice(s->ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  od_modal* h = new od_modal;
  ModalSys& M = h->m;
  M.s = s;
  M.p = q;
  if (M.p.tol == 0.0) M.p.tol = 1e-10;
  if (M.p.inner_tol == 0.0) M.p.inner_tol = 1e-12;
  if (M.p.inner_max_iter == 0) M.p.inner_max_iter = 100000;
  if (M.p.max_restarts == 0) M.p.max_restarts = 200;
  M.r = q.n_modes;
  M.m = q.krylov ? q.krylov : std::min(s->dofs, std::max(2 * q.n_modes + 10, q.n_modes + 20));
  if (M.m <= M.r + 1) M.m = std::min(s->dofs, M.r + 2);
  M.n = s->dofs;
  M.np = s->pcg.n_pad;
  M.ld = (M.np + 31) / 32 * 32;
  M.nch = std::max(1, nblk(M.n, kDotChunk));
  auto fail = [&](od_status st) {
    delete h;
    return st;
  };
  if (M.m <= M.r) {
    set_error("od_modal_create: the scene has too few DOFs for the requested modes");
    return fail(OD_ERR_INVALID_ARG);
  }
  cudaError_t e = cudaSuccess;
  const size_t basis = (size_t)(M.m + 1) * M.ld;
  auto alloc = [&](double** ptr, size_t count) {
    if (e == cudaSuccess) e = cudaMalloc(ptr, sizeof(double) * std::max<size_t>(1, count));
    if (e == cudaSuccess) e = cudaMemset(*ptr, 0, sizeof(double) * std::max<size_t>(1, count));
  };
  alloc(&M.Kh, (size_t)s->nvals);
  alloc(&M.Q, basis);
  alloc(&M.Y, basis);
  alloc(&M.Q2, basis);
  alloc(&M.Y2, basis);
  alloc(&M.w, (size_t)M.ld);
  alloc(&M.sv, (size_t)M.ld);
  alloc(&M.part, (size_t)(M.m + 1) * M.nch);
  alloc(&M.h, (size_t)M.m + 1);
  alloc(&M.S, (size_t)M.m * M.m);
  alloc(&M.phi, (size_t)M.r * M.ld);
  alloc(&M.st, 5 * (size_t)M.r);
  alloc(&M.full, 3 * (size_t)s->n_nodes);
  if (e != cudaSuccess) return fail(cuda_fail(e, "od_modal_create"));
  const od_status st = modal_setup(M);
  if (st != OD_OK) return fail(st);
  // reduced state: zero d, v, a, f; lambda
  std::vector<double> hst(5 * (size_t)M.r, 0.0);
  for (int i = 0; i < M.r; i++) hst[4 * (size_t)M.r + i] = M.lambda[i];
  e = cudaMemcpyAsync(M.st, hst.data(), sizeof(double) * hst.size(), cudaMemcpyHostToDevice, s->ctx->stream);
  if (e != cudaSuccess) return fail(cuda_fail(e, "od_modal_create"));
  const od_status ss = sync_stream(s);
  if (ss != OD_OK) return fail(ss);
  // the Lanczos buffers are no longer needed
  for (double** v : {&M.Q, &M.Y, &M.Q2, &M.Y2}) {
    cudaFree(*v);
    *v = nullptr;
  }
  M.info.n_modes = M.r;
  M.info.dofs = M.n;
  M.info.krylov = M.m;
  M.info.setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  *out = h;
  return OD_OK;
}

od_status od_modal_destroy(od_modal* modal) {
  if (!modal) return OD_OK;
  cudaSetDevice(modal->m.s->ctx->device);
  delete modal;
  return OD_OK;
}

od_status od_modal_set_external_forces(od_modal* modal, const double* f_ext) {
  OD_CHECK_ARG(modal, "od_modal_set_external_forces: modal is NULL");
  ModalSys& M = modal->m;
  Scene* s = M.s;
  cudaStream_t strm = s->ctx->stream;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  const double* f = s->fext;
  if (f_ext) {
    OD_CUDA(cudaMemsetAsync(M.w, 0, sizeof(double) * M.ld, strm));
    OD_CUDA(cudaMemcpyAsync(M.w, f_ext, sizeof(double) * M.n, cudaMemcpyHostToDevice, strm));
    f = M.w;
  }
  OD_TRY(mdot(M, M.phi, M.r, f));
  // the modal forces, and a = f (linearNewmark.cpp:52-55)
  OD_CUDA(cudaMemcpyAsync(M.st + 3 * (size_t)M.r, M.h, sizeof(double) * M.r, cudaMemcpyDeviceToDevice, strm));
  OD_CUDA(cudaMemcpyAsync(M.st + 2 * (size_t)M.r, M.h, sizeof(double) * M.r, cudaMemcpyDeviceToDevice, strm));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_modal_step(od_modal* modal, int steps) {
  OD_CHECK_ARG(modal && steps >= 0, "od_modal_step: NULL modal or negative step count");
  ModalSys& M = modal->m;
  Scene* s = M.s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  if (steps == 0) return OD_OK;
  const double h = M.p.dt;
  // the reference's constants (linearNewmark.cpp:27-30)
  const double betaDeltaT2 = M.p.beta * h * h;
  const double gammaDeltaT = M.p.gamma * h;
  const double minusBetaDeltaT2 = h * h * 0.5 - betaDeltaT2;
  const double minusGammaDeltaT = h - gammaDeltaT;
  OD_KL(s);
  modal_step_kernel<<<nblk(M.r, 128), 128, 0, s->ctx->stream>>>(M.r, steps, M.st, h, betaDeltaT2, gammaDeltaT,
                                                                minusBetaDeltaT2, minusGammaDeltaT, M.p.alpha_m,
                                                                M.p.beta_k);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

static od_status modal_full(od_modal* modal, int which, double* out, const char* what) {
  OD_CHECK_ARG(modal && out, what);
  ModalSys& M = modal->m;
  Scene* s = M.s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  const int n3 = 3 * s->n_nodes;
  OD_KL(s);
  full_order_kernel<<<nblk(n3, kMT), kMT, 0, s->ctx->stream>>>(n3, M.r, M.ld, s->node_dof, M.phi,
                                                                M.st + (size_t)which * M.r,
                                                                which == 0 ? s->u : nullptr, M.full);
  OD_CUDA(cudaGetLastError());
  OD_CUDA(cudaMemcpyAsync(out, M.full, sizeof(double) * n3, cudaMemcpyDeviceToHost, s->ctx->stream));
  OD_TRY(sync_stream(s));
  return OD_OK;
}

od_status od_modal_get_displacements(od_modal* modal, double* u) {
  return modal_full(modal, 0, u, "od_modal_get_displacements: NULL argument");
}

od_status od_modal_get_velocities(od_modal* modal, double* v) {
  return modal_full(modal, 1, v, "od_modal_get_velocities: NULL argument");
}

od_status od_modal_get_modes(od_modal* modal, double* lambda, double* basis) {
  OD_CHECK_ARG(modal && lambda, "od_modal_get_modes: NULL argument");
  ModalSys& M = modal->m;
  for (int i = 0; i < M.r; i++) lambda[i] = M.lambda[i];
  if (basis) {
    OD_CUDA(cudaSetDevice(M.s->ctx->device));
    OD_CUDA(cudaMemcpy2DAsync(basis, sizeof(double) * M.n, M.phi, sizeof(double) * M.ld, sizeof(double) * M.n, M.r,
                              cudaMemcpyDeviceToHost, M.s->ctx->stream));
    OD_TRY(sync_stream(M.s));
  }
  return OD_OK;
}

od_status od_modal_get_state(od_modal* modal, double* d, double* v, double* a) {
  OD_CHECK_ARG(modal, "od_modal_get_state: modal is NULL");
  ModalSys& M = modal->m;
  OD_CUDA(cudaSetDevice(M.s->ctx->device));
  std::vector<double> h(3 * (size_t)M.r);
  OD_CUDA(cudaMemcpyAsync(h.data(), M.st, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, M.s->ctx->stream));
  OD_TRY(sync_stream(M.s));
  if (d) std::memcpy(d, h.data(), sizeof(double) * M.r);
  if (v) std::memcpy(v, h.data() + M.r, sizeof(double) * M.r);
  if (a) std::memcpy(a, h.data() + 2 * (size_t)M.r, sizeof(double) * M.r);
  return OD_OK;
}

od_status od_modal_get_stiffness(od_modal* modal, double* values) {
  OD_CHECK_ARG(modal && values, "od_modal_get_stiffness: NULL argument");
  ModalSys& M = modal->m;
  OD_CUDA(cudaSetDevice(M.s->ctx->device));
  OD_CUDA(cudaMemcpyAsync(values, M.Kh, sizeof(double) * M.s->nvals, cudaMemcpyDeviceToHost, M.s->ctx->stream));
  OD_TRY(sync_stream(M.s));
  return OD_OK;
}

od_status od_modal_get_info(od_modal* modal, od_modal_info* info) {
  OD_CHECK_ARG(modal && info, "od_modal_get_info: NULL argument");
  *info = modal->m.info;
  return OD_OK;
}
