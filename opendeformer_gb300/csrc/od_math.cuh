// Per-element 3x3 kernels on the device: symmetric eigensolve, Givens QR,
// quaternion polar decomposition, invertible SVD, PSD projections.
//
// Templated on the floating type; FT = double reproduces the reference's
// double-precision branches and thresholds, FT = float its float ones
// (the reference's templates carry both, core/numerMethod.h).  Matrices are
// row-major 3x3 in registers.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace od {

template <class FT> struct Consts;
template <> struct Consts<double> {
  static constexpr double newton_eps = 1e-12;      // numerMethod.h:730
  static constexpr double omega_eps = 6.607e-8;    // numerMethod.h:873
  static constexpr double rr_eps = 1e-15;          // numerMethod.h:966
  static constexpr double tiny = 2.2250738585072014e-308;
  static constexpr double nit_a = 15.0, nit_b = 16.86;
};
template <> struct Consts<float> {
  static constexpr float newton_eps = 1e-6f;
  static constexpr float omega_eps = 3.388e-4f;
  static constexpr float rr_eps = 1e-7f;
  static constexpr float tiny = 1.17549435e-38f;
  static constexpr float nit_a = 7.0f, nit_b = 8.12f;
};

template <class FT> struct V3t { FT x, y, z; };

template <class FT> __device__ __forceinline__ V3t<FT> v_sub(V3t<FT> a, V3t<FT> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class FT> __device__ __forceinline__ FT v_dot(V3t<FT> a, V3t<FT> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class FT> __device__ __forceinline__ V3t<FT> v_cross(V3t<FT> a, V3t<FT> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class FT> __device__ __forceinline__ V3t<FT> v_scale(V3t<FT> a, FT s) { return {a.x * s, a.y * s, a.z * s}; }
// division as multiplication by the reciprocal (core/latool.h:51-55)
template <class FT> __device__ __forceinline__ V3t<FT> v_div(V3t<FT> a, FT s) { FT r = FT(1) / s; return {r * a.x, r * a.y, r * a.z}; }
template <class FT> __device__ __forceinline__ FT v_len2(V3t<FT> a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
template <class FT> __device__ __forceinline__ FT clampv(FT v, FT lo, FT hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <class FT> __device__ __forceinline__ FT det3(const FT* m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}
template <class FT> __device__ __forceinline__ void mul3(const FT* a, const FT* b, FT* c) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}

// Symmetric 3x3 eigen-decomposition, eigenvectors as rows
// (eigenSym3x3, core/numerMethod.h:327-429): trigonometric root for the
// first eigenvalue, then a 2x2 problem on its orthogonal complement.
// REFINE (FT = double): the trigonometric root in FP32, then two Newton
// steps on the deviator's characteristic polynomial l^3 - J2 l - J3 (the
// chosen root is the one of largest magnitude, where the derivative
// 3 l^2 - J2 is at least 2 J2, so the FP32 start's ~1e-7 error falls below
// FP64 rounding); FP64 transcendental functions are long instruction
// sequences on the FP64 pipe.
template <class FT, bool REFINE = false>
__device__ void eig_sym3(const FT* t, FT* vals, FT* vecs) {
  const FT pi = FT(3.141592653589793238462643383279502884);
  const FT s3 = FT(1.7320508075688772935274463415058723669428);
  // REFINE: fewer FP64 divisions and square roots below (a product by a
  // reciprocal, one root per normalised vector): the same values to an ulp
  const FT ave = REFINE ? (t[0] + t[3] + t[5]) * FT(1.0 / 3.0) : (t[0] + t[3] + t[5]) / FT(3);
  const FT d0 = t[0] - ave, d1 = t[3] - ave, d2 = t[5] - ave;
  const FT J2 = (d0 * d0 + d1 * d1 + d2 * d2) * FT(0.5) + t[1] * t[1] + t[2] * t[2] + t[4] * t[4];
  const FT J3 = d0 * (d1 * d2 - t[4] * t[4]) + t[1] * (t[4] * t[2] - t[1] * d2) + t[2] * (t[1] * t[4] - d1 * t[2]);
  const FT sq = sqrt(J2);
  const FT cs = REFINE ? (FT(3) * FT(0.5) * s3) * (J3 / (J2 * sq)) : (FT(3) * FT(0.5) * s3) * ((J3 / J2) / sq);
  if (isnan(cs) || isinf(cs)) {
    vals[0] = vals[1] = vals[2] = ave;
#pragma unroll
    for (int i = 0; i < 9; i++) vecs[i] = FT(0);
    vecs[0] = vecs[4] = vecs[8] = FT(1);
    return;
  }
  FT e0;
  if constexpr (REFINE) {
    const float pif = 3.14159265358979f;
    const float angf = acosf((float)clampv(cs, FT(-1), FT(1))) / 3.f;
    const float cf = angf < pif / 6.f ? cosf(angf) : cosf(angf + (2.f / 3.f) * pif);
    e0 = (FT(2) / s3) * sq * (FT)cf;
    const FT rdp = FT(1) / (FT(3) * e0 * e0 - J2);
    e0 -= ((e0 * e0 - J2) * e0 - J3) * rdp;
    e0 -= ((e0 * e0 - J2) * e0 - J3) * rdp;
  } else {
    FT ang = acos(clampv(cs, FT(-1), FT(1))) / FT(3);
    e0 = (FT(2) / s3) * sq * (ang < pi / FT(6) ? cos(ang) : cos(ang + (FT(2) / FT(3)) * pi));
  }
  vals[0] = e0 + ave;
  V3t<FT> r0 = {d0 - e0, t[1], t[2]}, r1 = {t[1], d1 - e0, t[4]}, r2 = {t[2], t[4], d2 - e0};
  // REFINE: the same choices on squared lengths, one reciprocal root
  auto unit = [&](V3t<FT> v, FT len2) { return REFINE ? v_scale(v, rsqrt(len2)) : v_div(v, sqrt(len2)); };
  FT l0 = v_len2(r0), l1 = v_len2(r1), l2 = v_len2(r2);
  if constexpr (!REFINE) {
    l0 = sqrt(l0);
    l1 = sqrt(l1);
    l2 = sqrt(l2);
  }
  auto norm0 = [&](V3t<FT> v, FT l) { return REFINE ? v_scale(v, rsqrt(l)) : v_div(v, l); };
  V3t<FT> s0, t1, t2;
  if (l0 > l1) {
    if (l0 > l2) { s0 = norm0(r0, l0); t1 = v_sub(r1, v_scale(s0, v_dot(s0, r1))); t2 = v_sub(r2, v_scale(s0, v_dot(s0, r2))); }
    else { s0 = norm0(r2, l2); t1 = v_sub(r0, v_scale(s0, v_dot(s0, r0))); t2 = v_sub(r1, v_scale(s0, v_dot(s0, r1))); }
  } else {
    if (l1 > l2) { s0 = norm0(r1, l1); t1 = v_sub(r0, v_scale(s0, v_dot(s0, r0))); t2 = v_sub(r2, v_scale(s0, v_dot(s0, r2))); }
    else { s0 = norm0(r2, l2); t1 = v_sub(r0, v_scale(s0, v_dot(s0, r0))); t2 = v_sub(r1, v_scale(s0, v_dot(s0, r1))); }
  }
  FT t1l = v_len2(t1), t2l = v_len2(t2);
  V3t<FT> s1 = t1l > t2l ? unit(t1, t1l) : unit(t2, t2l);
  V3t<FT> ev0 = v_cross(s0, s1);
  vecs[0] = ev0.x; vecs[1] = ev0.y; vecs[2] = ev0.z;
  auto mulm = [&](V3t<FT> v) {
    return V3t<FT>{d0 * v.x + t[1] * v.y + t[2] * v.z, t[1] * v.x + d1 * v.y + t[4] * v.z, t[2] * v.x + t[4] * v.y + d2 * v.z};
  };
  V3t<FT> m0 = mulm(s0), m1 = mulm(s1);
  FT a11 = v_dot(s0, m0), a12 = v_dot(s0, m1), a22 = v_dot(s1, m1);
  FT disc = sqrt((a11 - a22) * (a11 - a22) + FT(4) * a12 * a12);
  FT e1 = ((a11 + a22) - (a11 > a22 ? disc : -disc)) / FT(2);
  FT e2 = a11 + a22 - e1;
  vals[1] = e1 + ave;
  vals[2] = e2 + ave;
  V3t<FT> u0 = v_cross(v_sub(m0, v_scale(s0, e1)), ev0);
  V3t<FT> u1 = v_cross(v_sub(m1, v_scale(s1, e1)), ev0);
  FT u0l = v_len2(u0), u1l = v_len2(u1);
  V3t<FT> ev1 = (u0l != FT(0)) ? (u0l > u1l ? unit(u0, u0l) : unit(u1, u1l)) : s0;
  vecs[3] = ev1.x; vecs[4] = ev1.y; vecs[5] = ev1.z;
  V3t<FT> ev2 = v_cross(ev0, ev1);
  vecs[6] = ev2.x; vecs[7] = ev2.y; vecs[8] = ev2.z;
}

template <class FT>
__device__ __forceinline__ void givens(FT a, FT b, FT& c, FT& s, FT& r) {
  if (b == FT(0)) { c = a < FT(0) ? FT(-1) : FT(1); s = FT(0); r = fabs(a); }
  else if (a == FT(0)) { c = FT(0); s = b < FT(0) ? FT(1) : FT(-1); r = fabs(b); }
  else if (fabs(b) > fabs(a)) {
    FT tau = -a / b, u = sqrt(FT(1) + tau * tau);
    if (b < FT(0)) u = -u;
    s = -FT(1) / u; c = s * tau; r = b * u;
  } else {
    FT tau = -b / a, u = sqrt(FT(1) + tau * tau);
    if (a < FT(0)) u = -u;
    c = FT(1) / u; s = c * tau; r = a * u;
  }
}

// proper QR by three Givens rotations (properQRDecompostion3x3,
// core/numerMethod.h:431-507); returns the orthogonal factor only
template <class FT>
__device__ void qr3(const FT* m, FT* Q) {
  FT R[9];
#pragma unroll
  for (int i = 0; i < 9; i++) { R[i] = m[i]; Q[i] = FT(0); }
  FT c = 0, s = 0, r = 0;
  givens(R[3], R[6], c, s, r);
  Q[4] = Q[8] = c; Q[5] = s; Q[7] = -s;
  R[3] = r; R[6] = FT(0);
#pragma unroll
  for (int i = 0; i < 2; i++) {
    FT p = c * R[4 + i] - s * R[7 + i], q = s * R[4 + i] + c * R[7 + i];
    R[4 + i] = p; R[7 + i] = q;
  }
  givens(R[0], R[3], c, s, r);
  R[0] = r; R[3] = FT(0);
#pragma unroll
  for (int i = 0; i < 2; i++) {
    FT p = c * R[1 + i] - s * R[4 + i], q = s * R[1 + i] + c * R[4 + i];
    R[1 + i] = p; R[4 + i] = q;
  }
  Q[0] = c; Q[1] = s;
  Q[3] = Q[4] * -s; Q[4] *= c;
  Q[6] = Q[7] * -s; Q[7] *= c;
  givens(R[4], R[7], c, s, r);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    FT p = c * Q[3 * i + 1] - s * Q[3 * i + 2], q = s * Q[3 * i + 1] + c * Q[3 * i + 2];
    Q[3 * i + 1] = p; Q[3 * i + 2] = q;
  }
}

// Householder orthonormalisation of two 4-vectors (numerMethod.h:510-567)
template <class FT>
__device__ void orthonormalize2(FT* mat) {
  const FT tol = Consts<FT>::tiny;
  FT beta0 = 0, beta1 = 0, v0[3], v1[2];
  v0[0] = mat[1]; v0[1] = mat[2]; v0[2] = mat[3];
  FT n2 = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
  if (n2 <= tol) { v0[0] = v0[1] = v0[2] = FT(0); }
  else {
    FT c0 = mat[0], sg = sqrt(c0 * c0 + n2);
    if (c0 >= FT(0)) sg = -sg;
    FT f = c0 - sg;
    v0[0] /= f; v0[1] /= f; v0[2] /= f;
    beta0 = (sg - c0) / sg;
  }
  FT prod = mat[4] + v0[0] * mat[5] + v0[1] * mat[6] + v0[2] * mat[7];
  FT c0 = mat[5] - prod * beta0 * v0[0];
  v1[0] = mat[6] - prod * beta0 * v0[1];
  v1[1] = mat[7] - prod * beta0 * v0[2];
  n2 = v1[0] * v1[0] + v1[1] * v1[1];
  if (n2 <= tol) { v1[0] = v1[1] = FT(0); }
  else {
    FT sg = sqrt(c0 * c0 + n2);
    if (c0 >= FT(0)) sg = -sg;
    FT f = c0 - sg;
    v1[0] /= f; v1[1] /= f;
    beta1 = (sg - c0) / sg;
  }
  mat[0] = FT(1) - beta0; mat[1] = -beta0 * v0[0]; mat[2] = -beta0 * v0[1]; mat[3] = -beta0 * v0[2];
  FT S[9], l[3];
  S[0] = FT(1) - beta0 * v0[0] * v0[0];
  S[1] = -beta0 * v0[0] * v0[1]; S[3] = S[1];
  S[2] = -beta0 * v0[0] * v0[2]; S[6] = S[2];
  S[4] = FT(1) - beta0 * v0[1] * v0[1];
  S[5] = -beta0 * v0[1] * v0[2]; S[7] = S[5];
  S[8] = FT(1) - beta0 * v0[2] * v0[2];
  l[0] = FT(1) - beta1; l[1] = -beta1 * v1[0]; l[2] = -beta1 * v1[1];
  mat[4] = mat[1] * l[0] + mat[2] * l[1] + mat[3] * l[2];
  mat[5] = S[0] * l[0] + S[1] * l[1] + S[2] * l[2];
  mat[6] = S[3] * l[0] + S[4] * l[1] + S[5] * l[2];
  mat[7] = S[6] * l[0] + S[7] * l[1] + S[8] * l[2];
}

// Orthogonal polar factor R of F (polarDecompostion3x3,
// core/numerMethod.h:570-1016): Higham & Noferini's quaternion method.  The
// rotation of A = F/||F|| is the dominant eigenvector of a symmetric 4x4 B(A);
// its eigenvalue is the largest root of x^4 - 2x^2 - 8 det(A) x + b with
// b = 1 - 4 ||adj A||^2 (closed form, or Newton from sqrt 3 when b is near
// -1/3); the eigenvector follows from an LDL^T of B + lambda I with diagonal
// pivoting and one of: the closed form (quick path), inverse iteration, or a
// 2-vector subspace iteration with a Rayleigh-Ritz step.  R has
// det R = sign(det F).
template <class FT>
__device__ void polar3(const FT* F, FT* R) {
  FT A[9], B[16];
  FT fn = FT(0);
#pragma unroll
  for (int i = 0; i < 9; i++) fn += F[i] * F[i];
  fn = sqrt(fn);
  if (fn == FT(0)) {
#pragma unroll
    for (int i = 0; i < 9; i++) R[i] = FT(0);
    R[0] = R[4] = R[8] = FT(1);
    return;
  }
#pragma unroll
  for (int i = 0; i < 9; i++) A[i] = F[i] / fn;
  FT b = FT(0), t;
  t = A[4] * A[8] - A[5] * A[7]; b += t * t;
  t = A[3] * A[8] - A[5] * A[6]; b += t * t;
  t = A[3] * A[7] - A[4] * A[6]; b += t * t;
  t = A[1] * A[8] - A[2] * A[7]; b += t * t;
  t = A[0] * A[8] - A[2] * A[6]; b += t * t;
  t = A[0] * A[7] - A[1] * A[6]; b += t * t;
  t = A[1] * A[5] - A[2] * A[4]; b += t * t;
  t = A[0] * A[5] - A[2] * A[3]; b += t * t;
  t = A[0] * A[4] - A[1] * A[3]; b += t * t;
  b = FT(1) - FT(4) * b;
  B[0] = -A[0] - A[4] - A[8]; B[1] = -A[5] + A[7]; B[2] = -A[6] + A[2]; B[3] = -A[1] + A[3];
  B[4] = B[1]; B[5] = -A[0] + A[4] + A[8]; B[6] = -A[1] - A[3]; B[7] = -A[2] - A[6];
  B[8] = B[2]; B[9] = B[6]; B[10] = -A[4] + A[0] + A[8]; B[11] = -A[5] - A[7];
  B[12] = B[3]; B[13] = B[7]; B[14] = B[11]; B[15] = -A[8] + A[0] + A[4];

  FT dA = FT(1), omega = FT(0);
  const FT tau = FT(1e-4);
  const bool quick = b <= FT(1) - tau;
  if (quick) {
    int perm0 = 1, perm1 = 2;
    int rowIndex = 0;
    FT largest = fabs(A[0]);
    if (fabs(A[3]) > largest) { largest = fabs(A[3]); rowIndex = 1; }
    if (fabs(A[6]) > largest) rowIndex = 2;
    if (rowIndex != 0) { dA = -dA; if (rowIndex == 1) perm0 = 0; else perm1 = 0; }
    const int row = rowIndex;
    FT piv = A[row * 3];
    dA *= piv;
    if (dA != FT(0)) {
      FT lo = A[perm0 * 3] / piv;
      A[perm0 * 3 + 1] -= lo * A[row * 3 + 1];
      A[perm0 * 3 + 2] -= lo * A[row * 3 + 2];
      lo = A[perm1 * 3] / piv;
      A[perm1 * 3 + 1] -= lo * A[row * 3 + 1];
      A[perm1 * 3 + 2] -= lo * A[row * 3 + 2];
      int r2, s2;
      if (fabs(A[perm0 * 3 + 1]) > fabs(A[perm1 * 3 + 1])) { r2 = perm0; s2 = perm1; }
      else { dA = -dA; r2 = perm1; s2 = perm0; }
      FT p2 = A[r2 * 3 + 1];
      dA *= p2;
      FT lo2 = A[s2 * 3 + 1] / p2;
      dA *= (A[s2 * 3 + 2] - lo2 * A[r2 * 3 + 2]);
    }
  } else {
    int rp[3] = {0, 1, 2}, cp[3] = {0, 1, 2};
    for (int i = 0; i < 2; i++) {
      FT largest = FT(0);
      int ri = i, ci = i;
      for (int j = i; j < 3; j++)
        for (int k = i; k < 3; k++) {
          FT e = fabs(A[rp[j] * 3 + cp[k]]);
          if (e > largest) { largest = e; ri = j; ci = k; }
        }
      if (rp[i] != rp[ri]) { int tt = rp[i]; rp[i] = rp[ri]; rp[ri] = tt; dA = -dA; }
      if (cp[i] != cp[ci]) { int tt = cp[i]; cp[i] = cp[ci]; cp[ci] = tt; dA = -dA; }
      int row = rp[i], col = cp[i];
      FT piv = A[row * 3 + col];
      dA *= piv;
      if (dA == FT(0)) break;
      for (int j = i + 1; j < 3; j++) {
        int sr = rp[j];
        FT lo = A[sr * 3 + col] / piv;
        for (int k = i + 1; k < 3; k++) A[sr * 3 + cp[k]] -= lo * A[row * 3 + cp[k]];
      }
    }
    dA *= A[rp[2] * 3 + cp[2]];
    omega = fabs(A[rp[1] * 3 + cp[1]]);
  }
  const bool notpd = dA < FT(0);
  if (notpd) {
    dA = -dA;
#pragma unroll
    for (int i = 0; i < 16; i++) B[i] = -B[i];
  }
  const FT inv3 = FT(0.333333333333333333333333);
  FT lam;
  if (b >= tau - inv3) {
    FT c = FT(8) * dA;
    FT D0 = FT(1) + FT(3) * b;
    FT D1 = FT(-1) + (FT(27) / FT(16)) * c * c + FT(9) * b;
    FT sD0 = sqrt(D0);
    FT al = D1 / (D0 * sD0);
    FT z = (FT(4) * inv3) * (FT(1) + sD0 * cos(acos(clampv(al, FT(-1), FT(1))) * inv3));
    FT s = sqrt(z) * FT(0.5);
    FT arg = FT(4) - z + c / s;
    lam = s + FT(0.5) * sqrt(arg > FT(0) ? arg : FT(0));
  } else {
    lam = FT(1.7320508075688772935274463415058723669428);
    FT old;
    const FT c = FT(8) * dA;
    int guard = 0;
    do {
      FT p = lam * (lam * (lam * lam - FT(2)) - c) + b;
      FT dp = lam * (FT(4) * lam * lam - FT(4)) - c;
      old = lam;
      lam -= p / dp;
    } while (old - lam > Consts<FT>::newton_eps && ++guard < 100);
  }
  B[0] += lam; B[5] += lam; B[10] += lam; B[15] += lam;

  FT L[6];
  int ix[4] = {0, 1, 2, 3};
  {
    int di = 0;
    FT largest = B[0];
    for (int j = 1; j < 4; j++) {
      FT dd = B[ix[j] * 5];
      if (dd > largest) { largest = dd; di = j; }
    }
    if (di != 0) { int tt = ix[0]; ix[0] = ix[di]; ix[di] = tt; }
    int p = ix[0];
    L[0] = B[p * 4 + ix[1]] / largest;
    L[1] = B[p * 4 + ix[2]] / largest;
    L[2] = B[p * 4 + ix[3]] / largest;
    int r = ix[1], c;
    FT od;
    B[r * 5] -= L[0] * B[p * 4 + r];
    c = ix[2]; od = B[r * 4 + c] - L[0] * B[p * 4 + c]; B[r * 4 + c] = od; B[c * 4 + r] = od;
    c = ix[3]; od = B[r * 4 + c] - L[0] * B[p * 4 + c]; B[r * 4 + c] = od; B[c * 4 + r] = od;
    r = ix[2];
    B[r * 5] -= L[1] * B[p * 4 + r];
    c = ix[3]; od = B[r * 4 + c] - L[1] * B[p * 4 + c]; B[r * 4 + c] = od; B[c * 4 + r] = od;
    r = ix[3];
    B[r * 5] -= L[2] * B[p * 4 + r];
  }
  {
    int di = 1, p = ix[1];
    FT largest = B[p * 5];
    for (int j = 2; j < 4; j++) {
      FT dd = B[ix[j] * 5];
      if (dd > largest) { largest = dd; di = j; }
    }
    if (di != 1) {
      int tt = ix[1]; ix[1] = ix[di]; ix[di] = tt;
      FT tl = L[0]; L[0] = L[di - 1]; L[di - 1] = tl;
    }
    p = ix[1];
    L[3] = B[p * 4 + ix[2]] / largest;
    L[4] = B[p * 4 + ix[3]] / largest;
    int r = ix[2], c = ix[3];
    B[r * 5] -= L[3] * B[p * 4 + r];
    FT od = B[r * 4 + c] - L[3] * B[p * 4 + c];
    B[r * 4 + c] = od; B[c * 4 + r] = od;
    r = ix[3];
    B[r * 5] -= L[4] * B[p * 4 + r];
  }

  FT v[4];
  if (quick) {
    if (B[ix[2] * 5] < B[ix[3] * 5]) {
      int tt = ix[2]; ix[2] = ix[3]; ix[3] = tt;
      FT tl = L[1]; L[1] = L[2]; L[2] = tl;
      tl = L[3]; L[3] = L[4]; L[4] = tl;
    }
    L[5] = B[ix[2] * 4 + ix[3]] / B[ix[2] * 5];
    v[ix[0]] = L[0] * L[4] + L[1] * L[5] - L[0] * L[5] * L[3] - L[2];
    v[ix[1]] = L[5] * L[3] - L[4];
    v[ix[2]] = -L[5];
    v[ix[3]] = FT(1);
  } else {
    const FT b22 = B[ix[2] * 5], b33 = B[ix[3] * 5], b23 = B[ix[2] * 4 + ix[3]];
    const FT dd = b22 * b33 - b23 * b23;
    if (dd == FT(0)) {
      if (b22 == FT(0) && b33 == FT(0) && b23 == FT(0)) {
        v[ix[0]] = L[0] * L[4] - L[2];
        v[ix[1]] = -L[4];
        v[ix[2]] = FT(0); v[ix[3]] = FT(1);
      } else {
        FT aa = -b23, bb = b22, nn = sqrt(aa * aa + bb * bb);
        aa /= nn; bb /= nn;
        v[ix[3]] = bb; v[ix[2]] = aa;
        v[ix[1]] = -L[4] * bb - L[3] * aa;
        v[ix[0]] = -L[2] * bb - L[1] * aa - L[0] * v[ix[1]];
      }
    } else {
      const FT ID[5] = {FT(1) / B[ix[0] * 5], FT(1) / B[ix[1] * 5], b33, -b23, b22};
      const FT IL[5] = {-L[0], L[0] * L[3] - L[1], L[0] * L[4] - L[2], -L[3], -L[4]};
      if (omega > Consts<FT>::omega_eps) {
        FT w[4] = {IL[2], IL[4], FT(0), FT(1)};
        int nit = (int)ceil(Consts<FT>::nit_a / (Consts<FT>::nit_b + FT(2) * log10(omega)));
        for (int it = 0; it < nit; it++) {
          FT nn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
#pragma unroll
          for (int i = 0; i < 4; i++) w[i] /= nn;
          FT w1 = w[1];
          w[1] = IL[0] * w[0] + w1;
          w[2] = IL[1] * w[0] + IL[3] * w1 + w[2];
          w[3] = IL[2] * w[0] + IL[4] * w1 + w[3];
          w[0] *= ID[0]; w[1] *= ID[1];
          FT w2 = w[2];
          w[2] = (ID[2] * w2 + ID[3] * w[3]) / dd;
          w[3] = (ID[3] * w2 + ID[4] * w[3]) / dd;
          w[0] = w[0] + IL[0] * w[1] + IL[1] * w[2] + IL[2] * w[3];
          w[1] = w[1] + IL[3] * w[2] + IL[4] * w[3];
        }
        v[ix[0]] = w[0]; v[ix[1]] = w[1]; v[ix[2]] = w[2]; v[ix[3]] = w[3];
      } else {
        FT w[8] = {IL[1], IL[3], FT(1), FT(0), IL[2], IL[4], FT(0), FT(1)};
        orthonormalize2(w);
        for (int it = 0; it < 2; it++) {
          FT w1 = w[1];
          w[1] = IL[0] * w[0] + w1;
          w[2] = IL[1] * w[0] + IL[3] * w1 + w[2];
          w[3] = IL[2] * w[0] + IL[4] * w1 + w[3];
          FT w5 = w[5];
          w[5] = IL[0] * w[4] + w5;
          w[6] = IL[1] * w[4] + IL[3] * w5 + w[6];
          w[7] = IL[2] * w[4] + IL[4] * w5 + w[7];
          w[0] *= ID[0]; w[1] *= ID[1];
          FT w2 = w[2];
          w[2] = (ID[2] * w2 + ID[3] * w[3]) / dd;
          w[3] = (ID[3] * w2 + ID[4] * w[3]) / dd;
          // the second vector's second entry is scaled by ID[2], as the
          // reference does (numerMethod.h:928)
          w[4] *= ID[0]; w[5] *= ID[2];
          FT w6 = w[6];
          w[6] = (ID[2] * w6 + ID[3] * w[7]) / dd;
          w[7] = (ID[3] * w6 + ID[4] * w[7]) / dd;
          w[0] = w[0] + IL[0] * w[1] + IL[1] * w[2] + IL[2] * w[3];
          w[1] = w[1] + IL[3] * w[2] + IL[4] * w[3];
          w[4] = w[4] + IL[0] * w[5] + IL[1] * w[6] + IL[2] * w[7];
          w[5] = w[5] + IL[3] * w[6] + IL[4] * w[7];
        }
        orthonormalize2(w);
        FT t0[8], t1[8], BB[3];
        t0[0] = w[0] + L[0] * w[1] + L[1] * w[2] + L[2] * w[3];
        t0[1] = w[1] + L[3] * w[2] + L[4] * w[3];
        t0[2] = w[2]; t0[3] = w[3];
        t0[4] = w[4] + L[0] * w[5] + L[1] * w[6] + L[2] * w[7];
        t0[5] = w[5] + L[3] * w[6] + L[4] * w[7];
        t0[6] = w[6]; t0[7] = w[7];
        const FT d00 = B[ix[0] * 5], d11 = B[ix[1] * 5];
        t1[0] = t0[0] * d00; t1[1] = t0[1] * d11;
        t1[2] = t0[2] * b22 + t0[3] * b23; t1[3] = t0[2] * b23 + t0[3] * b33;
        t1[4] = t0[4] * d00; t1[5] = t0[5] * d11;
        t1[6] = t0[6] * b22 + t0[7] * b23; t1[7] = t0[6] * b23 + t0[7] * b33;
        BB[0] = t1[0] * t0[0] + t1[1] * t0[1] + t1[2] * t0[2] + t1[3] * t0[3];
        BB[1] = t1[0] * t0[4] + t1[1] * t0[5] + t1[2] * t0[6] + t1[3] * t0[7];
        BB[2] = t1[4] * t0[4] + t1[5] * t0[5] + t1[6] * t0[6] + t1[7] * t0[7];
        if (fabs(BB[1]) > Consts<FT>::rr_eps) {
          FT r = (BB[0] - BB[2]) * FT(0.5);
          FT w0 = r - sqrt(r * r + BB[1] * BB[1]);
#pragma unroll
          for (int i = 0; i < 4; i++) v[ix[i]] = w[i] * w0 + w[4 + i] * BB[1];
        } else if (BB[0] < BB[2]) {
#pragma unroll
          for (int i = 0; i < 4; i++) v[ix[i]] = w[i];
        } else {
#pragma unroll
          for (int i = 0; i < 4; i++) v[ix[i]] = w[4 + i];
        }
      }
    }
  }
  FT nn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
#pragma unroll
  for (int i = 0; i < 4; i++) v[i] /= nn;
  const FT v11 = v[1] * v[1], v22 = v[2] * v[2], v33 = v[3] * v[3];
  const FT v12 = v[1] * v[2], v03 = v[0] * v[3], v13 = v[1] * v[3];
  const FT v02 = v[0] * v[2], v23 = v[2] * v[3], v01 = v[0] * v[1];
  const FT sg = notpd ? FT(-1) : FT(1);
  // R = Q^T with Q the quaternion rotation (numerMethod.h:993-1007)
  R[0] = sg * (FT(1) - FT(2) * (v22 + v33)); R[3] = sg * (FT(2) * (v12 - v03)); R[6] = sg * (FT(2) * (v13 + v02));
  R[1] = sg * (FT(2) * (v12 + v03)); R[4] = sg * (FT(1) - FT(2) * (v11 + v33)); R[7] = sg * (FT(2) * (v23 - v01));
  R[2] = sg * (FT(2) * (v13 - v02)); R[5] = sg * (FT(2) * (v23 + v01)); R[8] = sg * (FT(1) - FT(2) * (v11 + v22));
}

// coordinateSystem (core/latool.h:542-552)
template <class FT>
__device__ __forceinline__ void coord_system(V3t<FT> v0, V3t<FT>& v1, V3t<FT>& v2) {
  if (fabs(v0.x) > fabs(v0.y)) {
    FT il = FT(1) / sqrt(v0.x * v0.x + v0.z * v0.z);
    v1 = {-v0.z * il, FT(0), v0.x * il};
  } else {
    FT il = FT(1) / sqrt(v0.y * v0.y + v0.z * v0.z);
    v1 = {FT(0), -v0.z * il, v0.y * il};
  }
  v2 = v_cross(v0, v1);
}

// Invertible SVD (modifiedDeformGradient, invertibleHyperelastic.cpp:116-245):
// U from eig(F F^T) made a rotation; V^T = U^T F / sigma with rank-deficient
// rows completed by cross products; the smallest sigma negated when det V < 0;
// sigma clamped below by thr.  Outputs U (row-major), VT, sigma.
template <class FT, bool REFINE = false>
__device__ void invertible_svd(const FT* F, FT thr, FT* sig, FT* U, FT* VT) {
  FT tri[6], ev[3], UT[9];
  tri[0] = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
  tri[1] = F[3] * F[0] + F[4] * F[1] + F[5] * F[2];
  tri[2] = F[6] * F[0] + F[7] * F[1] + F[8] * F[2];
  tri[3] = F[3] * F[3] + F[4] * F[4] + F[5] * F[5];
  tri[4] = F[6] * F[3] + F[7] * F[4] + F[8] * F[5];
  tri[5] = F[6] * F[6] + F[7] * F[7] + F[8] * F[8];
  eig_sym3<FT, REFINE>(tri, ev, UT);
  if (det3(UT) < FT(0)) { UT[0] = -UT[0]; UT[1] = -UT[1]; UT[2] = -UT[2]; }
  // REFINE: sigma = x rsqrt(x), and rsqrt(x) is 1 / sigma for the row scaling
  FT rs[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    if constexpr (REFINE) {
      rs[i] = ev[i] > FT(0) ? rsqrt(ev[i]) : FT(0);
      ev[i] = ev[i] > FT(0) ? ev[i] * rs[i] : FT(0);
    } else {
      ev[i] = ev[i] > FT(0) ? sqrt(ev[i]) : FT(0);
    }
  }
  auto inv = [&](int i) { return REFINE ? rs[i] : FT(1) / ev[i]; };
  mul3(UT, F, VT);
  const FT eps = FT(1e-8);
  const int cond = (ev[0] < eps) + ((ev[1] < eps) << 1) + ((ev[2] < eps) << 2);
  auto row = [&](int r) { return V3t<FT>{VT[3 * r], VT[3 * r + 1], VT[3 * r + 2]}; };
  auto setrow = [&](int r, V3t<FT> v) { VT[3 * r] = v.x; VT[3 * r + 1] = v.y; VT[3 * r + 2] = v.z; };
  auto scalerow = [&](int r, FT f) { VT[3 * r] *= f; VT[3 * r + 1] *= f; VT[3 * r + 2] *= f; };
  switch (cond) {
    case 0: {
      scalerow(0, inv(0)); scalerow(1, inv(1)); scalerow(2, inv(2));
      if (det3(VT) < FT(0)) {
        int sm = ev[0] < ev[1] ? (ev[0] < ev[2] ? 0 : 2) : (ev[1] < ev[2] ? 1 : 2);
        scalerow(sm, FT(-1));
        ev[sm] = -ev[sm];
      }
      break;
    }
    case 1: scalerow(1, inv(1)); scalerow(2, inv(2)); setrow(0, v_cross(row(1), row(2))); break;
    case 2: scalerow(0, inv(0)); scalerow(2, inv(2)); setrow(1, v_cross(row(2), row(0))); break;
    case 3: { scalerow(2, inv(2)); V3t<FT> a, c; coord_system(row(2), a, c); setrow(0, a); setrow(1, c); break; }
    case 4: scalerow(0, inv(0)); scalerow(1, inv(1)); setrow(2, v_cross(row(0), row(1))); break;
    case 5: { scalerow(1, inv(1)); V3t<FT> a, c; coord_system(row(1), a, c); setrow(2, a); setrow(0, c); break; }
    case 6: { scalerow(0, inv(0)); V3t<FT> a, c; coord_system(row(0), a, c); setrow(1, a); setrow(2, c); break; }
    default:
#pragma unroll
      for (int i = 0; i < 9; i++) VT[i] = FT(0);
      VT[0] = VT[4] = VT[8] = FT(1);
      break;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) sig[i] = ev[i] > thr ? ev[i] : thr;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) U[i * 3 + j] = UT[j * 3 + i];
}

// PSD projection of a packed symmetric 3x3 (tetelement.cpp:439-465)
template <class FT>
__device__ void psd3(FT* m) {
  // Positive leading minors (Sylvester) prove every eigenvalue positive, in
  // which case the projection leaves the matrix unchanged: skip the eigensolve.
  {
    const FT m01 = m[0] * m[3] - m[1] * m[1];
    const FT dt = m[0] * (m[3] * m[5] - m[4] * m[4]) - m[1] * (m[1] * m[5] - m[4] * m[2]) +
                  m[2] * (m[1] * m[4] - m[3] * m[2]);
    if (m[0] > FT(0) && m01 > FT(0) && dt > FT(0)) return;
  }
  FT QT[9], ev[3];
  eig_sym3(m, ev, QT);
  bool neg = false;
#pragma unroll
  for (int i = 0; i < 3; i++) if (ev[i] < FT(0)) { neg = true; ev[i] = FT(0); }
  if (!neg) return;
  // A = Q diag(ev) Q^T with Q = QT^T
  FT A00 = FT(0), A01 = FT(0), A02 = FT(0), A11 = FT(0), A12 = FT(0), A22 = FT(0);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    FT q0 = QT[3 * k], q1 = QT[3 * k + 1], q2 = QT[3 * k + 2];
    A00 += q0 * (QT[3 * k] * ev[k]);
    A01 += q0 * (QT[3 * k + 1] * ev[k]);
    A02 += q0 * (QT[3 * k + 2] * ev[k]);
    A11 += q1 * (QT[3 * k + 1] * ev[k]);
    A12 += q1 * (QT[3 * k + 2] * ev[k]);
    A22 += q2 * (QT[3 * k + 2] * ev[k]);
  }
  m[0] = A00; m[1] = A01; m[2] = A02; m[3] = A11; m[4] = A12; m[5] = A22;
}

// PSD projection of [[d, o], [o, d]] (tetelement.cpp:467-499)
template <class FT>
__device__ __forceinline__ void psd2(FT& d, FT& o) {
  FT e0 = d + o, e1 = d - o;
  int c = (e0 < FT(0)) + ((e1 < FT(0)) << 1);
  if (c == 1) { e1 *= FT(0.5); d = e1; o = -e1; }
  else if (c == 2) { e0 *= FT(0.5); d = e0; o = e0; }
  else if (c == 3) { d = FT(0); o = FT(0); }
}

}  // namespace od
