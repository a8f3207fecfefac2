// CPU restatement of the reference's implicit FEM step (test infrastructure).
//
// This is the oracle the GPU path is checked against.  It restates, in plain
// sequential double precision, every function on the hot path; each function
// cites the reference file:line it follows.  It is pinned against the
// compiled reference (oracle/_ref, built by oracle/build_ref.py) through the
// golden fixtures in tests/golden and the CPU tests.  Nothing in the product
// links it: only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
// bench.py load it, as the checker.
//
// Parts with no reference counterpart (the full-order Newmark integrator with
// a Newton loop, the 3x3 block-Jacobi and IC(0) preconditioners) are defined
// here for this project; their definitions are written next to the code.
//
// Build: g++ -O2 -std=c++17 -fPIC -ffp-contract=off -shared (oracle/build_oracle.py)
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <set>
#include <vector>

namespace {

// ---------------------------------------------------------------- indexing
// NodeIndexer::getGlobalIndex (core/nodeIndexer.cpp:12-25): compacted DOF =
// 3*node + axis minus the number of constrained DOFs below it, -1 if the DOF
// itself is constrained.
int global_index(const std::vector<int>& cd, int node, int axis) {
  int idx = 3 * node + axis;
  if (cd.empty()) return idx;
  int off = (int)(std::lower_bound(cd.begin(), cd.end(), idx) - cd.begin());
  if (off < (int)cd.size() && cd[off] == idx) return -1;
  return idx - off;
}

// Element::getLocalMatrixIndex (core/element.h:109-118): packed position of
// (a, b) in the 78-entry upper triangle of the 12x12 element matrix.
inline int local_index(int a, int b) {
  if (a > b) std::swap(a, b);
  return a * 12 - ((a - 1) * a) / 2 + b - a;
}

// ------------------------------------------------------------- small maths
struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 scale(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double at(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
// VectorBase::operator/ (core/latool.h:51-55) multiplies by the reciprocal
inline V3 divv(V3 a, double s) { double r = 1.0 / s; return {r * a.x, r * a.y, r * a.z}; }
inline double len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }

// getTetVolume (element/tetelement.cpp:6-12)
double tet_volume(V3 a, V3 b, V3 c, V3 d) {
  V3 ab = sub(b, a), ac = sub(c, a), ad = sub(d, a);
  return fabs(dot(ab, cross(ac, ad))) / 6.0;
}

// getTetShapeFunctionDerivatives (element/tetelement.cpp:18-48): 6V * grad N,
// the orientation chosen by the sign of (a-d).((b-d)x(c-d)).
void shape_grads(V3 a, V3 b, V3 c, V3 d, double* dn) {
  V3 da = sub(a, d), db = sub(b, d), dc = sub(c, d), ca = sub(a, c), cb = sub(b, c);
  V3 g[4];
  if (dot(da, cross(db, dc)) > 0.0) {
    g[0] = cross(db, dc); g[1] = cross(dc, da); g[2] = cross(da, db); g[3] = cross(cb, ca);
  } else {
    g[0] = cross(dc, db); g[1] = cross(da, dc); g[2] = cross(db, da); g[3] = cross(ca, cb);
  }
  for (int i = 0; i < 4; i++) { dn[3 * i] = g[i].x; dn[3 * i + 1] = g[i].y; dn[3 * i + 2] = g[i].z; }
}

// Tensor2::Determinant / Inverse (core/latool.h:184-207), row-major 3x3
double det3(const double* m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}
void inverse3(const double* t, double* r) {
  double inv = 1.0 / det3(t);
  r[0] = (t[4] * t[8] - t[5] * t[7]) * inv;
  r[1] = (t[2] * t[7] - t[1] * t[8]) * inv;
  r[2] = (t[1] * t[5] - t[2] * t[4]) * inv;
  r[3] = (t[5] * t[6] - t[3] * t[8]) * inv;
  r[4] = (t[0] * t[8] - t[2] * t[6]) * inv;
  r[5] = (t[2] * t[3] - t[0] * t[5]) * inv;
  r[6] = (t[3] * t[7] - t[4] * t[6]) * inv;
  r[7] = (t[1] * t[6] - t[0] * t[7]) * inv;
  r[8] = (t[0] * t[4] - t[1] * t[3]) * inv;
}
void matmul3(const double* a, const double* b, double* c) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}
inline double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ------------------------------------------------ symmetric 3x3 eigensolve
// eigenSym3x3 (core/numerMethod.h:327-429): trigonometric solution for the
// largest-magnitude deviatoric eigenvalue, then a 2x2 problem in the
// orthogonal complement.  tri = (a00, a01, a02, a11, a12, a22); vecs are
// the eigenvectors stored as rows.
void eigsym3(const double* tri, double* vals, double* vecs) {
  const double pi = 3.141592653589793238462643383279502884;
  const double ave = (tri[0] + tri[3] + tri[5]) / 3.0;
  const double d0 = tri[0] - ave, d1 = tri[3] - ave, d2 = tri[5] - ave;
  const double J2 = (d0 * d0 + d1 * d1 + d2 * d2) * 0.5 + tri[1] * tri[1] + tri[2] * tri[2] + tri[4] * tri[4];
  const double J3 = d0 * (d1 * d2 - tri[4] * tri[4]) + tri[1] * (tri[4] * tri[2] - tri[1] * d2) +
                    tri[2] * (tri[1] * tri[4] - d1 * tri[2]);
  const double s3 = 1.7320508075688772935274463415058723669428;
  const double sq = sqrt(J2);
  const double cs = (3.0 * 0.5 * s3) * ((J3 / J2) / sq);
  if (isnan(cs) || isinf(cs)) {
    vals[0] = vals[1] = vals[2] = ave;
    for (int i = 0; i < 9; i++) vecs[i] = 0.0;
    vecs[0] = vecs[4] = vecs[8] = 1.0;
    return;
  }
  double ang = acos(clampd(cs, -1.0, 1.0)) / 3.0;
  double e0 = (2.0 / s3) * sq * (ang < pi / 6.0 ? cos(ang) : cos(ang + (2.0 / 3.0) * pi));
  vals[0] = e0 + ave;
  V3 r0 = {d0 - e0, tri[1], tri[2]}, r1 = {tri[1], d1 - e0, tri[4]}, r2 = {tri[2], tri[4], d2 - e0};
  double l0 = sqrt(len2(r0)), l1 = sqrt(len2(r1)), l2 = sqrt(len2(r2));
  V3 s0, t1, t2;
  auto proj = [](V3 r, V3 s) { return sub(r, scale(s, dot(s, r))); };
  if (l0 > l1) {
    if (l0 > l2) { s0 = divv(r0, l0); t1 = proj(r1, s0); t2 = proj(r2, s0); }
    else { s0 = divv(r2, l2); t1 = proj(r0, s0); t2 = proj(r1, s0); }
  } else {
    if (l1 > l2) { s0 = divv(r1, l1); t1 = proj(r0, s0); t2 = proj(r2, s0); }
    else { s0 = divv(r2, l2); t1 = proj(r0, s0); t2 = proj(r1, s0); }
  }
  double t1l = len2(t1), t2l = len2(t2);
  V3 s1 = t1l > t2l ? divv(t1, sqrt(t1l)) : divv(t2, sqrt(t2l));
  V3 ev0 = cross(s0, s1);
  vecs[0] = ev0.x; vecs[1] = ev0.y; vecs[2] = ev0.z;
  auto mulm = [&](V3 v) {
    return V3{d0 * v.x + tri[1] * v.y + tri[2] * v.z, tri[1] * v.x + d1 * v.y + tri[4] * v.z,
              tri[2] * v.x + tri[4] * v.y + d2 * v.z};
  };
  V3 m0 = mulm(s0), m1 = mulm(s1);
  double a11 = dot(s0, m0), a12 = dot(s0, m1), a22 = dot(s1, m1);
  double disc = sqrt((a11 - a22) * (a11 - a22) + 4.0 * a12 * a12);
  double e1 = ((a11 + a22) - (a11 > a22 ? disc : -disc)) / 2.0;
  double e2 = a11 + a22 - e1;
  vals[1] = e1 + ave;
  vals[2] = e2 + ave;
  V3 u0 = cross(sub(m0, scale(s0, e1)), ev0);
  V3 u1 = cross(sub(m1, scale(s1, e1)), ev0);
  double u0l = len2(u0), u1l = len2(u1);
  V3 ev1;
  // the reference tests u0Len2 twice (numerMethod.h:422); reproduced as written
  if (u0l != 0.0 && u0l != 0.0) ev1 = u0l > u1l ? divv(u0, sqrt(u0l)) : divv(u1, sqrt(u1l));
  else ev1 = s0;
  vecs[3] = ev1.x; vecs[4] = ev1.y; vecs[5] = ev1.z;
  V3 ev2 = cross(ev0, ev1);
  vecs[6] = ev2.x; vecs[7] = ev2.y; vecs[8] = ev2.z;
}

// ------------------------------------------------------- Givens QR (3x3)
// properQRDecompostion3x3 (core/numerMethod.h:431-507): three Givens
// rotations zeroing (2,0), (1,0), (2,1); returns Q with det +1 (row-major).
void givens(double a, double b, double& c, double& s, double& r) {
  if (b == 0.0) { c = a < 0.0 ? -1.0 : 1.0; s = 0.0; r = fabs(a); }
  else if (a == 0.0) { c = 0.0; s = b < 0.0 ? 1.0 : -1.0; r = fabs(b); }
  else if (fabs(b) > fabs(a)) {
    double tau = -a / b, u = sqrt(1.0 + tau * tau);
    if (b < 0.0) u = -u;
    s = -1.0 / u; c = s * tau; r = b * u;
  } else {
    double tau = -b / a, u = sqrt(1.0 + tau * tau);
    if (a < 0.0) u = -u;
    c = 1.0 / u; s = c * tau; r = a * u;
  }
}
void qr3(const double* m, double* Qo, double* Ro) {
  double Q[9] = {0}, R[9];
  memcpy(R, m, sizeof(R));
  double c = 0, s = 0, r = 0;
  givens(R[3], R[6], c, s, r);
  Q[4] = Q[8] = c; Q[5] = s; Q[7] = -s;
  R[3] = r; R[6] = 0.0;
  for (int i = 0; i < 2; i++) {
    double p = c * R[4 + i] - s * R[7 + i], q = s * R[4 + i] + c * R[7 + i];
    R[4 + i] = p; R[7 + i] = q;
  }
  givens(R[0], R[3], c, s, r);
  R[0] = r; R[3] = 0.0;
  for (int i = 0; i < 2; i++) {
    double p = c * R[1 + i] - s * R[4 + i], q = s * R[1 + i] + c * R[4 + i];
    R[1 + i] = p; R[4 + i] = q;
  }
  Q[0] = c; Q[1] = s;
  Q[3] = Q[4] * -s; Q[4] *= c;
  Q[6] = Q[7] * -s; Q[7] *= c;
  givens(R[4], R[7], c, s, r);
  R[4] = r; R[7] = 0.0;
  double pp = c * R[5] - s * R[8], qq = s * R[5] + c * R[8];
  R[5] = pp; R[8] = qq;
  for (int i = 0; i < 3; i++) {
    double p = c * Q[3 * i + 1] - s * Q[3 * i + 2], q = s * Q[3 * i + 1] + c * Q[3 * i + 2];
    Q[3 * i + 1] = p; Q[3 * i + 2] = q;
  }
  memcpy(Qo, Q, sizeof(Q));
  if (Ro) memcpy(Ro, R, sizeof(R));
}

// -------------------------------------------------- polar decomposition
// polarDecompostion3x3 (core/numerMethod.h:570-1016), the quaternion method
// of Higham & Noferini (2016): the rotation of F/||F|| is the dominant
// eigenvector of a symmetric 4x4 matrix B built from F; its eigenvalue is the
// largest root of a quartic (closed form or Newton), and the eigenvector comes
// from an LDL^T factorisation of (B + lambda I) with pivoting, followed by one
// of three refinement branches.  Branch thresholds follow the reference.

// Householder orthonormalisation of two 4-vectors stored as mat[0..3],
// mat[4..7] (the anonymous-namespace Orthonormalize, numerMethod.h:510-567).
void orthonormalize2(double* mat) {
  const double tol = 2.2250738585072014e-308;  // numeric_limits<double>::min()
  double beta0 = 0, beta1 = 0, v0[3], v1[2];
  v0[0] = mat[1]; v0[1] = mat[2]; v0[2] = mat[3];
  double n2 = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
  if (n2 <= tol) { v0[0] = v0[1] = v0[2] = 0.0; }
  else {
    double c0 = mat[0], sg = sqrt(c0 * c0 + n2);
    if (c0 >= 0.0) sg = -sg;
    double f = c0 - sg;
    v0[0] /= f; v0[1] /= f; v0[2] /= f;
    beta0 = (sg - c0) / sg;
  }
  double prod = mat[4] + v0[0] * mat[5] + v0[1] * mat[6] + v0[2] * mat[7];
  double c0 = mat[5] - prod * beta0 * v0[0];
  v1[0] = mat[6] - prod * beta0 * v0[1];
  v1[1] = mat[7] - prod * beta0 * v0[2];
  n2 = v1[0] * v1[0] + v1[1] * v1[1];
  if (n2 <= tol) { v1[0] = v1[1] = 0.0; }
  else {
    double sg = sqrt(c0 * c0 + n2);
    if (c0 >= 0.0) sg = -sg;
    double f = c0 - sg;
    v1[0] /= f; v1[1] /= f;
    beta1 = (sg - c0) / sg;
  }
  mat[0] = 1.0 - beta0; mat[1] = -beta0 * v0[0]; mat[2] = -beta0 * v0[1]; mat[3] = -beta0 * v0[2];
  double S[9], l[3];
  S[0] = 1.0 - beta0 * v0[0] * v0[0];
  S[1] = -beta0 * v0[0] * v0[1]; S[3] = S[1];
  S[2] = -beta0 * v0[0] * v0[2]; S[6] = S[2];
  S[4] = 1.0 - beta0 * v0[1] * v0[1];
  S[5] = -beta0 * v0[1] * v0[2]; S[7] = S[5];
  S[8] = 1.0 - beta0 * v0[2] * v0[2];
  l[0] = 1.0 - beta1; l[1] = -beta1 * v1[0]; l[2] = -beta1 * v1[1];
  mat[4] = mat[1] * l[0] + mat[2] * l[1] + mat[3] * l[2];
  mat[5] = S[0] * l[0] + S[1] * l[1] + S[2] * l[2];
  mat[6] = S[3] * l[0] + S[4] * l[1] + S[5] * l[2];
  mat[7] = S[6] * l[0] + S[7] * l[1] + S[8] * l[2];
}

void polar3(const double* F, double* R, double* S) {
  double A[9], B[16];
  double fn = 0.0;
  for (int i = 0; i < 9; i++) fn += F[i] * F[i];
  fn = sqrt(fn);
  if (fn == 0.0) {
    for (int i = 0; i < 9; i++) { R[i] = 0.0; if (S) S[i] = 0.0; }
    R[0] = R[4] = R[8] = 1.0;
    return;
  }
  for (int i = 0; i < 9; i++) A[i] = F[i] / fn;
  // b = 1 - 4 ||adj(A)||^2 (the constant term of the quartic)
  double b = 0.0, t;
  t = A[4] * A[8] - A[5] * A[7]; b += t * t;
  t = A[3] * A[8] - A[5] * A[6]; b += t * t;
  t = A[3] * A[7] - A[4] * A[6]; b += t * t;
  t = A[1] * A[8] - A[2] * A[7]; b += t * t;
  t = A[0] * A[8] - A[2] * A[6]; b += t * t;
  t = A[0] * A[7] - A[1] * A[6]; b += t * t;
  t = A[1] * A[5] - A[2] * A[4]; b += t * t;
  t = A[0] * A[5] - A[2] * A[3]; b += t * t;
  t = A[0] * A[4] - A[1] * A[3]; b += t * t;
  b = 1.0 - 4.0 * b;
  // the symmetric 4x4 matrix whose dominant eigenvector is the quaternion
  B[0] = -A[0] - A[4] - A[8]; B[1] = -A[5] + A[7]; B[2] = -A[6] + A[2]; B[3] = -A[1] + A[3];
  B[4] = B[1]; B[5] = -A[0] + A[4] + A[8]; B[6] = -A[1] - A[3]; B[7] = -A[2] - A[6];
  B[8] = B[2]; B[9] = B[6]; B[10] = -A[4] + A[0] + A[8]; B[11] = -A[5] - A[7];
  B[12] = B[3]; B[13] = B[7]; B[14] = B[11]; B[15] = -A[8] + A[0] + A[4];

  double dA = 1.0, omega = 0.0;
  const double tau = 1e-4;
  const bool quick = b <= 1.0 - tau;
  if (quick) {
    // det(A) by LU with partial pivoting
    int perm[2] = {1, 2};
    int rowIndex = 0;
    double largest = fabs(A[0]);
    if (fabs(A[3]) > largest) { largest = fabs(A[3]); rowIndex = 1; }
    if (fabs(A[6]) > largest) rowIndex = 2;
    if (rowIndex != 0) { dA = -dA; perm[rowIndex - 1] = 0; }
    int row = rowIndex;
    double piv = A[row * 3];
    dA *= piv;
    if (dA != 0.0) {
      for (int j = 0; j < 2; j++) {
        int sr = perm[j];
        double lo = A[sr * 3] / piv;
        for (int k = 1; k < 3; k++) A[sr * 3 + k] -= lo * A[row * 3 + k];
      }
    }
    if (dA != 0.0) {
      int r2, s2;
      if (fabs(A[perm[0] * 3 + 1]) > fabs(A[perm[1] * 3 + 1])) { r2 = perm[0]; s2 = perm[1]; }
      else { dA = -dA; r2 = perm[1]; s2 = perm[0]; }
      double p2 = A[r2 * 3 + 1];
      dA *= p2;
      double lo = A[s2 * 3 + 1] / p2;
      dA *= (A[s2 * 3 + 2] - lo * A[r2 * 3 + 2]);
    }
  } else {
    // det(A) by LU with complete pivoting; omega = |second pivot|
    int rp[3] = {0, 1, 2}, cp[3] = {0, 1, 2};
    for (int i = 0; i < 2; i++) {
      double largest = 0.0;
      int ri = i, ci = i;
      for (int j = i; j < 3; j++)
        for (int k = i; k < 3; k++) {
          double e = fabs(A[rp[j] * 3 + cp[k]]);
          if (e > largest) { largest = e; ri = j; ci = k; }
        }
      if (rp[i] != rp[ri]) { std::swap(rp[i], rp[ri]); dA = -dA; }
      if (cp[i] != cp[ci]) { std::swap(cp[i], cp[ci]); dA = -dA; }
      int row = rp[i], col = cp[i];
      double piv = A[row * 3 + col];
      dA *= piv;
      if (dA == 0.0) break;
      for (int j = i + 1; j < 3; j++) {
        int sr = rp[j];
        double lo = A[sr * 3 + col] / piv;
        for (int k = i + 1; k < 3; k++) A[sr * 3 + cp[k]] -= lo * A[row * 3 + cp[k]];
      }
    }
    dA *= A[rp[2] * 3 + cp[2]];
    omega = fabs(A[rp[1] * 3 + cp[1]]);
  }
  const bool notpd = dA < 0.0;
  if (notpd) { dA = -dA; for (int i = 0; i < 16; i++) B[i] = -B[i]; }

  const double inv3 = 0.333333333333333333333333;
  double lam;
  if (b >= tau - inv3) {
    // closed-form largest root of x^4 - 2x^2 - 8 det(A) x + b
    double c = 8.0 * dA;
    double D0 = 1.0 + 3.0 * b;
    double D1 = -1.0 + (27.0 / 16.0) * c * c + 9.0 * b;
    double sD0 = sqrt(D0);
    double al = D1 / (D0 * sD0);
    double z = (4.0 * inv3) * (1.0 + sD0 * cos(acos(clampd(al, -1.0, 1.0)) * inv3));
    double s = sqrt(z) * 0.5;
    lam = s + 0.5 * sqrt(std::max(0.0, 4.0 - z + c / s));
  } else {
    // Newton from sqrt(3)
    lam = 1.7320508075688772935274463415058723669428;
    double old;
    double c = 8.0 * dA;
    do {
      double p = lam * (lam * (lam * lam - 2.0) - c) + b;
      double dp = lam * (4.0 * lam * lam - 4.0) - c;
      old = lam;
      lam -= p / dp;
    } while (old - lam > 1e-12);
  }
  B[0] += lam; B[5] += lam; B[10] += lam; B[15] += lam;

  // LDL^T with symmetric (diagonal) pivoting, two steps
  double L[6];
  int ix[4] = {0, 1, 2, 3};
  {
    int di = 0;
    double largest = B[0];
    for (int j = 1; j < 4; j++) {
      double dd = B[ix[j] * 4 + ix[j]];
      if (dd > largest) { largest = dd; di = j; }
    }
    if (di != 0) std::swap(ix[0], ix[di]);
    int p = ix[0];
    L[0] = B[p * 4 + ix[1]] / largest;
    L[1] = B[p * 4 + ix[2]] / largest;
    L[2] = B[p * 4 + ix[3]] / largest;
    int r = ix[1], c;
    double od;
    B[r * 4 + r] -= L[0] * B[p * 4 + r];
    c = ix[2]; od = B[r * 4 + c] - L[0] * B[p * 4 + c]; B[r * 4 + c] = od; B[c * 4 + r] = od;
    c = ix[3]; od = B[r * 4 + c] - L[0] * B[p * 4 + c]; B[r * 4 + c] = od; B[c * 4 + r] = od;
    r = ix[2];
    B[r * 4 + r] -= L[1] * B[p * 4 + r];
    c = ix[3]; od = B[r * 4 + c] - L[1] * B[p * 4 + c]; B[r * 4 + c] = od; B[c * 4 + r] = od;
    r = ix[3];
    B[r * 4 + r] -= L[2] * B[p * 4 + r];
  }
  {
    int di = 1, p = ix[1];
    double largest = B[p * 4 + p];
    for (int j = 2; j < 4; j++) {
      double dd = B[ix[j] * 4 + ix[j]];
      if (dd > largest) { largest = dd; di = j; }
    }
    if (di != 1) { std::swap(ix[1], ix[di]); std::swap(L[0], L[di - 1]); }
    p = ix[1];
    L[3] = B[p * 4 + ix[2]] / largest;
    L[4] = B[p * 4 + ix[3]] / largest;
    int r = ix[2], c = ix[3];
    B[r * 4 + r] -= L[3] * B[p * 4 + r];
    double od = B[r * 4 + c] - L[3] * B[p * 4 + c];
    B[r * 4 + c] = od; B[c * 4 + r] = od;
    r = ix[3];
    B[r * 4 + r] -= L[4] * B[p * 4 + r];
  }

  double v[4];
  if (quick) {
    if (B[ix[2] * 4 + ix[2]] < B[ix[3] * 4 + ix[3]]) {
      std::swap(ix[2], ix[3]);
      std::swap(L[1], L[2]); std::swap(L[3], L[4]);
    }
    L[5] = B[ix[2] * 4 + ix[3]] / B[ix[2] * 4 + ix[2]];
    v[ix[0]] = L[0] * L[4] + L[1] * L[5] - L[0] * L[5] * L[3] - L[2];
    v[ix[1]] = L[5] * L[3] - L[4];
    v[ix[2]] = -L[5];
    v[ix[3]] = 1.0;
  } else {
    const double b22 = B[ix[2] * 4 + ix[2]], b33 = B[ix[3] * 4 + ix[3]], b23 = B[ix[2] * 4 + ix[3]];
    double dd = b22 * b33 - b23 * b23;
    if (dd == 0.0) {
      if (b22 == 0.0 && b33 == 0.0 && b23 == 0.0) {
        v[ix[0]] = L[0] * L[4] - L[2];
        v[ix[1]] = -L[4];
        v[ix[2]] = 0.0; v[ix[3]] = 1.0;
      } else {
        double aa = -b23, bb = b22, nn = sqrt(aa * aa + bb * bb);
        aa /= nn; bb /= nn;
        v[ix[3]] = bb; v[ix[2]] = aa;
        v[ix[1]] = -L[4] * bb - L[3] * aa;
        v[ix[0]] = -L[2] * bb - L[1] * aa - L[0] * v[ix[1]];
      }
    } else {
      // inverse iteration with the factorisation
      double ID[5] = {1.0 / B[ix[0] * 4 + ix[0]], 1.0 / B[ix[1] * 4 + ix[1]], b33, -b23, b22};
      double IL[5] = {-L[0], L[0] * L[3] - L[1], L[0] * L[4] - L[2], -L[3], -L[4]};
      if (omega > 6.607e-8) {
        double w[4] = {IL[2], IL[4], 0.0, 1.0};
        int nit = (int)ceil(15.0 / (16.86 + 2.0 * log10(omega)));
        for (int it = 0; it < nit; it++) {
          double nn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
          for (int i = 0; i < 4; i++) w[i] /= nn;
          double w1 = w[1];
          w[1] = IL[0] * w[0] + w1;
          w[2] = IL[1] * w[0] + IL[3] * w1 + w[2];
          w[3] = IL[2] * w[0] + IL[4] * w1 + w[3];
          w[0] *= ID[0]; w[1] *= ID[1];
          double w2 = w[2];
          w[2] = (ID[2] * w2 + ID[3] * w[3]) / dd;
          w[3] = (ID[3] * w2 + ID[4] * w[3]) / dd;
          w[0] = w[0] + IL[0] * w[1] + IL[1] * w[2] + IL[2] * w[3];
          w[1] = w[1] + IL[3] * w[2] + IL[4] * w[3];
        }
        v[ix[0]] = w[0]; v[ix[1]] = w[1]; v[ix[2]] = w[2]; v[ix[3]] = w[3];
      } else {
        // subspace iteration on two vectors, then a 2x2 Rayleigh-Ritz step
        double w[8] = {IL[1], IL[3], 1.0, 0.0, IL[2], IL[4], 0.0, 1.0};
        orthonormalize2(w);
        for (int it = 0; it < 2; it++) {
          double w1 = w[1];
          w[1] = IL[0] * w[0] + w1;
          w[2] = IL[1] * w[0] + IL[3] * w1 + w[2];
          w[3] = IL[2] * w[0] + IL[4] * w1 + w[3];
          double w5 = w[5];
          w[5] = IL[0] * w[4] + w5;
          w[6] = IL[1] * w[4] + IL[3] * w5 + w[6];
          w[7] = IL[2] * w[4] + IL[4] * w5 + w[7];
          w[0] *= ID[0]; w[1] *= ID[1];
          double w2 = w[2];
          w[2] = (ID[2] * w2 + ID[3] * w[3]) / dd;
          w[3] = (ID[3] * w2 + ID[4] * w[3]) / dd;
          // the reference scales the second vector's second entry by ID[2]
          // (numerMethod.h:928); reproduced as written
          w[4] *= ID[0]; w[5] *= ID[2];
          double w6 = w[6];
          w[6] = (ID[2] * w6 + ID[3] * w[7]) / dd;
          w[7] = (ID[3] * w6 + ID[4] * w[7]) / dd;
          w[0] = w[0] + IL[0] * w[1] + IL[1] * w[2] + IL[2] * w[3];
          w[1] = w[1] + IL[3] * w[2] + IL[4] * w[3];
          w[4] = w[4] + IL[0] * w[5] + IL[1] * w[6] + IL[2] * w[7];
          w[5] = w[5] + IL[3] * w[6] + IL[4] * w[7];
        }
        orthonormalize2(w);
        double t0[8], t1[8], BB[3];
        t0[0] = w[0] + L[0] * w[1] + L[1] * w[2] + L[2] * w[3];
        t0[1] = w[1] + L[3] * w[2] + L[4] * w[3];
        t0[2] = w[2]; t0[3] = w[3];
        t0[4] = w[4] + L[0] * w[5] + L[1] * w[6] + L[2] * w[7];
        t0[5] = w[5] + L[3] * w[6] + L[4] * w[7];
        t0[6] = w[6]; t0[7] = w[7];
        double d00 = B[ix[0] * 4 + ix[0]], d11 = B[ix[1] * 4 + ix[1]];
        t1[0] = t0[0] * d00; t1[1] = t0[1] * d11;
        t1[2] = t0[2] * b22 + t0[3] * b23; t1[3] = t0[2] * b23 + t0[3] * b33;
        t1[4] = t0[4] * d00; t1[5] = t0[5] * d11;
        t1[6] = t0[6] * b22 + t0[7] * b23; t1[7] = t0[6] * b23 + t0[7] * b33;
        BB[0] = t1[0] * t0[0] + t1[1] * t0[1] + t1[2] * t0[2] + t1[3] * t0[3];
        BB[1] = t1[0] * t0[4] + t1[1] * t0[5] + t1[2] * t0[6] + t1[3] * t0[7];
        BB[2] = t1[4] * t0[4] + t1[5] * t0[5] + t1[6] * t0[6] + t1[7] * t0[7];
        if (fabs(BB[1]) > 1e-15) {
          double r = (BB[0] - BB[2]) * 0.5;
          double w0 = r - sqrt(r * r + BB[1] * BB[1]);
          for (int i = 0; i < 4; i++) v[ix[i]] = w[i] * w0 + w[4 + i] * BB[1];
        } else if (BB[0] < BB[2]) {
          for (int i = 0; i < 4; i++) v[ix[i]] = w[i];
        } else {
          for (int i = 0; i < 4; i++) v[ix[i]] = w[4 + i];
        }
      }
    }
  }
  double nn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
  for (int i = 0; i < 4; i++) v[i] /= nn;
  double v11 = v[1] * v[1], v22 = v[2] * v[2], v33 = v[3] * v[3];
  double v12 = v[1] * v[2], v03 = v[0] * v[3], v13 = v[1] * v[3];
  double v02 = v[0] * v[2], v23 = v[2] * v[3], v01 = v[0] * v[1];
  double Q[9];
  Q[0] = 1.0 - 2.0 * (v22 + v33); Q[1] = 2.0 * (v12 - v03); Q[2] = 2.0 * (v13 + v02);
  Q[3] = 2.0 * (v12 + v03); Q[4] = 1.0 - 2.0 * (v11 + v33); Q[5] = 2.0 * (v23 - v01);
  Q[6] = 2.0 * (v13 - v02); Q[7] = 2.0 * (v23 + v01); Q[8] = 1.0 - 2.0 * (v11 + v22);
  if (notpd) for (int i = 0; i < 9; i++) Q[i] = -Q[i];
  // R = Q^T (the reference stores the transpose, numerMethod.h:1005-1007)
  R[0] = Q[0]; R[1] = Q[3]; R[2] = Q[6];
  R[3] = Q[1]; R[4] = Q[4]; R[5] = Q[7];
  R[6] = Q[2]; R[7] = Q[5]; R[8] = Q[8];
  if (S)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) S[i * 3 + j] = Q[i * 3] * F[j] + Q[i * 3 + 1] * F[3 + j] + Q[i * 3 + 2] * F[6 + j];
}

// --------------------------------------------------------------- scene
struct Scene {
  int n_nodes = 0, n_tets = 0, dofs = 0;
  std::vector<V3> X, u;                 // rest positions, mesh displacements
  std::vector<int> tets;                // 4 per tet
  std::vector<int> facets;              // 3 per facet
  std::vector<int> cd;                  // sorted constrained DOFs
  std::vector<int> gidx;                // 12 per tet: compacted DOF or -1
  int kind = 0;                         // 0 corot, 1 NH, 2 StVK, 3 corotational plastic
  double rho = 0, lambda = 0, mu = 0, thr = 0, D[3] = {0, 0, 0};
  double yield = 0, creep = 0, max_plastic = 0;  // plastic parameters
  std::vector<double> plastic;          // plastic strain, 9 per tet (state, changes at every evaluation)
  double ldlt_sainv = 0.1, ldlt_drop = 0.01;  // InLDLTPreconditioner(sainvEpsilon, ldltEpsilon)
  double ic_eps = 1e-3, ic_relax = 0.0;       // InCholeskyPreconditioner(epsilon, relaxedScale)
  int ic0_natural = 0;                  // IC(0) in the DOF order (1) or by block colours (0)
  // pattern (reference layout)
  int nbc = 0, nrem = 0;
  std::vector<int> pcol, rows, oris, emap;
  int nvals = 0;
  std::vector<double> pre;              // per-tet precomputes
  std::vector<double> mass;             // mass values
};

// pattern: BlockedSymSparseMatrixAssembler + BlockedSymSparseMatrix ctor
// (core/sparseMatrix.h:90-274) fed by getMatrixStructure
// (material/fullOrderNonlinear.h:46-71).  Block start rows are always
// multiples of 3 in compacted-DOF space; the last row block of a column is
// narrower when it reaches past the matrix; the n % 3 trailing columns are
// stored as scalar columns.
void build_pattern(Scene& s) {
  const int n = s.dofs;
  s.nbc = n / 3;
  s.nrem = n - 3 * s.nbc;
  std::vector<std::set<int>> blockRowsOfCol(s.nbc);
  std::vector<std::set<int>> remRows(s.nrem);
  for (int e = 0; e < s.n_tets; e++) {
    const int* g = &s.gidx[12 * e];
    for (int a = 0; a < 12; a++) {
      if (g[a] < 0) continue;
      for (int b = a; b < 12; b++) {
        if (g[b] < 0) continue;
        int r = std::max(g[a], g[b]), c = std::min(g[a], g[b]);
        if (c / 3 < s.nbc) blockRowsOfCol[c / 3].insert(3 * (r / 3));
        else remRows[c - 3 * s.nbc].insert(r);
      }
    }
  }
  s.pcol.assign(s.nbc + s.nrem + 1, 0);
  s.oris.assign(s.nbc + s.nrem + 1, 0);
  s.rows.clear();
  int nv = 0;
  for (int c = 0; c < s.nbc; c++) {
    for (int r : blockRowsOfCol[c]) {
      s.rows.push_back(r);
      if (r == 3 * c) nv += 6;
      else nv += 3 * std::min(3, n - r);
    }
    s.pcol[c + 1] = (int)s.rows.size();
    s.oris[c + 1] = nv;
  }
  for (int k = 0; k < s.nrem; k++) {
    for (int r : remRows[k]) { s.rows.push_back(r); nv += 1; }
    s.pcol[s.nbc + k + 1] = (int)s.rows.size();
    s.oris[s.nbc + k + 1] = nv;
  }
  s.nvals = nv;
}

// value index of lower entry (r >= c): BlockedSymSparseMatrix::getIndices
// (core/sparseMatrix.h:528-579).  Diagonal blocks pack (0,0),(1,0),(2,0),
// (1,1),(2,1),(2,2); other blocks are column-major with the block's width.
int value_index(const Scene& s, int r, int c) {
  const int n = s.dofs;
  if (c / 3 < s.nbc) {
    int bc = c / 3, sc = c - 3 * bc, br = 3 * (r / 3);
    const int* b = &s.rows[s.pcol[bc]];
    const int* e = &s.rows[s.pcol[bc + 1]];
    const int* p = std::lower_bound(b, e, br);
    if (p == e || *p != br) return -1;
    int k = (int)(p - b), off = s.oris[bc];
    bool hasDiag = s.rows[s.pcol[bc]] == 3 * bc;
    if (br == 3 * bc) {
      static const int di[3] = {0, 3, 5};
      return off + (r - br) - sc + di[sc];
    }
    off += hasDiag ? 6 + 9 * (k - 1) : 9 * k;
    return off + sc * std::min(3, n - br) + (r - br);
  }
  int col = c - 3 * s.nbc + s.nbc;
  const int* b = &s.rows[s.pcol[col]];
  const int* e = &s.rows[s.pcol[col + 1]];
  const int* p = std::lower_bound(b, e, r);
  if (p == e || *p != r) return -1;
  return s.oris[col] + (int)(p - b);
}

// element -> value map (material/fullOrderNonlinear.h:73-110)
void build_emap(Scene& s) {
  s.emap.assign((size_t)78 * s.n_tets, -1);
  for (int e = 0; e < s.n_tets; e++) {
    const int* g = &s.gidx[12 * e];
    int* m = &s.emap[78 * (size_t)e];
    for (int a = 0; a < 12; a++)
      for (int b = a; b < 12; b++) {
        if (g[a] < 0 || g[b] < 0) continue;
        m[local_index(b, a)] = value_index(s, std::max(g[a], g[b]), std::min(g[a], g[b]));
      }
  }
}

inline V3 node_pos(const Scene& s, int n) { return s.X[n]; }
inline V3 node_cur(const Scene& s, int n) { return add(s.X[n], s.u[n]); }

// precomputes: corotational getCorotationalTetElementPrecomputes
// (element/tetelement.cpp:501-544): 10 blocks K0_ab (a <= b), 9 entries each,
// then Dm^-1; invertible-hyperelastic getPrecomputes (tetelement.cpp:253-266):
// 12 shape gradients then Dm^-1.
// corotational (kind 0): [90 K0][9 Dm^-1] per tet; plastic (kind 3) adds the
// 12 shape derivatives (getCorotationalTetElementPrecomputes,
// tetelement.cpp:501-544); invertible: [12 dN][9 Dm^-1]
void build_precomputes(Scene& s) {
  const int ne = s.n_tets;
  if (s.kind == 0) s.pre.assign((size_t)ne * 99, 0.0);
  else if (s.kind == 3) s.pre.assign((size_t)ne * 111, 0.0);
  else s.pre.assign((size_t)ne * 21, 0.0);
  for (int e = 0; e < ne; e++) {
    const int* t = &s.tets[4 * e];
    V3 p0 = node_pos(s, t[0]), p1 = node_pos(s, t[1]), p2 = node_pos(s, t[2]), p3 = node_pos(s, t[3]);
    double dn[12];
    shape_grads(p0, p1, p2, p3, dn);
    V3 ab = sub(p1, p0), ac = sub(p2, p0), ad = sub(p3, p0);
    double Dm[9] = {ab.x, ac.x, ad.x, ab.y, ac.y, ad.y, ab.z, ac.z, ad.z}, Dmi[9];
    inverse3(Dm, Dmi);
    if (s.kind == 0 || s.kind == 3) {
      double vol = tet_volume(p0, p1, p2, p3);
      double f = 1.0 / (36.0 * vol);
      double* K0 = &s.pre[(size_t)e * 90];
      const double* D = s.D;
      int k = 0;
      for (int a = 0; a < 4; a++)
        for (int b = a; b < 4; b++) {
          const double* Ba = dn + 3 * a;
          const double* Bb = dn + 3 * b;
          K0[k + 0] = (D[0] * Ba[0] * Bb[0] + D[2] * (Ba[1] * Bb[1] + Ba[2] * Bb[2])) * f;
          K0[k + 1] = (D[1] * Ba[0] * Bb[1] + D[2] * Ba[1] * Bb[0]) * f;
          K0[k + 2] = (D[1] * Ba[0] * Bb[2] + D[2] * Ba[2] * Bb[0]) * f;
          K0[k + 3] = (D[1] * Ba[1] * Bb[0] + D[2] * Ba[0] * Bb[1]) * f;
          K0[k + 4] = (D[0] * Ba[1] * Bb[1] + D[2] * (Ba[0] * Bb[0] + Ba[2] * Bb[2])) * f;
          K0[k + 5] = (D[1] * Ba[1] * Bb[2] + D[2] * Ba[2] * Bb[1]) * f;
          K0[k + 6] = (D[1] * Ba[2] * Bb[0] + D[2] * Ba[0] * Bb[2]) * f;
          K0[k + 7] = (D[1] * Ba[2] * Bb[1] + D[2] * Ba[1] * Bb[2]) * f;
          K0[k + 8] = (D[0] * Ba[2] * Bb[2] + D[2] * (Ba[0] * Bb[0] + Ba[1] * Bb[1])) * f;
          k += 9;
        }
      memcpy(&s.pre[(size_t)ne * 90 + 9 * (size_t)e], Dmi, sizeof(Dmi));
      if (s.kind == 3) memcpy(&s.pre[(size_t)ne * 99 + 12 * (size_t)e], dn, sizeof(dn));
    } else {
      memcpy(&s.pre[(size_t)e * 12], dn, sizeof(dn));
      memcpy(&s.pre[(size_t)ne * 12 + 9 * (size_t)e], Dmi, sizeof(Dmi));
    }
  }
}

// deformation gradient from current positions (tetelement.cpp:268-280, 556-565)
void deformation_gradient(const Scene& s, const int* t, const double* Dmi, double* F) {
  V3 c0 = node_cur(s, t[0]);
  for (int i = 0; i < 9; i++) F[i] = 0.0;
  for (int i = 1; i < 4; i++) {
    V3 ax = sub(node_cur(s, t[i]), c0);
    for (int j = 0; j < 3; j++) {
      double d = at(ax, j);
      for (int k = 0; k < 3; k++) F[j * 3 + k] += d * Dmi[(i - 1) * 3 + k];
    }
  }
}

static const int kDiag[12] = {0, 12, 23, 33, 42, 50, 57, 63, 68, 72, 75, 77};

// corotational element (tetelement.cpp:546-573 + 583-651): R from the polar
// decomposition of F (QR when the deformed volume drops below threshold times
// the rest volume), K_ab = R K0_ab R^T, f_a = sum_b (R K0_ab R^T x_b - R K0_ab X_b).
void corot_element(const Scene& s, int e, double* K78, double* f12) {
  const int* t = &s.tets[4 * e];
  const double* K0 = &s.pre[(size_t)e * 90];
  const double* Dmi = &s.pre[(size_t)s.n_tets * 90 + 9 * (size_t)e];
  double F[9], R[9];
  deformation_gradient(s, t, Dmi, F);
  V3 o[4], c[4];
  for (int i = 0; i < 4; i++) { o[i] = node_pos(s, t[i]); c[i] = node_cur(s, t[i]); }
  double v0 = tet_volume(o[0], o[1], o[2], o[3]);
  double v1 = tet_volume(c[0], c[1], c[2], c[3]);
  if (v1 >= s.thr * v0) polar3(F, R, nullptr);
  else qr3(F, R, nullptr);
  for (int i = 0; i < 12; i++) f12[i] = 0.0;
  const double* K = K0;
  double QK[9], QKT[9], QKQT[9];
  for (int a = 0; a < 4; a++) {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) QK[i * 3 + j] = R[i * 3] * K[j] + R[i * 3 + 1] * K[3 + j] + R[i * 3 + 2] * K[6 + j];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) QKQT[i * 3 + j] = QK[i * 3] * R[j * 3] + QK[i * 3 + 1] * R[j * 3 + 1] + QK[i * 3 + 2] * R[j * 3 + 2];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3 - i; j++) K78[kDiag[a * 3 + i] + j] = QKQT[i * 3 + i + j];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) f12[a * 3 + i] += QKQT[i * 3 + j] * at(c[a], j) - QK[i * 3 + j] * at(o[a], j);
    K += 9;
    for (int b = a + 1; b < 4; b++) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          QK[i * 3 + j] = R[i * 3] * K[j] + R[i * 3 + 1] * K[3 + j] + R[i * 3 + 2] * K[6 + j];
          QKT[i * 3 + j] = R[i * 3] * K[j * 3] + R[i * 3 + 1] * K[j * 3 + 1] + R[i * 3 + 2] * K[j * 3 + 2];
        }
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) QKQT[i * 3 + j] = QK[i * 3] * R[j * 3] + QK[i * 3 + 1] * R[j * 3 + 1] + QK[i * 3 + 2] * R[j * 3 + 2];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          K78[kDiag[a * 3 + i] + (b - a) * 3 - i + j] = QKQT[i * 3 + j];
          f12[a * 3 + i] += QKQT[i * 3 + j] * at(c[b], j) - QK[i * 3 + j] * at(o[b], j);
          f12[b * 3 + i] += QKQT[j * 3 + i] * at(c[a], j) - QKT[i * 3 + j] * at(o[a], j);
        }
      K += 9;
    }
  }
}

// corotational plastic element (corotationalPlastic.cpp:53-183,
// tetelement.cpp:654-729): F = R S by polar decomposition (R Q-factor and
// upper factor by QR when the deformed volume drops below threshold times
// the rest volume); elastic strain e = sym(S) - I - plastic; stress
// 2 mu e + lambda tr(e) I rotated by R; forces from the stress and the shape
// derivatives; stiffness R K0 R^T.  The plastic strain is updated at every
// evaluation: if |e| exceeds the yield criterion it grows by
// creep (|e| - yield)/|e| e and is scaled back to the maximum plastic
// strain.  Both norms follow the reference, which sums the squares of the
// first three entries (one row) three times (corotationalPlastic.cpp:156-160,
// 169-173).
void plastic_element(Scene& s, int e, double* K78, double* f12) {
  const int ne = s.n_tets;
  const int* t = &s.tets[4 * e];
  const double* K0 = &s.pre[(size_t)e * 90];
  const double* Dmi = &s.pre[(size_t)ne * 90 + 9 * (size_t)e];
  const double* dn = &s.pre[(size_t)ne * 99 + 12 * (size_t)e];
  double* ep = &s.plastic[9 * (size_t)e];
  double F[9], R[9], S[9];
  deformation_gradient(s, t, Dmi, F);
  V3 o[4], c[4];
  for (int i = 0; i < 4; i++) { o[i] = node_pos(s, t[i]); c[i] = node_cur(s, t[i]); }
  double v0 = tet_volume(o[0], o[1], o[2], o[3]);
  double v1 = tet_volume(c[0], c[1], c[2], c[3]);
  if (v1 >= s.thr * v0) polar3(F, R, S);
  else qr3(F, R, S);
  // computeElasticStress (corotationalPlastic.cpp:129-183)
  const double lambda = s.D[1], mu2 = 2.0 * s.D[2];
  double es[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) es[i * 3 + j] = 0.5 * (S[i * 3 + j] + S[j * 3 + i]) - ep[i * 3 + j];
  es[0] -= 1.0;
  es[4] -= 1.0;
  es[8] -= 1.0;
  double st[9];
  for (int i = 0; i < 9; i++) st[i] = mu2 * es[i];
  const double dg = lambda * (es[0] + es[4] + es[8]);
  st[0] += dg;
  st[4] += dg;
  st[8] += dg;
  double P[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) P[i * 3 + j] = R[i * 3] * st[j] + R[i * 3 + 1] * st[3 + j] + R[i * 3 + 2] * st[6 + j];
  double en = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) en += es[i] * es[i];
  en = sqrt(en);
  if (en > s.yield) {
    const double ratio = s.creep * (en - s.yield) / en;
    for (int i = 0; i < 9; i++) ep[i] += ratio * es[i];
    double pn = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) pn += ep[i] * ep[i];
    pn = sqrt(pn);
    if (pn > s.max_plastic) {
      const double fac = s.max_plastic / pn;
      for (int i = 0; i < 9; i++) ep[i] *= fac;
    }
  }
  // stiffness R K0_ab R^T (tetelement.cpp:665-716)
  const double* K = K0;
  double QK[9], QKQT[9];
  for (int a = 0; a < 4; a++) {
    for (int b = a; b < 4; b++) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) QK[i * 3 + j] = R[i * 3] * K[j] + R[i * 3 + 1] * K[3 + j] + R[i * 3 + 2] * K[6 + j];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) QKQT[i * 3 + j] = QK[i * 3] * R[j * 3] + QK[i * 3 + 1] * R[j * 3 + 1] + QK[i * 3 + 2] * R[j * 3 + 2];
      if (a == b) {
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3 - i; j++) K78[kDiag[a * 3 + i] + j] = QKQT[i * 3 + i + j];
      } else {
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) K78[kDiag[a * 3 + i] + (b - a) * 3 - i + j] = QKQT[i * 3 + j];
      }
      K += 9;
    }
  }
  // generateNodalVirtualWorks (tetelement.cpp:718-729)
  const double sixth = 1.0 / 6.0;
  for (int n = 0; n < 3; n++) {
    const double x = dn[3 * n], y = dn[3 * n + 1], z = dn[3 * n + 2];
    for (int i = 0; i < 3; i++) f12[3 * n + i] = (P[i * 3] * x + P[i * 3 + 1] * y + P[i * 3 + 2] * z) * sixth;
  }
  for (int i = 0; i < 3; i++) f12[9 + i] = -(f12[i] + f12[3 + i] + f12[6 + i]);
}

// coordinateSystem (core/latool.h:542-552)
void coordinate_system(V3 v0, V3& v1, V3& v2) {
  if (fabs(v0.x) > fabs(v0.y)) {
    double il = 1.0 / sqrt(v0.x * v0.x + v0.z * v0.z);
    v1 = {-v0.z * il, 0.0, v0.x * il};
  } else {
    double il = 1.0 / sqrt(v0.y * v0.y + v0.z * v0.z);
    v1 = {0.0, -v0.z * il, v0.y * il};
  }
  v2 = cross(v0, v1);
}

// InvertibleHyperelasticMaterial::modifiedDeformGradient
// (material/invertibleHyperelastic.cpp:116-245): SVD of F through the
// eigen-decomposition of F F^T; U made a rotation; V^T = U^T F / sigma with
// the rank-deficient cases completed by cross products; the smallest sigma
// negated when det V < 0; sigma clamped below by the inversion threshold.
void modified_svd(const double* F, double thr, double* sig, double* U, double* VT) {
  double tri[6], ev[3], UT[9];
  static const int di[3] = {0, 3, 5};
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++)
      tri[di[i] + j - i] = F[j * 3] * F[i * 3] + F[j * 3 + 1] * F[i * 3 + 1] + F[j * 3 + 2] * F[i * 3 + 2];
  eigsym3(tri, ev, UT);
  if (det3(UT) < 0.0) for (int i = 0; i < 3; i++) UT[i] = -UT[i];
  for (int i = 0; i < 3; i++) ev[i] = ev[i] > 0.0 ? sqrt(ev[i]) : 0.0;
  matmul3(UT, F, VT);
  const double eps = 1e-8;
  int cond = (ev[0] < eps) + ((ev[1] < eps) << 1) + ((ev[2] < eps) << 2);
  auto row = [&](int r) { return V3{VT[3 * r], VT[3 * r + 1], VT[3 * r + 2]}; };
  auto setrow = [&](int r, V3 v) { VT[3 * r] = v.x; VT[3 * r + 1] = v.y; VT[3 * r + 2] = v.z; };
  auto scalerow = [&](int r, double f) { for (int j = 0; j < 3; j++) VT[3 * r + j] *= f; };
  switch (cond) {
    case 0: {
      for (int i = 0; i < 3; i++) scalerow(i, 1.0 / ev[i]);
      if (det3(VT) < 0) {
        int sm = ev[0] < ev[1] ? (ev[0] < ev[2] ? 0 : 2) : (ev[1] < ev[2] ? 1 : 2);
        scalerow(sm, -1.0);
        ev[sm] = -ev[sm];
      }
      break;
    }
    case 1: scalerow(1, 1.0 / ev[1]); scalerow(2, 1.0 / ev[2]); setrow(0, cross(row(1), row(2))); break;
    case 2: scalerow(0, 1.0 / ev[0]); scalerow(2, 1.0 / ev[2]); setrow(1, cross(row(2), row(0))); break;
    case 3: { scalerow(2, 1.0 / ev[2]); V3 a, b; coordinate_system(row(2), a, b); setrow(0, a); setrow(1, b); break; }
    case 4: scalerow(0, 1.0 / ev[0]); scalerow(1, 1.0 / ev[1]); setrow(2, cross(row(0), row(1))); break;
    case 5: { scalerow(1, 1.0 / ev[1]); V3 a, b; coordinate_system(row(1), a, b); setrow(2, a); setrow(0, b); break; }
    case 6: { scalerow(0, 1.0 / ev[0]); V3 a, b; coordinate_system(row(0), a, b); setrow(1, a); setrow(2, b); break; }
    default:
      for (int i = 0; i < 9; i++) VT[i] = 0.0;
      VT[0] = VT[4] = VT[8] = 1.0;
      break;
  }
  for (int i = 0; i < 3; i++) sig[i] = std::max(ev[i], thr);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) U[i * 3 + j] = UT[j * 3 + i];
}

// PSD projection of the symmetric 3x3 (tetelement.cpp:439-465) and of the
// 2x2 blocks [[d, o], [o, d]] (tetelement.cpp:467-499)
void psd3(double* m) {
  double QT[9], ev[3];
  eigsym3(m, ev, QT);
  bool neg = false;
  for (int i = 0; i < 3; i++) if (ev[i] < 0) { neg = true; ev[i] = 0.0; }
  if (!neg) return;
  double Q[9], A[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Q[i * 3 + j] = QT[j * 3 + i];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) QT[i * 3 + j] *= ev[i];
  matmul3(Q, QT, A);
  m[0] = A[0]; m[1] = A[1]; m[2] = A[2]; m[3] = A[4]; m[4] = A[5]; m[5] = A[8];
}
void psd2(double& d, double& o) {
  double e0 = d + o, e1 = d - o;
  int c = (e0 < 0) + ((e1 < 0) << 1);
  if (c == 1) { e1 *= 0.5; d = e1; o = -e1; }
  else if (c == 2) { e0 *= 0.5; d = e0; o = e0; }
  else if (c == 3) { d = 0.0; o = 0.0; }
}

inline int tidx(int i, int j, int k, int l) { return i * 27 + j * 9 + k * 3 + l; }

// dP/dF in the diagonal (singular-value) frame, projected to PSD
// (InvertibleHyperelasticTetElement::getdPdF, tetelement.cpp:357-437)
void dPdF_diag(const double* sig, const double* g, const double* H, double* dP) {
  const double s2[3] = {sig[0] * sig[0], sig[1] * sig[1], sig[2] * sig[2]};
  const double I3 = s2[0] * s2[1] * s2[2];
  const double sc[3] = {sig[0] * sig[1], sig[0] * sig[2], sig[1] * sig[2]};
  double a00 = 2.0 * g[0] + 8.0 * s2[0] * g[1];
  double a01 = 2.0 * g[0] + 4.0 * (s2[0] + s2[1]) * g[1];
  double a02 = 2.0 * g[0] + 4.0 * (s2[0] + s2[2]) * g[1];
  double a11 = 2.0 * g[0] + 8.0 * s2[1] * g[1];
  double a12 = 2.0 * g[0] + 4.0 * (s2[1] + s2[2]) * g[1];
  double a22 = 2.0 * g[0] + 8.0 * s2[2] * g[1];
  double d00 = I3 * g[2] / s2[0], d01 = I3 * g[2] / sc[0], d02 = I3 * g[2] / sc[1];
  double d11 = I3 * g[2] / s2[1], d12 = I3 * g[2] / sc[2], d22 = I3 * g[2] / s2[2];
  double b00 = 4.0 * s2[0] * g[1] - 2.0 * d00, b01 = 4.0 * sc[0] * g[1] - 2.0 * d01;
  double b02 = 4.0 * sc[1] * g[1] - 2.0 * d02, b11 = 4.0 * s2[1] * g[1] - 2.0 * d11;
  double b12 = 4.0 * sc[2] * g[1] - 2.0 * d12, b22 = 4.0 * s2[2] * g[1] - 2.0 * d22;
  const double Hm[9] = {H[0], H[1], H[2], H[1], H[3], H[4], H[2], H[4], H[5]};
  V3 w[3];
  for (int i = 0; i < 3; i++) w[i] = {2.0 * sig[i], 4.0 * sig[i] * s2[i], 2.0 * I3 / sig[i]};
  auto hv = [&](V3 v) {
    return V3{Hm[0] * v.x + Hm[1] * v.y + Hm[2] * v.z, Hm[3] * v.x + Hm[4] * v.y + Hm[5] * v.z,
              Hm[6] * v.x + Hm[7] * v.y + Hm[8] * v.z};
  };
  double g00 = dot(w[0], hv(w[0])) + 4.0 * d00, g01 = dot(w[1], hv(w[0])) + 4.0 * d01;
  double g02 = dot(w[2], hv(w[0])) + 4.0 * d02, g11 = dot(w[1], hv(w[1])) + 4.0 * d11;
  double g12 = dot(w[2], hv(w[1])) + 4.0 * d12, g22 = dot(w[2], hv(w[2])) + 4.0 * d22;
  double tm[6] = {a00 + b00 + g00, g01, g02, a11 + b11 + g11, g12, a22 + b22 + g22};
  psd3(tm);
  psd2(a01, b01);
  psd2(a02, b02);
  psd2(a12, b12);
  for (int i = 0; i < 81; i++) dP[i] = 0.0;
  dP[tidx(0, 0, 0, 0)] = tm[0]; dP[tidx(0, 0, 1, 1)] = tm[1]; dP[tidx(0, 0, 2, 2)] = tm[2];
  dP[tidx(1, 1, 0, 0)] = tm[1]; dP[tidx(1, 1, 1, 1)] = tm[3]; dP[tidx(1, 1, 2, 2)] = tm[4];
  dP[tidx(2, 2, 0, 0)] = tm[2]; dP[tidx(2, 2, 1, 1)] = tm[4]; dP[tidx(2, 2, 2, 2)] = tm[5];
  dP[tidx(0, 1, 0, 1)] = a01; dP[tidx(0, 1, 1, 0)] = b01; dP[tidx(1, 0, 0, 1)] = b01; dP[tidx(1, 0, 1, 0)] = a01;
  dP[tidx(0, 2, 0, 2)] = a02; dP[tidx(0, 2, 2, 0)] = b02; dP[tidx(2, 0, 0, 2)] = b02; dP[tidx(2, 0, 2, 0)] = a02;
  dP[tidx(1, 2, 1, 2)] = a12; dP[tidx(1, 2, 2, 1)] = b12; dP[tidx(2, 1, 1, 2)] = b12; dP[tidx(2, 1, 2, 1)] = a12;
}

// invertible hyperelastic element (invertibleHyperelastic.cpp:231-270 and
// tetelement.cpp:282-355).  Energy derivatives in the invariants
// I1 = sum s^2, I2 = sum s^4, I3 = prod s^2 (invertibleHyperelastic.h:22-30):
// Neo-Hookean invertibleNeoHookean.cpp:11-20, StVK invertibleStVK.cpp:11-20.
void invhyper_element(const Scene& s, int e, double* K78, double* f12) {
  const int* t = &s.tets[4 * e];
  const double* dn = &s.pre[(size_t)e * 12];
  const double* Dmi = &s.pre[(size_t)s.n_tets * 12 + 9 * (size_t)e];
  double F[9], sig[3], U[9], VT[9];
  deformation_gradient(s, t, Dmi, F);
  modified_svd(F, s.thr, sig, U, VT);
  double s02 = sig[0] * sig[0], s12 = sig[1] * sig[1], s22 = sig[2] * sig[2];
  double I[3] = {s02 + s12 + s22, s02 * s02 + s12 * s12 + s22 * s22, s02 * s12 * s22};
  double g[3], H[6] = {0, 0, 0, 0, 0, 0};
  if (s.kind == 1) {
    g[0] = 0.5 * s.mu;
    g[1] = 0.0;
    g[2] = (-0.5 * s.mu + 0.25 * s.lambda * log(I[2])) / I[2];
    H[5] = (0.5 * s.mu + 0.25 * s.lambda * (1.0 - log(I[2]))) / (I[2] * I[2]);
  } else {
    g[0] = 0.25 * s.lambda * (I[0] - 3.0) - 0.5 * s.mu;
    g[1] = 0.25 * s.mu;
    g[2] = 0.0;
    H[0] = 0.25 * s.lambda;
  }
  // first Piola-Kirchhoff stress (invertibleHyperelastic.cpp:247-265)
  double de[3], RM[9], P[9];
  for (int i = 0; i < 3; i++)
    de[i] = 2.0 * g[0] * sig[i] + 4.0 * g[1] * sig[i] * sig[i] * sig[i] + 2.0 * g[2] * I[2] / sig[i];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) RM[i * 3 + j] = VT[i * 3 + j] * de[i];
  matmul3(U, RM, P);
  // stiffness
  double dP[81];
  dPdF_diag(sig, g, H, dP);
  V3 o[4];
  for (int i = 0; i < 4; i++) o[i] = node_pos(s, t[i]);
  double vol = tet_volume(o[0], o[1], o[2], o[3]);
  double fac = 1.0 / (36.0 * vol);
  V3 dN[4];
  for (int i = 0; i < 4; i++) {
    V3 d = {dn[3 * i], dn[3 * i + 1], dn[3 * i + 2]};
    dN[i] = {VT[0] * d.x + VT[1] * d.y + VT[2] * d.z, VT[3] * d.x + VT[4] * d.y + VT[5] * d.z,
             VT[6] * d.x + VT[7] * d.y + VT[8] * d.z};
  }
  double UT[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) UT[i * 3 + j] = U[j * 3 + i];
  for (int i = 0; i < 78; i++) K78[i] = 0.0;
  double sm[9], tmp[9], out[9];
  for (int a = 0; a < 4; a++) {
    for (int b = a; b < 4; b++) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double en = 0.0;
          for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) en += dP[tidx(i, k, j, l)] * at(dN[a], k) * at(dN[b], l);
          sm[i * 3 + j] = en;
        }
      matmul3(U, sm, tmp);
      matmul3(tmp, UT, out);
      if (b == a) {
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3 - i; j++) K78[kDiag[a * 3 + i] + j] = out[i * 3 + i + j] * fac;
      } else {
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) K78[kDiag[a * 3 + i] + (b - a) * 3 - i + j] = out[i * 3 + j] * fac;
      }
    }
  }
  // nodal forces f_a = P dN_a / 6, f_3 = -(f_0 + f_1 + f_2)
  for (int i = 0; i < 3; i++) {
    V3 d = {dn[3 * i], dn[3 * i + 1], dn[3 * i + 2]};
    double fx = P[0] * d.x + P[1] * d.y + P[2] * d.z;
    double fy = P[3] * d.x + P[4] * d.y + P[5] * d.z;
    double fz = P[6] * d.x + P[7] * d.y + P[8] * d.z;
    const double sixth = 1.0 / 6.0;
    f12[3 * i] = fx * sixth; f12[3 * i + 1] = fy * sixth; f12[3 * i + 2] = fz * sixth;
  }
  for (int i = 0; i < 3; i++) f12[9 + i] = -(f12[i] + f12[3 + i] + f12[6 + i]);
}

void element(Scene& s, int e, double* K78, double* f12) {
  if (s.kind == 0) corot_element(s, e, K78, f12);
  else if (s.kind == 3) plastic_element(s, e, K78, f12);
  else invhyper_element(s, e, K78, f12);
}

// assembly into the reference layout (corotationalHyperelastic.cpp:100-120)
void assemble(Scene& s, double* values, double* fint) {
  memset(values, 0, sizeof(double) * s.nvals);
  memset(fint, 0, sizeof(double) * s.dofs);
  double K[78], f[12];
  for (int e = 0; e < s.n_tets; e++) {
    element(s, e, K, f);
    const int* m = &s.emap[78 * (size_t)e];
    for (int k = 0; k < 78; k++) if (m[k] >= 0) values[m[k]] += K[k];
    const int* g = &s.gidx[12 * e];
    for (int k = 0; k < 12; k++) if (g[k] >= 0) fint[g[k]] += f[k];
  }
}

// consistent mass (tetelement.cpp:51-66, mechMaterial.cpp:69-98)
void build_mass(Scene& s) {
  s.mass.assign(s.nvals, 0.0);
  for (int e = 0; e < s.n_tets; e++) {
    const int* t = &s.tets[4 * e];
    double vol = tet_volume(node_pos(s, t[0]), node_pos(s, t[1]), node_pos(s, t[2]), node_pos(s, t[3]));
    double od = vol * 0.05, dg = vol * 0.1;
    const int* m = &s.emap[78 * (size_t)e];
    const int* g = &s.gidx[12 * e];
    for (int a = 0; a < 4; a++)
      for (int b = a; b < 4; b++) {
        double entry = s.rho * (a == b ? dg : od);
        for (int ax = 0; ax < 3; ax++) {
          if (g[3 * a + ax] >= 0 && g[3 * b + ax] >= 0) s.mass[m[local_index(3 * a + ax, 3 * b + ax)]] += entry;
        }
      }
  }
}

// SpMDV (core/numerMethod.h:134-262): y += A x with A stored as its lower
// triangle; every off-diagonal entry is used for both (r, c) and (c, r).
void spmdv(const Scene& s, const double* val, const double* x, double* y) {
  const int n = s.dofs;
  for (int bc = 0; bc < s.nbc; bc++) {
    int c0 = 3 * bc;
    const double* v = val + s.oris[bc];
    for (int k = s.pcol[bc]; k < s.pcol[bc + 1]; k++) {
      int r0 = s.rows[k];
      if (r0 == c0) {
        static const int di[3] = {0, 3, 5};
        for (int sc = 0; sc < 3; sc++)
          for (int sr = sc; sr < 3; sr++) {
            double a = v[sr - sc + di[sc]];
            y[c0 + sr] += a * x[c0 + sc];
            if (sr != sc) y[c0 + sc] += a * x[c0 + sr];
          }
        v += 6;
      } else {
        int w = std::min(3, n - r0);
        for (int sc = 0; sc < 3; sc++)
          for (int sr = 0; sr < w; sr++) {
            double a = v[sc * w + sr];
            y[r0 + sr] += a * x[c0 + sc];
            y[c0 + sc] += a * x[r0 + sr];
          }
        v += 3 * w;
      }
    }
  }
  for (int k = 0; k < s.nrem; k++) {
    int col = s.nbc + k, c = 3 * s.nbc + k;
    const double* v = val + s.oris[col];
    for (int q = s.pcol[col]; q < s.pcol[col + 1]; q++, v++) {
      int r = s.rows[q];
      y[r] += *v * x[c];
      if (r != c) y[c] += *v * x[r];
    }
  }
}

// diagonal (BlockedSymSparseMatrix::getDiagonal, sparseMatrix.h:413-426)
void diagonal(const Scene& s, const double* val, double* d) {
  for (int bc = 0; bc < s.nbc; bc++) {
    const double* v = val + s.oris[bc];
    d[3 * bc] = v[0]; d[3 * bc + 1] = v[3]; d[3 * bc + 2] = v[5];
  }
  for (int k = 0; k < s.nrem; k++) d[3 * s.nbc + k] = val[s.oris[s.nbc + k]];
}

// sparse vector with entries in first-touch order (the reference's
// FastSparseVector, core/latool.h:453-520)
struct TouchVec {
  std::vector<int> at, idx;
  std::vector<double> val;
  explicit TouchVec(int n) : at(n, -1) {}
  void add(int i, double x) {
    if (at[i] >= 0) { val[at[i]] += x; return; }
    at[i] = (int)idx.size(); idx.push_back(i); val.push_back(x);
  }
  double get(int i) const { return at[i] >= 0 ? val[at[i]] : 0.0; }
  void clear() { for (int i : idx) at[i] = -1; idx.clear(); val.clear(); }
};

// ---------------------------------------------------------- preconditioners
// 0 identity (preconditioner.h:14-16), 1 Jacobi (jacobiPreconditioner.cpp:
// 12-26: 1/d, or 1 when d <= 0), 2 3x3 block-Jacobi, 3 IC(0).
//
// Block-Jacobi (no reference counterpart): z_b = inverse(A_bb) r_b for every
// 3x3 diagonal block (symmetric, from the packed 6 values); the n % 3 scalar
// tail uses point Jacobi.  Inverse by the adjugate formula.
//
// IC(0) (no reference counterpart): scalar incomplete Cholesky with zero fill
// on the blocked pattern -- every scalar position between two blocks of
// three compacted DOFs (the last block may hold fewer) that a stored entry
// couples, zero where the reference layout stores nothing -- L L^T ~ P A P^T.
// P orders the blocks by a greedy colouring of the block graph (blocks in
// index order, each taking the lowest colour none of its coloured
// neighbours has; then by colour, by index), or keeps the DOF order.  A
// pivot not above 1e-12 times its diagonal restarts the factorisation with a
// diagonal shift.  Apply: z = P^T (L L^T)^-1 P r.
struct Precond {
  int kind = 0;
  std::vector<double> inv;        // Jacobi: n; block-Jacobi: 9 per block + tail
  // IC(0) in scalar CSR (rows sorted; diagonal last in each row), in the
  // factor's DOF order: newdof[DOF] = its factor row
  std::vector<int> rp, ci, newdof;
  std::vector<double> lv;
  double shift = 0.0;
  int natural = 0;
  // incomplete LDL^T (kind 4) in the reference's storage
  double sainv_eps = 0.1, ldlt_eps = 0.01;
  std::vector<double> lval, dinv;
  std::vector<int> lrow, lpcol;
  // threshold incomplete Cholesky (kind 5), reference storage: column c =
  // its diagonal then its rows below ascending; pcol n + 1 entries
  double ic_eps = 1e-3, ic_relax = 0.0;
  std::vector<double> cval;
  std::vector<int> crow, cpcol;
};

// Column c of the stored lower triangle as BlockedSymSparseMatrix::getColumn
// gives it (core/sparseMatrix.h:297-365): rows c and below in storage
// (ascending) order, zero values left out.
void lower_column(const Scene& s, const double* val, int c, std::vector<std::pair<int, double>>& out) {
  out.clear();
  const int n = s.dofs;
  if (c / 3 < s.nbc) {
    const int bc = c / 3, off = c - 3 * bc;
    const double* v = val + s.oris[bc];
    int k = s.pcol[bc];
    const int e = s.pcol[bc + 1];
    if (k == e) return;
    if (s.rows[k] == 3 * bc) {   // diagonal block, packed (0,0),(1,0),(2,0),(1,1),(2,1),(2,2)
      static const int first[3] = {0, 3, 5};
      for (int i = 0; i < 3 - off; i++)
        if (v[first[off] + i] != 0.0) out.push_back({c + i, v[first[off] + i]});
      k++;
      v += 6;
    }
    for (; k < e; k++) {
      const int r0 = s.rows[k];
      const int w = k == e - 1 ? std::min(3, n - r0) : 3;
      for (int i = 0; i < w; i++)
        if (v[off * w + i] != 0.0) out.push_back({r0 + i, v[off * w + i]});
      v += 3 * w;
    }
  } else {
    const int col = s.nbc + (c - 3 * s.nbc);
    const double* v = val + s.oris[col];
    for (int q = s.pcol[col]; q < s.pcol[col + 1]; q++)
      if (v[q - s.pcol[col]] != 0.0) out.push_back({s.rows[q], v[q - s.pcol[col]]});
  }
}

// InCholeskyPreconditioner::incompleteCholeskyDecomposition and
// proccessSingleColumn (solver/inCholeskyPreconditioner.cpp:18-130): a
// left-looking column factorisation.  Column i starts from A's column i
// (getColumn: diagonal first); every earlier column j with a stored entry
// in row i subtracts L_ij times its entries below row i (the columns are
// found through per-row chains: chain[r] lists the columns whose next
// unprocessed entry is in row r, with that entry's position).  Then, with d
// the running diagonal of column i (A_ii minus the squares of the entries
// already stored in row i), each off-diagonal v of row r is dropped when
// v^2 < |eps^2 d d_r| -- adding |v| relaxedScale to both d and d_r -- or
// kept; L_ii = sqrt(d) (d <= 0 replaced by eps^2 d^2), L_ri = v / L_ii, and
// d_r -= L_ri^2.  The last column takes sqrt(d) only.
void ric_factor(const Scene& s, const double* val, Precond& P) {
  const int n = s.dofs;
  P.cval.clear(); P.crow.clear(); P.cpcol.assign(1, 0);
  if (n == 0) return;
  std::vector<double> d(n, 0.0);
  std::vector<std::pair<int, double>> col;
  for (int c = 0; c < n; c++) {   // getDiagonal: the stored (c, c) entry or 0
    lower_column(s, val, c, col);
    d[c] = (!col.empty() && col[0].first == c) ? col[0].second : 0.0;
  }
  std::vector<std::pair<int, int>> chain(n, {-1, -1});
  const double eps2 = P.ic_eps * P.ic_eps;
  TouchVec w(n);
  std::vector<std::pair<int, double>> kept;
  auto column = [&](int c) {
    double diag = d[c];
    kept.clear();
    for (size_t k = 1; k < w.idx.size(); k++) {   // every entry after the first (the diagonal)
      const int r = w.idx[k];
      const double v = w.val[k];
      if (v == 0.0) continue;
      if (v * v < fabs(eps2 * diag * d[r])) {
        const double comp = fabs(v) * P.ic_relax;
        diag += comp;
        d[r] += comp;
      } else {
        kept.push_back({r, v});
      }
    }
    const int start = P.cpcol[c];
    P.cpcol.push_back(start + 1 + (int)kept.size());
    std::sort(kept.begin(), kept.end(), [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
      return a.first < b.first;
    });
    if (!kept.empty()) {
      const int r = kept[0].first;
      chain[c] = chain[r];
      chain[r] = {c, start + 1};
    }
    if (diag <= 0.0) diag = eps2 * diag * diag;
    const double root = sqrt(diag);
    P.cval.push_back(root);
    P.crow.push_back(c);
    const double inv = 1.0 / root;
    for (auto& e : kept) {
      const double l = e.second * inv;
      P.crow.push_back(e.first);
      P.cval.push_back(e.second * inv);
      d[e.first] -= l * l;
    }
  };
  auto load = [&](int c) {
    w.clear();
    lower_column(s, val, c, col);
    for (auto& e : col) w.add(e.first, e.second);
  };
  load(0);
  column(0);
  for (int i = 1; i < n - 1; i++) {
    load(i);
    std::pair<int, int> link = chain[i];
    while (link.first >= 0) {
      const int j = link.first, at = link.second, next = at + 1;
      const double upper = P.cval[at];
      for (int k = next; k < P.cpcol[j + 1]; k++) w.add(P.crow[k], -upper * P.cval[k]);
      link = chain[j];
      if (next < P.cpcol[j + 1]) {
        const int r = P.crow[next];
        chain[j] = chain[r];
        chain[r] = {j, next};
      }
    }
    column(i);
  }
  P.cval.push_back(sqrt(d[n - 1]));
  P.crow.push_back(n - 1);
  P.cpcol.push_back(P.cpcol[n - 1] + 1);
}

// solvePreconditionerSystem (:132-162): L y = r by columns, L^T z = y by
// row dots from the last row up
void ric_apply(int n, const Precond& P, const double* r, double* z) {
  const double sub0 = r[0] / P.cval[0];
  z[0] = sub0;
  for (int j = 1; j < n; j++) z[j] = r[j];
  for (int q = 1; q < P.cpcol[1]; q++) z[P.crow[q]] -= P.cval[q] * sub0;
  for (int c = 1; c < n; c++) {
    const int st = P.cpcol[c], en = P.cpcol[c + 1];
    const double sub = z[c] / P.cval[st];
    z[c] = sub;
    for (int q = st + 1; q < en; q++) z[P.crow[q]] -= P.cval[q] * sub;
  }
  z[n - 1] /= P.cval[P.cpcol[n - 1]];
  for (int i = n - 2; i >= 0; i--) {
    double dot = 0.0;
    const int st = P.cpcol[i], en = P.cpcol[i + 1];
    for (int q = st + 1; q < en; q++) dot += z[P.crow[q]] * P.cval[q];
    z[i] = (z[i] - dot) / P.cval[st];
  }
}

// Scalar columns of the symmetric matrix, both triangles, as
// BlockedSymSparseMatrix::getFullIndices lists them (core/sparseMatrix.h:
// 454-523): walking the stored values in index order, value k at lower
// position (R, C) is appended to column C as (R, k) and, off the diagonal,
// to column R as (C, k).
void full_columns(const Scene& s, std::vector<std::vector<std::pair<int, int>>>& cols) {
  const int n = s.dofs;
  cols.assign(n, {});
  auto put = [&](int R, int Cc, int k) {
    cols[Cc].push_back({R, k});
    if (R != Cc) cols[R].push_back({Cc, k});
  };
  for (int bc = 0; bc < s.nbc; bc++) {
    int c0 = 3 * bc, off = s.oris[bc];
    for (int k = s.pcol[bc]; k < s.pcol[bc + 1]; k++) {
      int r0 = s.rows[k];
      if (r0 == c0) {
        static const int di[3] = {0, 3, 5};
        for (int sc = 0; sc < 3; sc++)
          for (int sr = sc; sr < 3; sr++) put(c0 + sr, c0 + sc, off + sr - sc + di[sc]);
        off += 6;
      } else {
        int w = std::min(3, n - r0);
        for (int sc = 0; sc < 3; sc++)
          for (int sr = 0; sr < w; sr++) put(r0 + sr, c0 + sc, off + sc * w + sr);
        off += 3 * w;
      }
    }
  }
  for (int k = 0; k < s.nrem; k++) {
    int col = s.nbc + k, c = 3 * s.nbc + k, off = s.oris[col];
    for (int q = s.pcol[col]; q < s.pcol[col + 1]; q++, off++) put(s.rows[q], c, off);
  }
}

// InLDLTPreconditioner::incompleteLDLTDecomposition
// (solver/inLDLTPreconditioner.cpp:34-149).  Z starts as the identity; step
// i takes column z_i, forms v = A z_i (SpMSV over the full columns), d_i =
// z_i . v, then p_j = v . z_j for every later column meeting v's rows (rows
// visited in v's first-touch order, each row's Z entries newest first),
// stores L_ji = p_j / d_i when |L_ji| > ldltEpsilon, and replaces z_j by
// z_j - (p_j / d_i) z_i keeping entries with |.| > sainvEpsilon.  Each row
// keeps every entry ever written to it with the column's generation at the
// time; an entry is live while its column is still pending and the
// generation is current.
void ldlt_factor(const Scene& s, const double* val, Precond& P) {
  const int n = s.dofs;
  std::vector<std::vector<std::pair<int, int>>> cols;
  full_columns(s, cols);
  struct RowEntry { int col, gen; double v; };
  std::vector<std::vector<std::pair<int, double>>> Z(n);
  std::vector<std::vector<RowEntry>> rowsZ(n);
  std::vector<int> gen(n, 0);
  std::vector<char> done(n, 0);
  for (int j = 0; j < n; j++) { Z[j].push_back({j, 1.0}); rowsZ[j].push_back({j, 0, 1.0}); }
  P.lval.clear(); P.lrow.clear(); P.lpcol.assign(n > 0 ? 1 : 0, 0); P.dinv.assign(n, 0.0);
  if (n == 0) return;
  TouchVec v(n), low(n), w(n);
  auto a_times = [&](const std::vector<std::pair<int, double>>& zi) {
    for (auto& e : zi)
      for (auto& pr : cols[e.first]) v.add(pr.first, val[pr.second] * e.second);
    double d = 0.0;
    for (auto& e : zi) d += e.second * v.get(e.first);
    return d;
  };
  for (int i = 0; i + 1 < n; i++) {
    std::vector<std::pair<int, double>> zi;
    zi.swap(Z[i]);
    done[i] = 1;
    const double inv = 1.0 / a_times(zi);
    P.dinv[i] = inv;
    for (size_t k = 0; k < v.idx.size(); k++) {
      const double x = v.val[k];
      if (x == 0.0) continue;
      const std::vector<RowEntry>& re = rowsZ[v.idx[k]];
      for (size_t q = re.size(); q-- > 0;) {
        const RowEntry& e = re[q];
        if (!done[e.col] && e.gen == gen[e.col]) low.add(e.col, x * e.v);
      }
    }
    for (size_t k = 0; k < low.idx.size(); k++) {
      const double l = low.val[k] * inv;
      if (fabs(l) > P.ldlt_eps) { P.lval.push_back(l); P.lrow.push_back(low.idx[k]); }
    }
    P.lpcol.push_back((int)P.lval.size());
    v.clear();
    for (size_t k = 0; k < low.idx.size(); k++) {
      if (low.val[k] == 0.0) continue;
      const double f = low.val[k] * inv;
      const int j = low.idx[k];
      for (auto& e : Z[j]) w.add(e.first, e.second);
      gen[j]++;
      for (auto& e : zi) w.add(e.first, -f * e.second);
      Z[j].clear();
      for (size_t m = 0; m < w.idx.size(); m++)
        if (fabs(w.val[m]) > P.sainv_eps) {
          Z[j].push_back({w.idx[m], w.val[m]});
          rowsZ[w.idx[m]].push_back({j, gen[j], w.val[m]});
        }
      w.clear();
    }
    low.clear();
  }
  P.dinv[n - 1] = 1.0 / a_times(Z[n - 1]);
}

// InLDLTPreconditioner::solvePreconditionerSystem (:151-184): L y = r by
// columns, y *= D^-1, L^T z = y by row dots from the last row up.
void ldlt_apply(int n, const Precond& P, const double* r, double* z) {
  memcpy(z, r, sizeof(double) * n);
  for (int c = 0; c + 1 < n; c++) {
    const double sub = z[c];
    for (int q = P.lpcol[c]; q < P.lpcol[c + 1]; q++) z[P.lrow[q]] -= P.lval[q] * sub;
  }
  for (int i = 0; i < n; i++) z[i] *= P.dinv[i];
  for (int i = n - 2; i >= 0; i--) {
    double dot = 0.0;
    for (int q = P.lpcol[i]; q < P.lpcol[i + 1]; q++) dot += z[P.lrow[q]] * P.lval[q];
    z[i] -= dot;
  }
}

// row-oriented (up-looking) IC(0) of A + alpha diag(A) on the stored lower
// pattern: for row i and each stored column j < i,
//   L_ij = (A_ij - sum_{k<j} L_ik L_jk) / L_jj,
//   L_ii = sqrt(A_ii (1 + alpha) - sum_{k<i} L_ik^2).
// Returns false on breakdown (a pivot not above 1e-12 times its diagonal).
bool ic0_factor(Precond& P, const double* val, const std::vector<int>& src, int n, double alpha) {
  for (size_t k = 0; k < src.size(); k++) P.lv[k] = src[k] >= 0 ? val[src[k]] : 0.0;
  for (int i = 0; i < n; i++) {
    int bi = P.rp[i], ei = P.rp[i + 1];
    for (int q = bi; q < ei; q++) {
      int j = P.ci[q];
      double sum = P.lv[q];
      if (j == i) sum *= (1.0 + alpha);
      int a = bi, b = P.rp[j], eb = P.rp[j + 1] - 1;  // row j's last entry is its diagonal
      while (a < q && b < eb) {
        if (P.ci[a] == P.ci[b]) { sum -= P.lv[a] * P.lv[b]; a++; b++; }
        else if (P.ci[a] < P.ci[b]) a++;
        else b++;
      }
      if (j < i) {
        P.lv[q] = sum / P.lv[P.rp[j + 1] - 1];
      } else {
        double d = val[src[q]] * (1.0 + alpha);
        if (!(sum > 1e-12 * d)) return false;
        P.lv[q] = sqrt(sum);
      }
    }
  }
  return true;
}

void scalar_lower_csr(const Scene& s, std::vector<int>& rp, std::vector<int>& ci, std::vector<int>& src) {
  const int n = s.dofs;
  std::vector<std::vector<std::pair<int, int>>> rowsv(n);
  for (int bc = 0; bc < s.nbc; bc++) {
    int c0 = 3 * bc, off = s.oris[bc];
    for (int k = s.pcol[bc]; k < s.pcol[bc + 1]; k++) {
      int r0 = s.rows[k];
      if (r0 == c0) {
        static const int di[3] = {0, 3, 5};
        for (int sc = 0; sc < 3; sc++)
          for (int sr = sc; sr < 3; sr++) rowsv[c0 + sr].push_back({c0 + sc, off + sr - sc + di[sc]});
        off += 6;
      } else {
        int w = std::min(3, n - r0);
        for (int sc = 0; sc < 3; sc++)
          for (int sr = 0; sr < w; sr++) rowsv[r0 + sr].push_back({c0 + sc, off + sc * w + sr});
        off += 3 * w;
      }
    }
  }
  for (int k = 0; k < s.nrem; k++) {
    int col = s.nbc + k, c = 3 * s.nbc + k, off = s.oris[col];
    for (int q = s.pcol[col]; q < s.pcol[col + 1]; q++, off++) rowsv[s.rows[q]].push_back({c, off});
  }
  rp.assign(n + 1, 0);
  ci.clear(); src.clear();
  for (int r = 0; r < n; r++) {
    std::sort(rowsv[r].begin(), rowsv[r].end());
    for (auto& p : rowsv[r]) { ci.push_back(p.first); src.push_back(p.second); }
    rp[r + 1] = (int)ci.size();
  }
}

// The IC(0) pattern in the factor's order (see Precond): rows rp/ci, the
// reference-layout position of every entry (src, -1 where none is stored)
// and newdof.
void ic0_pattern(const Scene& s, bool natural, std::vector<int>& rp, std::vector<int>& ci, std::vector<int>& src,
                 std::vector<int>& newdof) {
  const int n = s.dofs, nb = (n + 2) / 3;
  std::vector<int> lrp, lci, lsrc;
  scalar_lower_csr(s, lrp, lci, lsrc);
  std::vector<std::vector<int>> adj(nb);
  for (int i = 0; i < n; i++)
    for (int q = lrp[i]; q < lrp[i + 1]; q++) {
      const int bi = i / 3, bj = lci[q] / 3;
      if (bi != bj) { adj[bi].push_back(bj); adj[bj].push_back(bi); }
    }
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  std::vector<int> order(nb);
  for (int b = 0; b < nb; b++) order[b] = b;
  if (!natural) {
    std::vector<int> colour(nb, -1);
    for (int b = 0; b < nb; b++) {
      std::vector<char> used;
      for (int c : adj[b])
        if (colour[c] >= 0) {
          if ((int)used.size() <= colour[c]) used.resize(colour[c] + 1, 0);
          used[colour[c]] = 1;
        }
      int c = 0;
      while (c < (int)used.size() && used[c]) c++;
      colour[b] = c;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return colour[a] < colour[b]; });
  }
  std::vector<int> newblock(nb);
  for (int R = 0; R < nb; R++) newblock[order[R]] = R;
  newdof.assign(n, 0);
  int next = 0;
  for (int R = 0; R < nb; R++)
    for (int d = 3 * order[R]; d < std::min(n, 3 * order[R] + 3); d++) newdof[d] = next++;
  auto lookup = [&](int i, int j) {   // reference-layout position of (i, j), j <= i, or -1
    const int* b = &lci[lrp[i]];
    const int* e = &lci[lrp[i + 1]];
    const int* f = std::lower_bound(b, e, j);
    return (f != e && *f == j) ? lsrc[lrp[i] + (int)(f - b)] : -1;
  };
  std::vector<std::vector<std::pair<int, int>>> rowsv(n);
  for (int b = 0; b < nb; b++) {
    std::vector<int> nbrs = adj[b];
    nbrs.push_back(b);
    for (int i = 3 * b; i < std::min(n, 3 * b + 3); i++)
      for (int b2 : nbrs)
        for (int j = 3 * b2; j < std::min(n, 3 * b2 + 3); j++)
          if (newdof[j] <= newdof[i]) rowsv[newdof[i]].push_back({newdof[j], lookup(std::max(i, j), std::min(i, j))});
  }
  rp.assign(n + 1, 0);
  ci.clear();
  src.clear();
  for (int r = 0; r < n; r++) {
    std::sort(rowsv[r].begin(), rowsv[r].end());
    for (auto& e : rowsv[r]) { ci.push_back(e.first); src.push_back(e.second); }
    rp[r + 1] = (int)ci.size();
  }
}

void precond_setup(const Scene& s, const double* val, Precond& P) {
  const int n = s.dofs;
  if (P.kind == 1) {
    P.inv.resize(n);
    diagonal(s, val, P.inv.data());
    for (int i = 0; i < n; i++) P.inv[i] = P.inv[i] > 0.0 ? 1.0 / P.inv[i] : 1.0;
  } else if (P.kind == 2) {
    P.inv.assign(9 * s.nbc + s.nrem, 0.0);
    for (int bc = 0; bc < s.nbc; bc++) {
      const double* v = val + s.oris[bc];
      double m[9] = {v[0], v[1], v[2], v[1], v[3], v[4], v[2], v[4], v[5]};
      inverse3(m, &P.inv[9 * bc]);
    }
    for (int k = 0; k < s.nrem; k++) {
      double d = val[s.oris[s.nbc + k]];
      P.inv[9 * s.nbc + k] = d > 0.0 ? 1.0 / d : 1.0;
    }
  } else if (P.kind == 3) {
    std::vector<int> src;
    ic0_pattern(s, P.natural != 0, P.rp, P.ci, src, P.newdof);
    P.lv.resize(P.ci.size());
    // shifted IC(0): factor A + alpha diag(A) with alpha = 0, 1e-3, 2e-3, ...
    // until every pivot exceeds 1e-12 times its shifted diagonal
    double alpha = 0.0;
    for (int attempt = 0; attempt < 40; attempt++) {
      if (ic0_factor(P, val, src, n, alpha)) break;
      alpha = alpha == 0.0 ? 1e-3 : 2.0 * alpha;
    }
    P.shift = alpha;
  } else if (P.kind == 4) {
    ldlt_factor(s, val, P);
  } else if (P.kind == 5) {
    ric_factor(s, val, P);
  }
}

void precond_apply(const Scene& s, const Precond& P, const double* r, double* z) {
  const int n = s.dofs;
  if (P.kind == 0) memcpy(z, r, sizeof(double) * n);
  else if (P.kind == 1) for (int i = 0; i < n; i++) z[i] = P.inv[i] * r[i];
  else if (P.kind == 2) {
    for (int bc = 0; bc < s.nbc; bc++) {
      const double* m = &P.inv[9 * bc];
      const double* rr = r + 3 * bc;
      for (int i = 0; i < 3; i++) z[3 * bc + i] = m[3 * i] * rr[0] + m[3 * i + 1] * rr[1] + m[3 * i + 2] * rr[2];
    }
    for (int k = 0; k < s.nrem; k++) z[3 * s.nbc + k] = P.inv[9 * s.nbc + k] * r[3 * s.nbc + k];
  } else if (P.kind == 4) {
    ldlt_apply(n, P, r, z);
  } else if (P.kind == 5) {
    ric_apply(n, P, r, z);
  } else {
    std::vector<double> y(n);   // in the factor's order
    for (int i = 0; i < n; i++) y[P.newdof[i]] = r[i];
    for (int i = 0; i < n; i++) {
      double sum = y[i];
      int e = P.rp[i + 1] - 1;
      for (int q = P.rp[i]; q < e; q++) sum -= P.lv[q] * y[P.ci[q]];
      y[i] = sum / P.lv[e];
    }
    for (int i = n - 1; i >= 0; i--) {
      int e = P.rp[i + 1] - 1;
      y[i] /= P.lv[e];
      double yi = y[i];
      for (int q = P.rp[i]; q < e; q++) y[P.ci[q]] -= P.lv[q] * yi;
    }
    for (int i = 0; i < n; i++) z[i] = y[P.newdof[i]];
  }
}

// PCG (solver/cgSolver.cpp:13-57): warm start from x, stop when
// ||r||^2 <= tol^2 ||b||^2 or after maxit iterations.
int pcg(const Scene& s, const double* val, const double* b, double* x, double tol, int maxit, int pkind) {
  const int n = s.dofs;
  std::vector<double> r(n, 0.0), d(n, 0.0), t(n, 0.0);
  spmdv(s, val, x, r.data());
  for (int i = 0; i < n; i++) r[i] = b[i] - r[i];
  Precond P;
  P.kind = pkind;
  P.sainv_eps = s.ldlt_sainv;
  P.ldlt_eps = s.ldlt_drop;
  P.ic_eps = s.ic_eps;
  P.ic_relax = s.ic_relax;
  P.natural = s.ic0_natural;
  precond_setup(s, val, P);
  precond_apply(s, P, r.data(), d.data());
  auto dotp = [n](const double* a, const double* c) { double acc = 0; for (int i = 0; i < n; i++) acc += a[i] * c[i]; return acc; };
  double delta = dotp(r.data(), d.data());
  double eps = dotp(b, b) * tol * tol;
  double rn = dotp(r.data(), r.data());
  int it = 0;
  while (it < maxit && rn > eps) {
    it++;
    std::fill(t.begin(), t.end(), 0.0);
    spmdv(s, val, d.data(), t.data());
    double alpha = delta / dotp(d.data(), t.data());
    for (int i = 0; i < n; i++) { x[i] += alpha * d[i]; r[i] -= alpha * t[i]; }
    precond_apply(s, P, r.data(), t.data());
    double pd = delta;
    delta = dotp(r.data(), t.data());
    double beta = delta / pd;
    for (int i = 0; i < n; i++) d[i] = beta * d[i] + t[i];
    rn = dotp(r.data(), r.data());
  }
  return it;
}

// ------------------------------------------------- plane collision damping
// Plane n.x + c = 0 against a deformed tetrahedron P[4]
// (collision/intersection.cpp:12-117): the part of the tetrahedron on the
// negative side (n.x + c < 1e-6) gives a centroid and a direction whose
// length is six times that part's volume (all four vertices inside: the
// plane normal times the full volume; none: the vertex nearest the plane
// and a zero direction).  Edge points are clamped to the edge.
V3 plane_edge_point(V3 n, double c, V3 pa, V3 pb) {
  V3 ab = sub(pb, pa);
  double t = (-c - dot(n, pa)) / dot(n, ab);
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  return add(pa, scale(ab, t));
}

V3 unit(V3 a) { return divv(a, sqrt(len2(a))); }

void plane_tet(V3 n, double c, const V3* P, V3& centroid, V3& dir) {
  V3 neg[4], pos[4];
  int nn = 0, np = 0;
  for (int i = 0; i < 4; i++) {
    if (dot(n, P[i]) + c < 1e-6) neg[nn++] = P[i];
    else pos[np++] = P[i];
  }
  if (nn == 0) {
    double best = 1.7976931348623157e308;
    for (int i = 0; i < 4; i++) {
      double d = dot(n, P[i]) + c;
      if (d < best) { best = d; centroid = P[i]; }
    }
    dir = {0.0, 0.0, 0.0};
  } else if (nn == 1) {
    V3 q0 = plane_edge_point(n, c, neg[0], pos[0]);
    V3 q1 = plane_edge_point(n, c, neg[0], pos[1]);
    V3 q2 = plane_edge_point(n, c, neg[0], pos[2]);
    centroid = scale(add(add(add(neg[0], q0), q1), q2), 0.25);
    V3 ab = sub(q0, neg[0]), ac = sub(q1, neg[0]), ad = sub(q2, neg[0]);
    double sv = dot(ab, cross(ac, ad));
    dir = scale(unit(add(add(cross(ab, ac), cross(ac, ad)), cross(ad, ab))), fabs(sv));
    if (sv < 0.0) dir = scale(dir, -1.0);
  } else if (nn == 2) {
    V3 q0 = plane_edge_point(n, c, neg[0], pos[0]);
    V3 q1 = plane_edge_point(n, c, neg[0], pos[1]);
    V3 q2 = plane_edge_point(n, c, neg[1], pos[0]);
    V3 q3 = plane_edge_point(n, c, neg[1], pos[1]);
    V3 ab = sub(neg[1], neg[0]);
    V3 c0 = add(add(add(neg[0], neg[1]), q2), q3);
    double v0 = fabs(dot(sub(neg[1], neg[0]), cross(sub(q2, neg[0]), sub(q3, neg[0]))));
    V3 c1 = add(add(add(neg[0], q0), q1), q2);
    double v1 = fabs(dot(sub(q0, neg[0]), cross(sub(q1, neg[0]), sub(q2, neg[0]))));
    V3 c2 = add(add(add(neg[0], q1), q2), q3);
    double v2 = fabs(dot(sub(q1, neg[0]), cross(sub(q2, neg[0]), sub(q3, neg[0]))));
    centroid = scale(divv(add(add(scale(c0, v0), scale(c1, v1)), scale(c2, v2)), v0 + v1 + v2), 0.25);
    V3 d = add(add(add(add(add(cross(sub(q0, neg[0]), sub(q1, neg[0])), cross(sub(q3, neg[1]), sub(q2, neg[1]))),
                       cross(ab, sub(q2, neg[0]))), cross(sub(q2, neg[0]), sub(q0, neg[0]))),
                   cross(sub(q3, neg[0]), ab)), cross(sub(q1, neg[0]), sub(q3, neg[0])));
    dir = scale(unit(d), v0 + v1 + v2);
    if (dot(sub(neg[1], neg[0]), cross(sub(pos[0], neg[0]), sub(pos[1], neg[0]))) < 0.0) dir = scale(dir, -1.0);
  } else if (nn == 3) {
    V3 q0 = plane_edge_point(n, c, neg[0], pos[0]);
    V3 q1 = plane_edge_point(n, c, neg[1], pos[0]);
    V3 q2 = plane_edge_point(n, c, neg[2], pos[0]);
    V3 ab = sub(q0, pos[0]), ac = sub(q1, pos[0]), ad = sub(q2, pos[0]);
    V3 cs = add(add(add(P[0], P[1]), P[2]), P[3]);
    double sv = dot(sub(neg[0], pos[0]), cross(sub(neg[1], pos[0]), sub(neg[2], pos[0])));
    double v = fabs(sv);
    V3 c0 = add(add(add(pos[0], q0), q1), q2);
    double v0 = fabs(dot(ab, cross(ac, ad)));
    centroid = scale(divv(sub(scale(cs, v), scale(c0, v0)), v - v0), 0.25);
    dir = scale(unit(add(add(cross(ab, ac), cross(ac, ad)), cross(ad, ab))), v - v0);
    if (sv > 0.0) dir = scale(dir, -1.0);
  } else {
    centroid = scale(add(add(add(P[0], P[1]), P[2]), P[3]), 0.25);
    double vol = fabs(dot(sub(P[1], P[0]), cross(sub(P[2], P[0]), sub(P[3], P[0]))));
    dir = scale(n, vol);
  }
}

// barycentric coordinates from sub-volumes (intersection.cpp:119-148); all
// 0.25 when six times the volume is at most 1e-6
void barycentric(const V3* P, V3 p, double w[4]) {
  V3 ab = sub(P[1], P[0]), ac = sub(P[2], P[0]), ad = sub(P[3], P[0]);
  V3 bc = sub(P[2], P[1]), bd = sub(P[3], P[1]);
  V3 ap = sub(p, P[0]), bp = sub(p, P[1]);
  double va = fabs(dot(bp, cross(bc, bd)));
  double vb = fabs(dot(ap, cross(ac, ad)));
  double vc = fabs(dot(ap, cross(ab, ad)));
  double vd = fabs(dot(ap, cross(ab, ac)));
  double vol = fabs(dot(ab, cross(ac, ad)));
  if (vol <= 1e-6) { w[0] = w[1] = w[2] = w[3] = 0.25; return; }
  double inv = 1.0 / vol;
  w[0] = va * inv; w[1] = vb * inv; w[2] = vc * inv; w[3] = vd * inv;
}

// MeshPlaneCollisionDampingForcer::addDampingMatrix
// (collision/penaltyDampingForcer.cpp:8-61) for element e: with w the
// barycentric coordinates of the centroid, u = dir / |dir| and the velocity
// there approaching the plane (v.u < 0), the 12x12 block (a, b) of the
// element matrix receives w_a w_b T with T = (coeff dir) u^T; packed entries
// (row-wise upper triangle).  In the reference the diagonal blocks take
// T(i, j) for the entry (i, i + j) -- kept as it is.  Returns false when
// nothing is added.
bool plane_damping_element(const Scene& s, int e, const V3* vel, V3 n, double c, double coeff, double out[78]) {
  static const int diag[12] = {0, 12, 23, 33, 42, 50, 57, 63, 68, 72, 75, 77};
  const int* t = &s.tets[4 * e];
  V3 P[4];
  for (int i = 0; i < 4; i++) P[i] = add(s.X[t[i]], s.u[t[i]]);
  V3 cen = {0.0, 0.0, 0.0}, dir = {0.0, 0.0, 0.0};   // (the reference's Vector3 starts at zero)
  plane_tet(n, c, P, cen, dir);
  double w[4];
  barycentric(P, cen, w);
  V3 u = {0.0, 0.0, 0.0};
  if (len2(dir) != 0.0) u = unit(dir);
  V3 v = {0.0, 0.0, 0.0};
  for (int i = 0; i < 4; i++) v = add(v, scale(vel[t[i]], w[i]));
  if (!(dot(v, u) < 0.0)) return false;
  V3 cd = scale(dir, coeff);
  double T[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) T[i][j] = at(cd, i) * at(u, j);
  for (int k = 0; k < 78; k++) out[k] = 0.0;
  for (int a = 0; a < 4; a++) {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3 - i; j++) out[diag[3 * a + i] + j] = w[a] * w[a] * T[i][j];
    for (int b = a + 1; b < 4; b++)
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[diag[3 * a + i] + (b - a) * 3 - i + j] = w[a] * w[b] * T[i][j];
  }
  return true;
}

// values += the forcer's contributions of elements elems (in that order)
void plane_damping(const Scene& s, const V3* vel, V3 n, double c, double coeff, int count, const int* elems,
                   double* values) {
  double blk[78];
  for (int k = 0; k < count; k++) {
    const int e = elems[k];
    if (!plane_damping_element(s, e, vel, n, c, coeff, blk)) continue;
    for (int q = 0; q < 78; q++) {
      const int idx = s.emap[78 * (size_t)e + q];
      if (idx >= 0) values[idx] += blk[q];
    }
  }
}

void write_free(Scene& s, const double* d) {
  for (int nd = 0; nd < s.n_nodes; nd++)
    for (int ax = 0; ax < 3; ax++) {
      int g = global_index(s.cd, nd, ax);
      if (g >= 0) {
        if (ax == 0) s.u[nd].x = d[g]; else if (ax == 1) s.u[nd].y = d[g]; else s.u[nd].z = d[g];
      }
    }
}

}  // namespace

// ------------------------------------------------------------------- C API
extern "C" {

struct odo_scene {
  Scene s;
  // integrator state
  std::vector<double> v, dv, a, d, fext, K;
  double h = 0, alphaM = 0, betaK = 0, beta = 0.25, gamma = 0.5, tol = 1e-8;
  int maxit = 1000, pkind = 1, newton = 1;
  Precond ldlt;   // stand-alone incomplete LDL^T factor (odo_ldlt_*)
  Precond ic;     // stand-alone threshold incomplete Cholesky factor (odo_ic_*)
  std::vector<double> D;   // external damping matrix values (empty: none)
};

odo_scene* odo_scene_create(int n_nodes, const double* X, int n_tets, const int* tets, int n_facets,
                            const int* facets, int n_cdofs, const int* cdofs, int kind, double rho,
                            double youngs, double poisson, double threshold) {
  odo_scene* o = new odo_scene();
  Scene& s = o->s;
  s.n_nodes = n_nodes;
  s.n_tets = n_tets;
  s.X.resize(n_nodes);
  s.u.assign(n_nodes, V3{0, 0, 0});
  for (int i = 0; i < n_nodes; i++) s.X[i] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
  s.tets.assign(tets, tets + 4 * (size_t)n_tets);
  s.facets.assign(facets, facets + 3 * (size_t)n_facets);
  s.cd.assign(cdofs, cdofs + n_cdofs);
  std::sort(s.cd.begin(), s.cd.end());
  s.cd.erase(std::unique(s.cd.begin(), s.cd.end()), s.cd.end());
  s.dofs = 3 * n_nodes - (int)s.cd.size();
  s.gidx.resize(12 * (size_t)n_tets);
  for (int e = 0; e < n_tets; e++)
    for (int a = 0; a < 4; a++)
      for (int ax = 0; ax < 3; ax++) s.gidx[12 * e + 3 * a + ax] = global_index(s.cd, s.tets[4 * e + a], ax);
  s.kind = kind;
  s.rho = rho;
  s.thr = threshold;
  // Lame parameters (corotationalHyperelastic.cpp:8-18, invertibleNeoHookean.cpp:5-9)
  s.lambda = poisson * youngs / ((1.0 + poisson) * (1.0 - 2.0 * poisson));
  s.mu = youngs / (2.0 * (1.0 + poisson));
  s.D[0] = s.lambda + 2.0 * s.mu; s.D[1] = s.lambda; s.D[2] = s.mu;
  build_pattern(s);
  build_emap(s);
  build_precomputes(s);
  build_mass(s);
  if (kind == 3) s.plastic.assign(9 * (size_t)n_tets, 0.0);
  return o;
}

// corotational plastic parameters and zero plastic strain for a kind-3
// scene (CorotationalPlasticMaterial ctor, corotationalPlastic.cpp:8-22,
// getPrecomputes :24-51)
void odo_set_plastic(odo_scene* o, double yield, double creep, double max_strain) {
  o->s.yield = yield;
  o->s.creep = creep;
  o->s.max_plastic = max_strain;
  o->s.plastic.assign(9 * (size_t)o->s.n_tets, 0.0);
}
void odo_plastic_state(odo_scene* o, double* out) {
  memcpy(out, o->s.plastic.data(), sizeof(double) * o->s.plastic.size());
}

void odo_scene_destroy(odo_scene* o) { delete o; }
int odo_dofs(odo_scene* o) { return o->s.dofs; }

void odo_pattern_sizes(odo_scene* o, int* sizes) {
  const Scene& s = o->s;
  sizes[0] = s.dofs; sizes[1] = s.nbc; sizes[2] = s.nrem;
  sizes[3] = (int)s.rows.size(); sizes[4] = s.nvals;
}

void odo_pattern(odo_scene* o, int* pcol, int* rows, int* oris, int* emap) {
  const Scene& s = o->s;
  memcpy(pcol, s.pcol.data(), sizeof(int) * s.pcol.size());
  memcpy(rows, s.rows.data(), sizeof(int) * s.rows.size());
  memcpy(oris, s.oris.data(), sizeof(int) * s.oris.size());
  if (emap) memcpy(emap, s.emap.data(), sizeof(int) * s.emap.size());
}

void odo_set_displacements(odo_scene* o, const double* u) {
  for (int i = 0; i < o->s.n_nodes; i++) o->s.u[i] = {u[3 * i], u[3 * i + 1], u[3 * i + 2]};
}
void odo_get_displacements(odo_scene* o, double* u) {
  for (int i = 0; i < o->s.n_nodes; i++) { u[3 * i] = o->s.u[i].x; u[3 * i + 1] = o->s.u[i].y; u[3 * i + 2] = o->s.u[i].z; }
}

void odo_element_values(odo_scene* o, double* K78, double* f12) {
  for (int e = 0; e < o->s.n_tets; e++) element(o->s, e, K78 + 78 * (size_t)e, f12 + 12 * (size_t)e);
}
void odo_assemble(odo_scene* o, double* values, double* fint) { assemble(o->s, values, fint); }
void odo_mass(odo_scene* o, double* values) { memcpy(values, o->s.mass.data(), sizeof(double) * o->s.nvals); }
void odo_spmdv(odo_scene* o, const double* values, const double* x, double* y) { spmdv(o->s, values, x, y); }
// IC(0) node order: 1 keeps the DOF order, 0 (default) orders blocks by colour
void odo_set_ic0_natural(odo_scene* o, int natural) { o->s.ic0_natural = natural; }

int odo_pcg(odo_scene* o, const double* values, const double* b, double* x, double tol, int maxit, int pkind) {
  return pcg(o->s, values, b, x, tol, maxit, pkind);
}

// drop bounds of the incomplete LDL^T (preconditioner kind 4)
void odo_set_ldlt(odo_scene* o, double sainv_eps, double ldlt_eps) {
  o->s.ldlt_sainv = sainv_eps;
  o->s.ldlt_drop = ldlt_eps;
}

// stand-alone factor of A = values (kept for odo_ldlt_get / odo_ldlt_apply);
// returns the number of stored L entries
int odo_ldlt_factor(odo_scene* o, const double* values) {
  o->ldlt = Precond();
  o->ldlt.kind = 4;
  o->ldlt.sainv_eps = o->s.ldlt_sainv;
  o->ldlt.ldlt_eps = o->s.ldlt_drop;
  ldlt_factor(o->s, values, o->ldlt);
  return (int)o->ldlt.lval.size();
}

void odo_ldlt_get(odo_scene* o, double* values, int* rows, int* pcol, double* inv_diag) {
  const Precond& P = o->ldlt;
  if (!P.lval.empty()) memcpy(values, P.lval.data(), sizeof(double) * P.lval.size());
  if (!P.lrow.empty()) memcpy(rows, P.lrow.data(), sizeof(int) * P.lrow.size());
  if (!P.lpcol.empty()) memcpy(pcol, P.lpcol.data(), sizeof(int) * P.lpcol.size());
  if (!P.dinv.empty()) memcpy(inv_diag, P.dinv.data(), sizeof(double) * P.dinv.size());
}

void odo_ldlt_apply(odo_scene* o, const double* rhs, double* out) { ldlt_apply(o->s.dofs, o->ldlt, rhs, out); }

// threshold incomplete Cholesky (preconditioner kind 5): parameters, a
// stand-alone factor of A = values (returns its stored entries), its
// arrays and its apply
void odo_set_ic(odo_scene* o, double eps, double relax) {
  o->s.ic_eps = eps;
  o->s.ic_relax = relax;
}
int odo_ic_factor(odo_scene* o, const double* values) {
  o->ic = Precond();
  o->ic.kind = 5;
  o->ic.ic_eps = o->s.ic_eps;
  o->ic.ic_relax = o->s.ic_relax;
  ric_factor(o->s, values, o->ic);
  return (int)o->ic.cval.size();
}
void odo_ic_get(odo_scene* o, double* values, int* rows, int* pcol) {
  const Precond& P = o->ic;
  if (!P.cval.empty()) memcpy(values, P.cval.data(), sizeof(double) * P.cval.size());
  if (!P.crow.empty()) memcpy(rows, P.crow.data(), sizeof(int) * P.crow.size());
  if (!P.cpcol.empty()) memcpy(pcol, P.cpcol.data(), sizeof(int) * P.cpcol.size());
}
void odo_ic_apply(odo_scene* o, const double* rhs, double* out) { ric_apply(o->s.dofs, o->ic, rhs, out); }

// plane collision damping values (reference layout, from zero) for elements
// elems against the plane normal.x + constant = 0, node velocities vel
void odo_plane_damping(odo_scene* o, const double* vel, const double* normal, double constant, double coeff, int n,
                       const int* elems, double* values) {
  const Scene& s = o->s;
  std::vector<V3> v(s.n_nodes);
  for (int i = 0; i < s.n_nodes; i++) v[i] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
  memset(values, 0, sizeof(double) * s.nvals);
  plane_damping(s, v.data(), {normal[0], normal[1], normal[2]}, constant, coeff, n, elems, values);
}

// the integrators' external damping matrix: cleared (clearExternalDampingForceMatrix),
// or replaced by the plane forcer with the integrator's node velocities
// (getMeshVerticesVelocities: constrained DOFs 0)
void odo_clear_damping(odo_scene* o) { o->D.clear(); }
void odo_integrator_plane_damping(odo_scene* o, const double* normal, double constant, double coeff, int n,
                                  const int* elems) {
  const Scene& s = o->s;
  std::vector<V3> v(s.n_nodes, V3{0.0, 0.0, 0.0});
  for (int nd = 0; nd < s.n_nodes; nd++)
    for (int ax = 0; ax < 3; ax++) {
      const int g = global_index(s.cd, nd, ax);
      const double x = g >= 0 ? o->v[g] : 0.0;
      if (ax == 0) v[nd].x = x; else if (ax == 1) v[nd].y = x; else v[nd].z = x;
    }
  o->D.assign(s.nvals, 0.0);
  plane_damping(s, v.data(), {normal[0], normal[1], normal[2]}, constant, coeff, n, elems, o->D.data());
}

// Loads (Forcer, core/forcer.cpp:8-96): body force density times V/4 per
// node (tetelement.cpp:68-77), tractions times the deformed facet area / 3
// per vertex (tetelement.cpp:79-89); constrained DOFs dropped.
void odo_loads(odo_scene* o, const double* body, int n_groups, const double* tractions,
               const int* group_sizes, const int* facet_ids, double* fext) {
  Scene& s = o->s;
  memset(fext, 0, sizeof(double) * s.dofs);
  if (body) {
    for (int e = 0; e < s.n_tets; e++) {
      const int* t = &s.tets[4 * e];
      double vol = tet_volume(node_pos(s, t[0]), node_pos(s, t[1]), node_pos(s, t[2]), node_pos(s, t[3]));
      double f = vol / 4.0;
      for (int a = 0; a < 4; a++)
        for (int ax = 0; ax < 3; ax++) {
          double w = f * body[ax];
          int g = s.gidx[12 * e + 3 * a + ax];
          if (w != 0.0 && g >= 0) fext[g] += w;
        }
    }
  }
  int q = 0;
  for (int gi = 0; gi < n_groups; gi++) {
    const double* tr = tractions + 3 * gi;
    for (int k = 0; k < group_sizes[gi]; k++, q++) {
      const int* fc = &s.facets[3 * facet_ids[q]];
      V3 a = node_cur(s, fc[0]), b = node_cur(s, fc[1]), c = node_cur(s, fc[2]);
      double area = sqrt(len2(cross(sub(b, a), sub(c, a)))) * 0.5;
      double f = area / 3.0;
      for (int vtx = 0; vtx < 3; vtx++)
        for (int ax = 0; ax < 3; ax++) {
          double w = f * tr[ax];
          int g = global_index(s.cd, fc[vtx], ax);
          if (w != 0.0 && g >= 0) fext[g] += w;
        }
    }
  }
}

void odo_integrator_setup(odo_scene* o, double dt, double alphaM, double betaK, double beta, double gamma,
                          int newton, double tol, int maxit, int pkind) {
  const int n = o->s.dofs;
  o->h = dt; o->alphaM = alphaM; o->betaK = betaK; o->beta = beta; o->gamma = gamma;
  o->newton = newton; o->tol = tol; o->maxit = maxit; o->pkind = pkind;
  o->v.assign(n, 0.0); o->dv.assign(n, 0.0); o->a.assign(n, 0.0); o->d.assign(n, 0.0);
  o->fext.assign(n, 0.0); o->K.assign(o->s.nvals, 0.0);
}

void odo_set_fext(odo_scene* o, const double* f) { memcpy(o->fext.data(), f, sizeof(double) * o->s.dofs); }

// backward Euler (intergrator/nonlinearImplicitBackwardEuler.h:82-116), with
// the per-step displacement write-back u += h v on free DOFs
int odo_be_step(odo_scene* o, int nsteps) {
  Scene& s = o->s;
  const int n = s.dofs;
  std::vector<double> fint(n), rhs(n);
  int iters = 0;
  for (int st = 0; st < nsteps; st++) {
    assemble(s, o->K.data(), fint.data());
    for (int i = 0; i < s.nvals; i++) o->K[i] = o->K[i] * (o->h + o->betaK) + o->alphaM * s.mass[i];
    if (!o->D.empty())   // tagentMatrix->Add(1, *dampMatrix) (nonlinearImplicitBackwardEuler.h:88)
      for (int i = 0; i < s.nvals; i++) o->K[i] += o->D[i];
    std::fill(rhs.begin(), rhs.end(), 0.0);
    spmdv(s, o->K.data(), o->v.data(), rhs.data());
    for (int i = 0; i < n; i++) rhs[i] = o->h * (o->fext[i] - fint[i] - rhs[i]);
    for (int i = 0; i < s.nvals; i++) o->K[i] = o->K[i] * o->h + s.mass[i];
    iters += pcg(s, o->K.data(), rhs.data(), o->dv.data(), o->tol, o->maxit, o->pkind);
    for (int i = 0; i < n; i++) o->v[i] += o->dv[i];
    for (int nd = 0, k = 0; nd < s.n_nodes; nd++)
      for (int ax = 0; ax < 3; ax++) {
        if (global_index(s.cd, nd, ax) < 0) continue;
        double du = o->v[k++] * o->h;
        if (ax == 0) s.u[nd].x += du; else if (ax == 1) s.u[nd].y += du; else s.u[nd].z += du;
      }
  }
  return iters;
}

// Full-order Newmark (beta, gamma) with a Newton loop on the acceleration.
// No reference counterpart at full order; the predictor/corrector formulas are
// those of the reference's modal integrator (intergrator/linearNewmark.cpp:
// 27-30, 57-79) applied to every DOF, with damping C = alpha_M M + beta_K K(d)
// (+ the external damping matrix D when one is set, in r and in A as gamma h D):
//   d~ = d + h v + (1/2 - beta) h^2 a;   v~ = v + (1 - gamma) h a
//   a_0 = a; for k < newton:
//     d_k = d~ + beta h^2 a_k;  v_k = v~ + gamma h a_k   (d_k written to the mesh)
//     r = f_ext - f_int(d_k) - [M (alpha_M v_k + a_k) + beta_K K v_k]
//     A = (1 + gamma h alpha_M) M + (gamma h beta_K + beta h^2) K
//     PCG(A, r) from da = 0;  a_{k+1} = a_k + da
//   d = d~ + beta h^2 a;  v = v~ + gamma h a
int odo_nm_step(odo_scene* o, int nsteps) {
  Scene& s = o->s;
  const int n = s.dofs;
  const double h = o->h, bh2 = o->beta * h * h, gh = o->gamma * h;
  std::vector<double> dp(n), vp(n), fint(n), r(n), t1(n), t2(n), y(n), da(n);
  int iters = 0;
  for (int st = 0; st < nsteps; st++) {
    for (int i = 0; i < n; i++) {
      dp[i] = o->d[i] + h * o->v[i] + (0.5 - o->beta) * h * h * o->a[i];
      vp[i] = o->v[i] + (1.0 - o->gamma) * h * o->a[i];
    }
    for (int it = 0; it < o->newton; it++) {
      for (int i = 0; i < n; i++) t1[i] = dp[i] + bh2 * o->a[i];
      write_free(s, t1.data());
      assemble(s, o->K.data(), fint.data());
      for (int i = 0; i < n; i++) {
        double vk = vp[i] + gh * o->a[i];
        t1[i] = o->alphaM * vk + o->a[i];
        t2[i] = vk;
      }
      std::fill(y.begin(), y.end(), 0.0);
      spmdv(s, s.mass.data(), t1.data(), y.data());
      std::fill(t1.begin(), t1.end(), 0.0);
      spmdv(s, o->K.data(), t2.data(), t1.data());
      if (!o->D.empty()) spmdv(s, o->D.data(), t2.data(), y.data());   // + D v_k
      for (int i = 0; i < n; i++) r[i] = o->fext[i] - fint[i] - (y[i] + o->betaK * t1[i]);
      const double cK = gh * o->betaK + bh2, cM = 1.0 + gh * o->alphaM;
      for (int i = 0; i < s.nvals; i++) o->K[i] = o->K[i] * cK + cM * s.mass[i];
      if (!o->D.empty())
        for (int i = 0; i < s.nvals; i++) o->K[i] += gh * o->D[i];
      std::fill(da.begin(), da.end(), 0.0);
      iters += pcg(s, o->K.data(), r.data(), da.data(), o->tol, o->maxit, o->pkind);
      for (int i = 0; i < n; i++) o->a[i] += da[i];
    }
    for (int i = 0; i < n; i++) {
      o->d[i] = dp[i] + bh2 * o->a[i];
      o->v[i] = vp[i] + gh * o->a[i];
    }
    write_free(s, o->d.data());
  }
  return iters;
}

void odo_state(odo_scene* o, double* d, double* v, double* a) {
  const int n = o->s.dofs;
  if (d) memcpy(d, o->d.data(), sizeof(double) * n);
  if (v) memcpy(v, o->v.data(), sizeof(double) * n);
  if (a) memcpy(a, o->a.data(), sizeof(double) * n);
}

void odo_polar(const double* F, double* R, double* S) { polar3(F, R, S); }
void odo_qr(const double* F, double* Q, double* R) { qr3(F, Q, R); }
void odo_eigsym(const double* tri6, double* vals, double* vecs) { eigsym3(tri6, vals, vecs); }

}  // extern "C"
