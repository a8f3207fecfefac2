// Per-tetrahedron kernels: precomputes, mass, loads and the material
// kernels (corotational linear, invertible Neo-Hookean / StVK) producing the
// 78 packed stiffness values and 12 nodal forces of every element, scattered
// without atomics: elements are coloured so that one launch (one colour)
// never touches a matrix value or force entry twice.
//
// One thread per element; element data is structure-of-arrays in colour
// order (pre[k * ne + e], emap[k * ne + e]) so every per-element load and the
// map loads are coalesced.  The staged outputs (the gathered assembly's
// input) are element-major, grouped by local node block (c_kslot below).
#include "od_internal.h"
#include "od_math.cuh"

namespace od {

// packed position of (i, i) in the 78-entry upper triangle of the 12x12
// element matrix (tetelement.cpp:284)
__constant__ int c_diag12[12] = {0, 12, 23, 33, 42, 50, 57, 63, 68, 72, 75, 77};

// Staged element values (the assembly's input) are element-major: 78
// stiffness values per element with the entries of each local node block
// contiguous -- blocks (0,0), (0,1), (0,2), (0,3), (1,1), ..., (3,3), a
// diagonal block's 6 upper entries, an off-diagonal block's 9 row-major --
// so that the assembly threads of one matrix block read one contiguous run
// of each contributing element; then 12 forces per element in local DOF
// order.  c_kslot maps the packed entry k (row-major upper triangle, the
// reference's order) to its slot.
__constant__ int c_kslot[78] = {0,  1,  2,  6,  7,  8,  15, 16, 17, 24, 25, 26, 3,  4,  9,  10, 11, 18, 19, 20,
                                27, 28, 29, 5,  12, 13, 14, 21, 22, 23, 30, 31, 32, 33, 34, 35, 39, 40, 41, 48,
                                49, 50, 36, 37, 42, 43, 44, 51, 52, 53, 38, 45, 46, 47, 54, 55, 56, 57, 58, 59,
                                63, 64, 65, 60, 61, 66, 67, 68, 62, 69, 70, 71, 72, 73, 74, 75, 76, 77};
__device__ __forceinline__ size_t kst(int k, int e) { return (size_t)e * 78 + c_kslot[k]; }
__device__ __forceinline__ size_t fst(int k, int e) { return (size_t)e * 12 + k; }

__device__ __forceinline__ V3t<double> ld3(const double* p, int n) {
  return {p[3 * n], p[3 * n + 1], p[3 * n + 2]};
}

__device__ __forceinline__ double tet_vol(V3t<double> a, V3t<double> b, V3t<double> c, V3t<double> d) {
  V3t<double> ab = v_sub(b, a), ac = v_sub(c, a), ad = v_sub(d, a);
  return fabs(v_dot(ab, v_cross(ac, ad))) / 6.0;
}

// ------------------------------------------------------------ precomputes
// getCorotationalTetElementPrecomputes (tetelement.cpp:501-544) and
// InvertibleHyperelasticTetElement::getPrecomputes (tetelement.cpp:253-266),
// written in element (colour) order.
__global__ void precompute_kernel(int ne, int kind, const int4* __restrict__ tets,
                                  const double* __restrict__ X, double D0, double D1, double D2,
                                  double* __restrict__ pre) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int4 t = tets[e];
  V3t<double> p0 = ld3(X, t.x), p1 = ld3(X, t.y), p2 = ld3(X, t.z), p3 = ld3(X, t.w);
  // shape-function gradients scaled by 6V (tetelement.cpp:18-48)
  V3t<double> da = v_sub(p0, p3), db = v_sub(p1, p3), dc = v_sub(p2, p3), ca = v_sub(p0, p2), cb = v_sub(p1, p2);
  V3t<double> g[4];
  if (v_dot(da, v_cross(db, dc)) > 0.0) {
    g[0] = v_cross(db, dc); g[1] = v_cross(dc, da); g[2] = v_cross(da, db); g[3] = v_cross(cb, ca);
  } else {
    g[0] = v_cross(dc, db); g[1] = v_cross(da, dc); g[2] = v_cross(db, da); g[3] = v_cross(ca, cb);
  }
  double vol = tet_vol(p0, p1, p2, p3);
  V3t<double> ab = v_sub(p1, p0), ac = v_sub(p2, p0), ad = v_sub(p3, p0);
  double Dm[9] = {ab.x, ac.x, ad.x, ab.y, ac.y, ad.y, ab.z, ac.z, ad.z}, Di[9];
  double inv = 1.0 / det3(Dm);
  Di[0] = (Dm[4] * Dm[8] - Dm[5] * Dm[7]) * inv;
  Di[1] = (Dm[2] * Dm[7] - Dm[1] * Dm[8]) * inv;
  Di[2] = (Dm[1] * Dm[5] - Dm[2] * Dm[4]) * inv;
  Di[3] = (Dm[5] * Dm[6] - Dm[3] * Dm[8]) * inv;
  Di[4] = (Dm[0] * Dm[8] - Dm[2] * Dm[6]) * inv;
  Di[5] = (Dm[2] * Dm[3] - Dm[0] * Dm[5]) * inv;
  Di[6] = (Dm[3] * Dm[7] - Dm[4] * Dm[6]) * inv;
  Di[7] = (Dm[1] * Dm[6] - Dm[0] * Dm[7]) * inv;
  Di[8] = (Dm[0] * Dm[4] - Dm[1] * Dm[3]) * inv;
  if (kind == OD_MATERIAL_COROTATIONAL || kind == OD_MATERIAL_COROTATIONAL_PLASTIC) {
    const double f = 1.0 / (36.0 * vol);
    int k = 0;
    for (int a = 0; a < 4; a++) {
      const double Ba[3] = {g[a].x, g[a].y, g[a].z};
      for (int b = a; b < 4; b++) {
        const double Bb[3] = {g[b].x, g[b].y, g[b].z};
        pre[(size_t)(k + 0) * ne + e] = (D0 * Ba[0] * Bb[0] + D2 * (Ba[1] * Bb[1] + Ba[2] * Bb[2])) * f;
        pre[(size_t)(k + 1) * ne + e] = (D1 * Ba[0] * Bb[1] + D2 * Ba[1] * Bb[0]) * f;
        pre[(size_t)(k + 2) * ne + e] = (D1 * Ba[0] * Bb[2] + D2 * Ba[2] * Bb[0]) * f;
        pre[(size_t)(k + 3) * ne + e] = (D1 * Ba[1] * Bb[0] + D2 * Ba[0] * Bb[1]) * f;
        pre[(size_t)(k + 4) * ne + e] = (D0 * Ba[1] * Bb[1] + D2 * (Ba[0] * Bb[0] + Ba[2] * Bb[2])) * f;
        pre[(size_t)(k + 5) * ne + e] = (D1 * Ba[1] * Bb[2] + D2 * Ba[2] * Bb[1]) * f;
        pre[(size_t)(k + 6) * ne + e] = (D1 * Ba[2] * Bb[0] + D2 * Ba[0] * Bb[2]) * f;
        pre[(size_t)(k + 7) * ne + e] = (D1 * Ba[2] * Bb[1] + D2 * Ba[1] * Bb[2]) * f;
        pre[(size_t)(k + 8) * ne + e] = (D0 * Ba[2] * Bb[2] + D2 * (Ba[0] * Bb[0] + Ba[1] * Bb[1])) * f;
        k += 9;
      }
    }
    for (int i = 0; i < 9; i++) pre[(size_t)(90 + i) * ne + e] = Di[i];
    pre[(size_t)99 * ne + e] = vol;
    if (kind == OD_MATERIAL_COROTATIONAL_PLASTIC)  // shape derivatives for the stress forces
      for (int a = 0; a < 4; a++) {
        pre[(size_t)(100 + 3 * a) * ne + e] = g[a].x;
        pre[(size_t)(101 + 3 * a) * ne + e] = g[a].y;
        pre[(size_t)(102 + 3 * a) * ne + e] = g[a].z;
      }
  } else {
    for (int a = 0; a < 4; a++) {
      pre[(size_t)(3 * a) * ne + e] = g[a].x;
      pre[(size_t)(3 * a + 1) * ne + e] = g[a].y;
      pre[(size_t)(3 * a + 2) * ne + e] = g[a].z;
    }
    for (int i = 0; i < 9; i++) pre[(size_t)(12 + i) * ne + e] = Di[i];
    pre[(size_t)21 * ne + e] = vol;
  }
}

// ------------------------------------------------------------ mass / loads
__device__ __forceinline__ int local12(int a, int b) { return a * 12 - ((a - 1) * a) / 2 + b - a; }

// consistent mass, rho V / 10 on the diagonal and rho V / 20 off it, same
// axis only (tetelement.cpp:51-66, mechMaterial.cpp:69-98); one colour
__global__ void mass_kernel(int e0, int e1, int ne, int vslot, double rho, const double* __restrict__ pre,
                            const int* __restrict__ emap, double* __restrict__ M) {
  int e = e0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e1) return;
  double vol = pre[(size_t)vslot * ne + e];
  double od = vol * 0.05, dg = vol * 0.1;
  for (int a = 0; a < 4; a++)
    for (int b = a; b < 4; b++) {
      double entry = rho * (a == b ? dg : od);
      for (int ax = 0; ax < 3; ax++) {
        int idx = emap[(size_t)local12(3 * a + ax, 3 * b + ax) * ne + e];
        if (idx >= 0) M[idx] += entry;
      }
    }
}

// V/4 per incident element, summed per node (body-force weights); one colour
__global__ void node_vol_kernel(int e0, int e1, int ne, int vslot, const int4* __restrict__ tets,
                                const double* __restrict__ pre, double* __restrict__ nv) {
  int e = e0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e1) return;
  int4 t = tets[e];
  double q = pre[(size_t)vslot * ne + e] / 4.0;
  nv[t.x] += q; nv[t.y] += q; nv[t.z] += q; nv[t.w] += q;
}

// external forces in one launch: per padded DOF its body force (nodal
// volume x force density, TetElement::getBodyVirtualWorks,
// tetelement.cpp:68-77), then its uniform traction entries over deformed
// facets, area / 3 per vertex (TetFacet::getSurfVirtualWorks,
// tetelement.cpp:79-89), added in the order the loads were given -- the
// order in which Forcer accumulates them (forcer.cpp:8-96)
__global__ void loads_kernel(int n, int dofs, const int* __restrict__ free_pos, const double* __restrict__ nv,
                             double bx, double by, double bz, const int* __restrict__ lptr,
                             const int* __restrict__ lsrc, const int* __restrict__ fids,
                             const double* __restrict__ tvec, double scale, const int* __restrict__ facets,
                             const double* __restrict__ X, const double* __restrict__ u,
                             double* __restrict__ fext) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0.0;
  if (i < dofs) {
    const int p = free_pos[i];
    const int ax = p % 3;
    acc = nv[p / 3] * (ax == 0 ? bx : (ax == 1 ? by : bz));
    if (lptr) {
      for (int j = lptr[i]; j < lptr[i + 1]; j++) {
        const int k = lsrc[j];
        const int f = fids[k];
        const int nd[3] = {facets[3 * f], facets[3 * f + 1], facets[3 * f + 2]};
        V3t<double> q[3];
        for (int v = 0; v < 3; v++)
          q[v] = {X[3 * nd[v]] + u[3 * nd[v]], X[3 * nd[v] + 1] + u[3 * nd[v] + 1], X[3 * nd[v] + 2] + u[3 * nd[v] + 2]};
        const V3t<double> cr = v_cross(v_sub(q[1], q[0]), v_sub(q[2], q[0]));
        const double fac = (sqrt(v_len2(cr)) * 0.5) / 3.0;
        const double w = fac * (scale * tvec[3 * k + ax]);
        if (w != 0.0) acc += w;
      }
    }
  }
  fext[i] = acc;
}

// ------------------------------------------------- double-float arithmetic
// A value as hi + lo of two floats (about 46 significant bits), for the
// mixed-precision path's element stiffness contraction: on this part the
// FP64 units run at 1/70 of the FP32 rate and also execute every FP32 <->
// FP64 conversion, so operands are split and results rebuilt with integer
// bit operations, and the products and sums run on the FP32 units
// (error-free TwoProduct by FMA and TwoSum, Dekker / Knuth).
struct DFv {
  float hi, lo;
};

// x = hi + lo + d with |d| <= 2^-47 |x|: hi is x with its significand cut to
// 24 bits, lo the next 24 bits of the remainder.  Magnitudes below the
// normal float range give 0; infinities and NaNs pass through hi.
__device__ __forceinline__ DFv df_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  const int ef = e - 1023 + 127;
  DFv r{0.f, 0.f};
  if (ef >= 255) {
    r.hi = __uint_as_float(sign | (e == 2047 && m ? 0x7FC00000u : 0x7F800000u));
    return r;
  }
  if (ef <= 0) return r;
  r.hi = __uint_as_float(sign | ((unsigned)ef << 23) | (unsigned)(m >> 29));
  const unsigned rem = (unsigned)(m & 0x1FFFFFFFull);   // the remainder, in units of 2^(e-1075)
  if (rem == 0) return r;
  const int top = 31 - __clz((int)rem);                  // its leading bit, 0..28
  const unsigned frac = (top >= 23 ? (rem >> (top - 23)) : (rem << (23 - top))) & 0x7FFFFFu;
  const int elo = e - 1075 + top + 127;
  if (elo > 0) r.lo = __uint_as_float(sign | ((unsigned)elo << 23) | frac);
  return r;
}

// exact float -> double by bit operations (zero and subnormal floats give 0)
__device__ __forceinline__ double df_widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned ef = (u >> 23) & 0xFFu;
  if (ef == 0) return __longlong_as_double((long long)sign);
  const unsigned long long e = ef == 255 ? 0x7FFull : (unsigned long long)(ef - 127 + 1023);
  return __longlong_as_double((long long)(sign | (e << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

__device__ __forceinline__ double df_value(DFv a) { return df_widen(a.hi) + df_widen(a.lo); }

__device__ __forceinline__ DFv df_mul(DFv a, DFv b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);   // a.hi b.hi = p + e exactly
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float s = p + e;
  return DFv{s, e - (s - p)};
}

__device__ __forceinline__ DFv df_add(DFv a, DFv b) {
  const float s = a.hi + b.hi;
  const float v = s - a.hi;
  const float t = (a.hi - (s - v)) + (b.hi - v);   // a.hi + b.hi = s + t exactly
  const float lo = (t + a.lo) + b.lo;
  const float r = s + lo;
  return DFv{r, lo - (r - s)};
}

// -------------------------------------------------- corotational element
// F = [x1-x0, x2-x0, x3-x0] Dm^-1; R = polar(F), or the proper QR factor when
// the deformed volume is below threshold * rest volume
// (tetelement.cpp:546-573); K_ab = R K0_ab R^T packed into 78 values and
// f_a = sum_b (R K0_ab R^T x_b - R K0_ab X_b) (tetelement.cpp:583-651).
// MODE 0 scatters into K / fint through the element map (one colour per
// launch); MODE 1 stores per-element values in original element order;
// MODE 2 stores them in the colour-ordered staging arrays (all elements in
// one launch, scattered afterwards colour by colour).
template <int MODE, bool DF = false>
__device__ __forceinline__ void corot_elem(int e, int ne, const int4* __restrict__ tets,
                                           const double* __restrict__ X, const double* __restrict__ u,
                                           const double* __restrict__ pre, double thr,
                                           const int* __restrict__ emap, const int* __restrict__ gdof,
                                           double* __restrict__ K, double* __restrict__ fint,
                                           double* __restrict__ out78, double* __restrict__ out12,
                                           const int* __restrict__ perm) {
  int4 t = tets[e];
  const int nd[4] = {t.x, t.y, t.z, t.w};
  V3t<double> o[4], c[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    o[i] = ld3(X, nd[i]);
    V3t<double> du = ld3(u, nd[i]);
    c[i] = {o[i].x + du.x, o[i].y + du.y, o[i].z + du.z};
  }
  double Di[9], F[9];
#pragma unroll
  for (int i = 0; i < 9; i++) { Di[i] = pre[(size_t)(90 + i) * ne + e]; F[i] = 0.0; }
#pragma unroll
  for (int i = 1; i < 4; i++) {
    double ax[3] = {c[i].x - c[0].x, c[i].y - c[0].y, c[i].z - c[0].z};
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) F[j * 3 + k] += ax[j] * Di[(i - 1) * 3 + k];
  }
  const double v0 = pre[(size_t)99 * ne + e];
  const double v1 = tet_vol(c[0], c[1], c[2], c[3]);
  double R[9];
  if (v1 >= thr * v0) polar3<double>(F, R);
  else qr3<double>(F, R);

  double f[12];
#pragma unroll
  for (int i = 0; i < 12; i++) f[i] = 0.0;
  const size_t obase = MODE == 1 ? (size_t)perm[e] * 78 : 0;
  auto put = [&](int k, double val) {
    if (MODE == 0) {
      int idx = emap[(size_t)k * ne + e];
      if (idx >= 0) K[idx] += val;
    } else if (MODE == 1) {
      out78[obase + k] = val;
    } else {
      out78[kst(k, e)] = val;
    }
  };
  if constexpr (DF) {
    // The mixed-precision path: forces f_a = R sum_b K0_ab (R^T c_b - o_b) in
    // FP64 (the same sum regrouped, the cancellation of R^T c_b against o_b
    // taken first) and the stiffness R K0_ab R^T in double-float.
    double y[4][3], g[4][3];
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const double cb[3] = {c[b].x, c[b].y, c[b].z}, ob[3] = {o[b].x, o[b].y, o[b].z};
#pragma unroll
      for (int i = 0; i < 3; i++) {
        y[b][i] = (R[i] * cb[0] + R[3 + i] * cb[1] + R[6 + i] * cb[2]) - ob[i];
        g[b][i] = 0.0;
      }
    }
    DFv dR[9];
#pragma unroll
    for (int i = 0; i < 9; i++) dR[i] = df_split(R[i]);
    int blk = 0;
#pragma unroll 1
    for (int a = 0; a < 4; a++) {
#pragma unroll 1
      for (int b = a; b < 4; b++) {
        double K0[9];
#pragma unroll
        for (int i = 0; i < 9; i++) K0[i] = pre[(size_t)(9 * blk + i) * ne + e];
        blk++;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          g[a][i] += K0[i * 3] * y[b][0] + K0[i * 3 + 1] * y[b][1] + K0[i * 3 + 2] * y[b][2];
          if (b != a) g[b][i] += K0[i] * y[a][0] + K0[3 + i] * y[a][1] + K0[6 + i] * y[a][2];
        }
        DFv dQK[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++)
            dQK[i * 3 + j] = df_add(df_add(df_mul(dR[i * 3], df_split(K0[j])), df_mul(dR[i * 3 + 1], df_split(K0[3 + j]))),
                                    df_mul(dR[i * 3 + 2], df_split(K0[6 + j])));
        auto qkqt = [&](int i, int j) {
          return df_value(df_add(df_add(df_mul(dQK[i * 3], dR[j * 3]), df_mul(dQK[i * 3 + 1], dR[j * 3 + 1])),
                                 df_mul(dQK[i * 3 + 2], dR[j * 3 + 2])));
        };
        if (a == b) {
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3 - i; j++) put(c_diag12[a * 3 + i] + j, qkqt(i, i + j));
        } else {
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) put(c_diag12[a * 3 + i] + (b - a) * 3 - i + j, qkqt(i, j));
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int i = 0; i < 3; i++) f[a * 3 + i] = R[i * 3] * g[a][0] + R[i * 3 + 1] * g[a][1] + R[i * 3 + 2] * g[a][2];
  } else {
  int blk = 0;
#pragma unroll 1
  for (int a = 0; a < 4; a++) {
    double K0[9], QK[9], QKQT[9];
#pragma unroll
    for (int i = 0; i < 9; i++) K0[i] = pre[(size_t)(9 * blk + i) * ne + e];
    blk++;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) QK[i * 3 + j] = R[i * 3] * K0[j] + R[i * 3 + 1] * K0[3 + j] + R[i * 3 + 2] * K0[6 + j];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) QKQT[i * 3 + j] = QK[i * 3] * R[j * 3] + QK[i * 3 + 1] * R[j * 3 + 1] + QK[i * 3 + 2] * R[j * 3 + 2];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3 - i; j++) put(c_diag12[a * 3 + i] + j, QKQT[i * 3 + i + j]);
    const double ca[3] = {c[a].x, c[a].y, c[a].z}, oa[3] = {o[a].x, o[a].y, o[a].z};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) f[a * 3 + i] += QKQT[i * 3 + j] * ca[j] - QK[i * 3 + j] * oa[j];
#pragma unroll 1
    for (int b = a + 1; b < 4; b++) {
      double QKT[9];
#pragma unroll
      for (int i = 0; i < 9; i++) K0[i] = pre[(size_t)(9 * blk + i) * ne + e];
      blk++;
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
          QK[i * 3 + j] = R[i * 3] * K0[j] + R[i * 3 + 1] * K0[3 + j] + R[i * 3 + 2] * K0[6 + j];
          QKT[i * 3 + j] = R[i * 3] * K0[j * 3] + R[i * 3 + 1] * K0[j * 3 + 1] + R[i * 3 + 2] * K0[j * 3 + 2];
        }
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) QKQT[i * 3 + j] = QK[i * 3] * R[j * 3] + QK[i * 3 + 1] * R[j * 3 + 1] + QK[i * 3 + 2] * R[j * 3 + 2];
      const double cb[3] = {c[b].x, c[b].y, c[b].z}, ob[3] = {o[b].x, o[b].y, o[b].z};
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
          put(c_diag12[a * 3 + i] + (b - a) * 3 - i + j, QKQT[i * 3 + j]);
          f[a * 3 + i] += QKQT[i * 3 + j] * cb[j] - QK[i * 3 + j] * ob[j];
          f[b * 3 + i] += QKQT[j * 3 + i] * ca[j] - QKT[i * 3 + j] * oa[j];
        }
    }
  }
  }
  if (MODE == 0) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      int g = gdof[(size_t)k * ne + e];
      if (g >= 0) fint[g] += f[k];
    }
  } else if (MODE == 1) {
#pragma unroll
    for (int k = 0; k < 12; k++) out12[(size_t)perm[e] * 12 + k] = f[k];
  } else {
#pragma unroll
    for (int k = 0; k < 12; k++) out12[fst(k, e)] = f[k];
  }
}

// ------------------------------------------- invertible hyperelastic element
// Invertible SVD of F, energy derivatives in the invariants I1 = sum s^2,
// I2 = sum s^4, I3 = prod s^2 (invertibleHyperelastic.h:22-30): Neo-Hookean
// (invertibleNeoHookean.cpp:11-20) or StVK (invertibleStVK.cpp:11-20);
// P = U diag(2 g1 s + 4 g2 s^3 + 2 g3 I3 / s) V^T (invertibleHyperelastic.cpp:
// 247-265); dP/dF in the singular-value frame projected to PSD
// (tetelement.cpp:357-499) -- only its 21 structural non-zeros are formed;
// K_ab = U [sum_kl dP_ikjl (V^T dN_a)_k (V^T dN_b)_l] U^T / (36 V)
// (tetelement.cpp:282-342); f_a = P dN_a / 6, f_3 = -(f_0 + f_1 + f_2)
// (tetelement.cpp:344-355).
template <int MODE, bool DF = false>
__device__ __forceinline__ void invhyper_elem(int e, int ne, int stvk, const int4* __restrict__ tets,
                                              const double* __restrict__ X, const double* __restrict__ u,
                                              const double* __restrict__ pre, double thr, double lambda, double mu,
                                              const int* __restrict__ emap, const int* __restrict__ gdof,
                                              double* __restrict__ K, double* __restrict__ fint,
                                              double* __restrict__ out78, double* __restrict__ out12,
                                              const int* __restrict__ perm) {
  int4 t = tets[e];
  const int nd[4] = {t.x, t.y, t.z, t.w};
  V3t<double> c[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    V3t<double> x = ld3(X, nd[i]), du = ld3(u, nd[i]);
    c[i] = {x.x + du.x, x.y + du.y, x.z + du.z};
  }
  double F[9];
#pragma unroll
  for (int i = 0; i < 9; i++) F[i] = 0.0;
#pragma unroll
  for (int i = 1; i < 4; i++) {
    double ax[3] = {c[i].x - c[0].x, c[i].y - c[0].y, c[i].z - c[0].z};
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) F[j * 3 + k] += ax[j] * pre[(size_t)(12 + (i - 1) * 3 + k) * ne + e];
  }
  double sig[3], U[9], VT[9];
  invertible_svd<double, DF>(F, thr, sig, U, VT);
  const double s02 = sig[0] * sig[0], s12 = sig[1] * sig[1], s22 = sig[2] * sig[2];
  const double I1 = s02 + s12 + s22, I3 = s02 * s12 * s22;
  double g0, g1, g2, h0 = 0.0, h5 = 0.0;
  if (!stvk) {
    g0 = 0.5 * mu;
    g1 = 0.0;
    if constexpr (DF) {   // one reciprocal of I3 for both
      const double lI3 = log(I3), rI3 = 1.0 / I3;
      g2 = (-0.5 * mu + 0.25 * lambda * lI3) * rI3;
      h5 = (0.5 * mu + 0.25 * lambda * (1.0 - lI3)) * (rI3 * rI3);
    } else {
      g2 = (-0.5 * mu + 0.25 * lambda * log(I3)) / I3;
      h5 = (0.5 * mu + 0.25 * lambda * (1.0 - log(I3))) / (I3 * I3);
    }
  } else {
    g0 = 0.25 * lambda * (I1 - 3.0) - 0.5 * mu;
    g1 = 0.25 * mu;
    g2 = 0.0;
    h0 = 0.25 * lambda;
  }
  // dP/dF non-zeros (tetelement.cpp:357-437)
  const double sc01 = sig[0] * sig[1], sc02 = sig[0] * sig[2], sc12 = sig[1] * sig[2];
  double a01 = 2.0 * g0 + 4.0 * (s02 + s12) * g1;
  double a02 = 2.0 * g0 + 4.0 * (s02 + s22) * g1;
  double a12 = 2.0 * g0 + 4.0 * (s12 + s22) * g1;
  const double a00 = 2.0 * g0 + 8.0 * s02 * g1, a11 = 2.0 * g0 + 8.0 * s12 * g1, a22 = 2.0 * g0 + 8.0 * s22 * g1;
  // d_ij = I3 g2 / (s_i s_j); the mixed path forms them as products
  // (I3 / (s_i s_j) is the product of the other factors: FP64 divisions are
  // long instruction sequences on this part), and so its forces' I3 / s_i;
  // the FP64 path keeps the reference's expressions.
  const double d00 = DF ? g2 * (s12 * s22) : I3 * g2 / s02, d01 = DF ? g2 * (sc01 * s22) : I3 * g2 / sc01,
               d02 = DF ? g2 * (sc02 * s12) : I3 * g2 / sc02;
  const double d11 = DF ? g2 * (s02 * s22) : I3 * g2 / s12, d12 = DF ? g2 * (sc12 * s02) : I3 * g2 / sc12,
               d22 = DF ? g2 * (s02 * s12) : I3 * g2 / s22;
  const double b00 = 4.0 * s02 * g1 - 2.0 * d00, b11 = 4.0 * s12 * g1 - 2.0 * d11, b22 = 4.0 * s22 * g1 - 2.0 * d22;
  double b01 = 4.0 * sc01 * g1 - 2.0 * d01, b02 = 4.0 * sc02 * g1 - 2.0 * d02, b12 = 4.0 * sc12 * g1 - 2.0 * d12;
  // Hessian in the invariants is diag-like: only H00 (StVK) or H22 (NH) set
  double w[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    w[i][0] = 2.0 * sig[i];
    w[i][1] = 4.0 * sig[i] * (i == 0 ? s02 : (i == 1 ? s12 : s22));
    w[i][2] = DF ? 2.0 * sig[i] * (i == 0 ? s12 * s22 : (i == 1 ? s02 * s22 : s02 * s12)) : 2.0 * I3 / sig[i];
  }
  // w_i . (H w_j) with H = diag(h0, 0, h5) in the invariants (the only
  // non-zero Hessian entries of both energies)
  auto qf = [&](int i, int j) { return w[i][0] * (h0 * w[j][0]) + w[i][2] * (h5 * w[j][2]); };
  double T[6] = {a00 + b00 + (qf(0, 0) + 4.0 * d00), qf(1, 0) + 4.0 * d01, qf(2, 0) + 4.0 * d02,
                 a11 + b11 + (qf(1, 1) + 4.0 * d11), qf(2, 1) + 4.0 * d12, a22 + b22 + (qf(2, 2) + 4.0 * d22)};
  psd3<double>(T);
  psd2<double>(a01, b01);
  psd2<double>(a02, b02);
  psd2<double>(a12, b12);
  const double Tm[3][3] = {{T[0], T[1], T[2]}, {T[1], T[3], T[4]}, {T[2], T[4], T[5]}};
  const double Al[3][3] = {{0.0, a01, a02}, {a01, 0.0, a12}, {a02, a12, 0.0}};
  const double Be[3][3] = {{0.0, b01, b02}, {b01, 0.0, b12}, {b02, b12, 0.0}};

  // P = U diag(de) V^T
  double de[3], P[9];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    if constexpr (DF) {   // I3 / s_i as the product s_i s_j^2 s_k^2
      const double i3s = sig[i] * (i == 0 ? s12 * s22 : (i == 1 ? s02 * s22 : s02 * s12));
      de[i] = 2.0 * g0 * sig[i] + 4.0 * g1 * sig[i] * sig[i] * sig[i] + 2.0 * g2 * i3s;
    } else {
      de[i] = 2.0 * g0 * sig[i] + 4.0 * g1 * sig[i] * sig[i] * sig[i] + 2.0 * g2 * I3 / sig[i];
    }
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      P[i * 3 + j] = U[i * 3] * (VT[j] * de[0]) + U[i * 3 + 1] * (VT[3 + j] * de[1]) + U[i * 3 + 2] * (VT[6 + j] * de[2]);

  // a_n = V^T dN_n
  double an[4][3];
#pragma unroll
  for (int nn = 0; nn < 4; nn++) {
    double d0 = pre[(size_t)(3 * nn) * ne + e], d1 = pre[(size_t)(3 * nn + 1) * ne + e], d2 = pre[(size_t)(3 * nn + 2) * ne + e];
#pragma unroll
    for (int i = 0; i < 3; i++) an[nn][i] = VT[3 * i] * d0 + VT[3 * i + 1] * d1 + VT[3 * i + 2] * d2;
  }
  const double fac = 1.0 / (36.0 * pre[(size_t)21 * ne + e]);
  const size_t obase = MODE == 1 ? (size_t)perm[e] * 78 : 0;
  auto put = [&](int k, double val) {
    if (MODE == 0) {
      int idx = emap[(size_t)k * ne + e];
      if (idx >= 0) K[idx] += val;
    } else if (MODE == 1) {
      out78[obase + k] = val;
    } else {
      out78[kst(k, e)] = val;
    }
  };
  if constexpr (DF) {
    // the contraction U [sum_kl dP_ikjl an_a,k an_b,l] U^T / (36 V) in
    // double-float, the same terms in the same order as below
    // Tm symmetric (6 values), Al and Be symmetric with zero diagonals (3 each)
    DFv dan[4][3], dU[9], dT6[6], dA3[3], dB3[3];
#pragma unroll
    for (int nn = 0; nn < 4; nn++)
#pragma unroll
      for (int i = 0; i < 3; i++) dan[nn][i] = df_split(an[nn][i]);
#pragma unroll
    for (int i = 0; i < 9; i++) dU[i] = df_split(U[i]);
#pragma unroll
    for (int i = 0; i < 6; i++) dT6[i] = df_split(T[i]);
    dA3[0] = df_split(a01); dA3[1] = df_split(a02); dA3[2] = df_split(a12);
    dB3[0] = df_split(b01); dB3[1] = df_split(b02); dB3[2] = df_split(b12);
    auto sym6 = [](int i, int j) { return i <= j ? i * 3 - (i * (i - 1)) / 2 + (j - i) : j * 3 - (j * (j - 1)) / 2 + (i - j); };
    auto off3 = [](int i, int j) { return i + j - 1; };   // (0,1) -> 0, (0,2) -> 1, (1,2) -> 2
    const DFv dfac = df_split(fac);
#pragma unroll 1
    for (int a = 0; a < 4; a++) {
#pragma unroll 1
      for (int b = a; b < 4; b++) {
        DFv sm[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) {
            DFv en{0.f, 0.f};
            if (i == j) {
#pragma unroll
              for (int k = 0; k < 3; k++)
                en = df_add(en, df_mul(df_mul(k == i ? dT6[sym6(i, i)] : dA3[off3(i, k)], dan[a][k]), dan[b][k]));
            } else if (i < j) {
              en = df_add(en, df_mul(df_mul(dT6[sym6(i, j)], dan[a][i]), dan[b][j]));
              en = df_add(en, df_mul(df_mul(dB3[off3(i, j)], dan[a][j]), dan[b][i]));
            } else {
              en = df_add(en, df_mul(df_mul(dB3[off3(i, j)], dan[a][j]), dan[b][i]));
              en = df_add(en, df_mul(df_mul(dT6[sym6(i, j)], dan[a][i]), dan[b][j]));
            }
            sm[i * 3 + j] = en;
          }
        DFv tmp[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++)
            tmp[i * 3 + j] = df_add(df_add(df_mul(dU[i * 3], sm[j]), df_mul(dU[i * 3 + 1], sm[3 + j])),
                                    df_mul(dU[i * 3 + 2], sm[6 + j]));
        auto outv = [&](int i, int j) {
          const DFv o = df_add(df_add(df_mul(tmp[i * 3], dU[j * 3]), df_mul(tmp[i * 3 + 1], dU[j * 3 + 1])),
                               df_mul(tmp[i * 3 + 2], dU[j * 3 + 2]));
          return df_value(df_mul(o, dfac));
        };
        if (a == b) {
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3 - i; j++) put(c_diag12[a * 3 + i] + j, outv(i, i + j));
        } else {
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) put(c_diag12[a * 3 + i] + (b - a) * 3 - i + j, outv(i, j));
        }
      }
    }
  } else {
#pragma unroll 1
  for (int a = 0; a < 4; a++) {
#pragma unroll 1
    for (int b = a; b < 4; b++) {
      double sm[9];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
          double en = 0.0;
          if (i == j) {
#pragma unroll
            for (int k = 0; k < 3; k++) en += (k == i ? Tm[i][i] : Al[i][k]) * an[a][k] * an[b][k];
          } else if (i < j) {
            en += Tm[i][j] * an[a][i] * an[b][j];
            en += Be[i][j] * an[a][j] * an[b][i];
          } else {
            en += Be[i][j] * an[a][j] * an[b][i];
            en += Tm[i][j] * an[a][i] * an[b][j];
          }
          sm[i * 3 + j] = en;
        }
      double tmp[9], out[9];
      mul3(U, sm, tmp);
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) out[i * 3 + j] = tmp[i * 3] * U[j * 3] + tmp[i * 3 + 1] * U[j * 3 + 1] + tmp[i * 3 + 2] * U[j * 3 + 2];
      if (a == b) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3 - i; j++) put(c_diag12[a * 3 + i] + j, out[i * 3 + i + j] * fac);
      } else {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) put(c_diag12[a * 3 + i] + (b - a) * 3 - i + j, out[i * 3 + j] * fac);
      }
    }
  }
  }
  double f[12];
  const double sixth = 1.0 / 6.0;
#pragma unroll
  for (int nn = 0; nn < 3; nn++) {
    double d0 = pre[(size_t)(3 * nn) * ne + e], d1 = pre[(size_t)(3 * nn + 1) * ne + e], d2 = pre[(size_t)(3 * nn + 2) * ne + e];
#pragma unroll
    for (int i = 0; i < 3; i++) f[3 * nn + i] = (P[3 * i] * d0 + P[3 * i + 1] * d1 + P[3 * i + 2] * d2) * sixth;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) f[9 + i] = -(f[i] + f[3 + i] + f[6 + i]);
  if (MODE == 0) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      int g = gdof[(size_t)k * ne + e];
      if (g >= 0) fint[g] += f[k];
    }
  } else if (MODE == 1) {
#pragma unroll
    for (int k = 0; k < 12; k++) out12[(size_t)perm[e] * 12 + k] = f[k];
  } else {
#pragma unroll
    for (int k = 0; k < 12; k++) out12[fst(k, e)] = f[k];
  }
}

template <int MODE, bool DF = false>
__global__ void __launch_bounds__(128) corot_kernel(int e0, int e1, int ne, const int4* __restrict__ tets,
                                                    const double* __restrict__ X, const double* __restrict__ u,
                                                    const double* __restrict__ pre, double thr,
                                                    const int* __restrict__ emap, const int* __restrict__ gdof,
                                                    double* __restrict__ K, double* __restrict__ fint,
                                                    double* __restrict__ out78, double* __restrict__ out12,
                                                    const int* __restrict__ perm) {
  const int e = e0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (e < e1) corot_elem<MODE, DF>(e, ne, tets, X, u, pre, thr, emap, gdof, K, fint, out78, out12, perm);
}

template <int MODE, bool DF = false>
__global__ void __launch_bounds__(128) invhyper_kernel(int e0, int e1, int ne, int stvk, const int4* __restrict__ tets,
                                                       const double* __restrict__ X, const double* __restrict__ u,
                                                       const double* __restrict__ pre, double thr, double lambda,
                                                       double mu, const int* __restrict__ emap,
                                                       const int* __restrict__ gdof, double* __restrict__ K,
                                                       double* __restrict__ fint, double* __restrict__ out78,
                                                       double* __restrict__ out12, const int* __restrict__ perm) {
  const int e = e0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (e < e1)
    invhyper_elem<MODE, DF>(e, ne, stvk, tets, X, u, pre, thr, lambda, mu, emap, gdof, K, fint, out78, out12, perm);
}

// ---- several scenes per launch: tile j of scene s (directory prefix) is
// its elements [128 j, 128 j + 128); every scene's values land in its own
// staging arrays
__global__ void __launch_bounds__(128) corot_batch_kernel(int n_sc, const int* __restrict__ prefix,
                                                          const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  const int e = (blockIdx.x - prefix[s]) * 128 + threadIdx.x;
  if (e >= D.n_tets) return;
  // batched scenes all run the mixed-precision solver: double-float stiffness
  corot_elem<2, true>(e, D.n_tets, D.tets, D.X, D.u, D.pre, D.thr, D.emap, D.gdof, nullptr, nullptr, D.stage_k,
                      D.stage_f, nullptr);
}

__global__ void __launch_bounds__(128) invhyper_batch_kernel(int n_sc, const int* __restrict__ prefix,
                                                             const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  const int e = (blockIdx.x - prefix[s]) * 128 + threadIdx.x;
  if (e >= D.n_tets) return;
  // batched scenes all run the mixed-precision solver: double-float contraction
  invhyper_elem<2, true>(e, D.n_tets, D.kind == OD_MATERIAL_STVK, D.tets, D.X, D.u, D.pre, D.thr, D.lambda, D.mu,
                         D.emap, D.gdof, nullptr, nullptr, D.stage_k, D.stage_f, nullptr);
}

// Corotational plastic element (corotationalPlastic.cpp:53-183,
// tetelement.cpp:654-729).  F = R S: polar decomposition (S = R^T F), or QR
// when the deformed volume falls below threshold x rest volume (S = Q^T F,
// the upper factor).  Elastic strain e = sym(S) - I - plastic strain; stress
// 2 mu e + lambda tr(e) I, rotated by R; forces f_a = (R stress) dN_a / 6
// (a < 3), f_3 = -(f_0 + f_1 + f_2); stiffness R K0_ab R^T.  Every
// evaluation updates the element's plastic strain (in place, as the
// reference does): when the strain norm exceeds the yield criterion it grows
// by creep (|e| - yield)/|e| e and is scaled back to the maximum.  Both
// norms follow the reference, which adds the squares of the first three
// entries three times (corotationalPlastic.cpp:156-160, 169-173).
// pre: [90 K0][9 Dm^-1][V][12 dN] per element (SoA); plastic: [9][ne].
template <int MODE>
__device__ __forceinline__ void plastic_elem(int e, int ne, const int4* __restrict__ tets,
                                             const double* __restrict__ X, const double* __restrict__ u,
                                             const double* __restrict__ pre, double thr, double lambda, double mu,
                                             double yield, double creep, double max_plastic,
                                             double* __restrict__ plastic, double* __restrict__ out78,
                                             double* __restrict__ out12, const int* __restrict__ perm) {
  int4 t = tets[e];
  const int nd[4] = {t.x, t.y, t.z, t.w};
  V3t<double> c[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    V3t<double> x = ld3(X, nd[i]), du = ld3(u, nd[i]);
    c[i] = {x.x + du.x, x.y + du.y, x.z + du.z};
  }
  double F[9];
#pragma unroll
  for (int i = 0; i < 9; i++) F[i] = 0.0;
#pragma unroll
  for (int i = 1; i < 4; i++) {
    double ax[3] = {c[i].x - c[0].x, c[i].y - c[0].y, c[i].z - c[0].z};
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) F[j * 3 + k] += ax[j] * pre[(size_t)(90 + (i - 1) * 3 + k) * ne + e];
  }
  const double v0 = pre[(size_t)99 * ne + e];
  const double v1 = tet_vol(c[0], c[1], c[2], c[3]);
  double R[9], S[9];
  if (v1 >= thr * v0) polar3<double>(F, R);
  else qr3<double>(F, R);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) S[i * 3 + j] = R[i] * F[j] + R[3 + i] * F[3 + j] + R[6 + i] * F[6 + j];
  // elastic strain, stress, plastic update (computeElasticStress)
  double ep[9], es[9];
#pragma unroll
  for (int i = 0; i < 9; i++) ep[i] = plastic[(size_t)i * ne + e];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) es[i * 3 + j] = 0.5 * (S[i * 3 + j] + S[j * 3 + i]) - ep[i * 3 + j];
  es[0] -= 1.0;
  es[4] -= 1.0;
  es[8] -= 1.0;
  const double mu2 = 2.0 * mu;
  double st[9];
#pragma unroll
  for (int i = 0; i < 9; i++) st[i] = mu2 * es[i];
  const double dg = lambda * (es[0] + es[4] + es[8]);
  st[0] += dg;
  st[4] += dg;
  st[8] += dg;
  double P[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) P[i * 3 + j] = R[i * 3] * st[j] + R[i * 3 + 1] * st[3 + j] + R[i * 3 + 2] * st[6 + j];
  double en = 0.0;  // the reference's sum: each of the first three squares three times, in its order
#pragma unroll
  for (int i = 0; i < 3; i++) {
    en += es[i] * es[i];
    en += es[i] * es[i];
    en += es[i] * es[i];
  }
  en = sqrt(en);
  if (en > yield) {
    const double ratio = creep * (en - yield) / en;
#pragma unroll
    for (int i = 0; i < 9; i++) ep[i] += ratio * es[i];
    double pn = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      pn += ep[i] * ep[i];
      pn += ep[i] * ep[i];
      pn += ep[i] * ep[i];
    }
    pn = sqrt(pn);
    if (pn > max_plastic) {
      const double fac = max_plastic / pn;
#pragma unroll
      for (int i = 0; i < 9; i++) ep[i] *= fac;
    }
#pragma unroll
    for (int i = 0; i < 9; i++) plastic[(size_t)i * ne + e] = ep[i];
  }
  auto put = [&](int k, double val) {
    if (MODE == 1) out78[(size_t)perm[e] * 78 + k] = val;
    else out78[kst(k, e)] = val;
  };
  int blk = 0;
#pragma unroll 1
  for (int a = 0; a < 4; a++) {
#pragma unroll 1
    for (int b = a; b < 4; b++) {
      double K0[9], QK[9], QKQT[9];
#pragma unroll
      for (int i = 0; i < 9; i++) K0[i] = pre[(size_t)(9 * blk + i) * ne + e];
      blk++;
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) QK[i * 3 + j] = R[i * 3] * K0[j] + R[i * 3 + 1] * K0[3 + j] + R[i * 3 + 2] * K0[6 + j];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
          QKQT[i * 3 + j] = QK[i * 3] * R[j * 3] + QK[i * 3 + 1] * R[j * 3 + 1] + QK[i * 3 + 2] * R[j * 3 + 2];
      if (a == b) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3 - i; j++) put(c_diag12[a * 3 + i] + j, QKQT[i * 3 + i + j]);
      } else {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) put(c_diag12[a * 3 + i] + (b - a) * 3 - i + j, QKQT[i * 3 + j]);
      }
    }
  }
  double f[12];
  const double sixth = 1.0 / 6.0;
#pragma unroll
  for (int n = 0; n < 3; n++) {
    const double x = pre[(size_t)(100 + 3 * n) * ne + e], y = pre[(size_t)(101 + 3 * n) * ne + e],
                 z = pre[(size_t)(102 + 3 * n) * ne + e];
#pragma unroll
    for (int i = 0; i < 3; i++) f[3 * n + i] = (P[i * 3] * x + P[i * 3 + 1] * y + P[i * 3 + 2] * z) * sixth;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) f[9 + i] = -(f[i] + f[3 + i] + f[6 + i]);
  if (MODE == 1) {
#pragma unroll
    for (int k = 0; k < 12; k++) out12[(size_t)perm[e] * 12 + k] = f[k];
  } else {
#pragma unroll
    for (int k = 0; k < 12; k++) out12[fst(k, e)] = f[k];
  }
}

template <int MODE>
__global__ void __launch_bounds__(128) plastic_kernel(int ne, const int4* __restrict__ tets,
                                                      const double* __restrict__ X, const double* __restrict__ u,
                                                      const double* __restrict__ pre, double thr, double lambda,
                                                      double mu, double yield, double creep, double max_plastic,
                                                      double* __restrict__ plastic, double* __restrict__ out78,
                                                      double* __restrict__ out12, const int* __restrict__ perm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < ne)
    plastic_elem<MODE>(e, ne, tets, X, u, pre, thr, lambda, mu, yield, creep, max_plastic, plastic, out78, out12,
                       perm);
}

__global__ void __launch_bounds__(128) plastic_batch_kernel(int n_sc, const int* __restrict__ prefix,
                                                            const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  const int e = (blockIdx.x - prefix[s]) * 128 + threadIdx.x;
  if (e >= D.n_tets) return;
  plastic_elem<2>(e, D.n_tets, D.tets, D.X, D.u, D.pre, D.thr, D.lambda, D.mu, D.yield, D.creep, D.max_plastic,
                  D.plastic, D.stage_k, D.stage_f, nullptr);
}

// atomic-free scatter of staged element values, one colour per launch
// (corotationalHyperelastic.cpp:100-120): no two elements of a colour share
// a matrix value or a force entry.  One thread per (element, entry): entries
// 0..77 are stiffness values, 78..89 forces; for a fixed entry consecutive
// threads read consecutive staged values and map entries.
__global__ void scatter_kernel(int e0, int cnt, int ne, const double* __restrict__ k78, const double* __restrict__ f12,
                               const int* __restrict__ emap, const int* __restrict__ gdof, double* __restrict__ K,
                               double* __restrict__ fint) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 90LL * cnt) return;
  const int k = (int)(t / cnt);
  const int e = e0 + (int)(t - (long long)k * cnt);
  if (k < 78) {
    const int idx = emap[(size_t)k * ne + e];
    if (idx >= 0) K[idx] += k78[kst(k, e)];
  } else {
    const int g = gdof[(size_t)(k - 78) * ne + e];
    if (g >= 0) fint[g] += f12[fst(k - 78, e)];
  }
}

// gathered assembly: value i of K (and entry i of the forces) is the sum of
// its element contributions in the reference's assembly order (element
// index, then the element's entry index; the loops of
// material/corotationalHyperelastic.cpp:67-97), started from zero, so the
// additions happen in the reference's sequence.  One thread per destination,
// no atomics, no colour passes.
__device__ __forceinline__ void gather_one(long long i, int nk, const int* __restrict__ kptr,
                                           const int* __restrict__ ksrc, const double* __restrict__ k78,
                                           double* __restrict__ K, int nf, const int* __restrict__ fptr,
                                           const int* __restrict__ fsrc, const double* __restrict__ f12,
                                           double* __restrict__ fint, int accumulate) {
  const int* ptr = kptr;
  const int* src = ksrc;
  const double* val = k78;
  double* out = K;
  if (i >= nk) {
    i -= nk;
    if (i >= nf) return;
    ptr = fptr; src = fsrc; val = f12; out = fint;
  }
  const int j1 = ptr[i + 1];
  double acc = accumulate ? out[i] : 0.0;
  for (int j = ptr[i]; j < j1; j++) acc += val[src[j]];
  out[i] = acc;
}

__global__ void __launch_bounds__(256) gather_kernel(int nk, const int* __restrict__ kptr,
                                                     const int* __restrict__ ksrc, const double* __restrict__ k78,
                                                     double* __restrict__ K, int nf, const int* __restrict__ fptr,
                                                     const int* __restrict__ fsrc, const double* __restrict__ f12,
                                                     double* __restrict__ fint, int accumulate) {
  gather_one((long long)blockIdx.x * blockDim.x + threadIdx.x, nk, kptr, ksrc, k78, K, nf, fptr, fsrc, f12, fint,
             accumulate);
}

// multi-scene scatter of colour c: tile j of scene s covers the colour's
// threads [256 j, 256 j + 256) (90 per element: 78 stiffness values, 12
// forces)
__global__ void scatter_batch_kernel(int n_sc, const int* __restrict__ prefix, int c,
                                     const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  const int e0 = D.color_off[c], cnt = D.color_off[c + 1] - e0;
  const int t = (blockIdx.x - prefix[s]) * 256 + threadIdx.x;
  if (t >= 90 * cnt) return;
  const int ne = D.n_tets;
  const int k = t / cnt;
  const int e = e0 + (t - k * cnt);
  if (k < 78) {
    const int idx = D.emap[(size_t)k * ne + e];
    if (idx >= 0) D.K[idx] += D.stage_k[kst(k, e)];
  } else {
    const int g = D.gdof[(size_t)(k - 78) * ne + e];
    if (g >= 0) D.fint[g] += D.stage_f[fst(k - 78, e)];
  }
}

// ---- the gather lists, built on the device once per scene: count the
// contributions of every destination, scan the counts into the list
// offsets, place every source with an atomic cursor, then sort each list
// by (original element index, entry index) -- the reference's assembly
// order, whatever order the atomics placed them in.
constexpr int kScanBlock = 1024;

__global__ void gl_count_kernel(long long n, const int* __restrict__ dest, int* __restrict__ cnt) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int d = dest[t];
    if (d >= 0) atomicAdd(&cnt[d + 1], 1);
  }
}

// inclusive scan of each 1024-entry block in place; the block's total to sums
__global__ void __launch_bounds__(kScanBlock) gl_scan_block_kernel(int n, int* __restrict__ data,
                                                                   int* __restrict__ sums) {
  __shared__ int warp_tot[kScanBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  int v = i < n ? data[i] : 0;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) warp_tot[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int w = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v += warp_tot[warp - 1];
  if (i < n) data[i] = v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kScanBlock) gl_add_kernel(int n, int* __restrict__ data,
                                                            const int* __restrict__ offs) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) data[i] += offs[blockIdx.x];
}

// map entry t = k * ne + e (e the element's staged position) -> its staged
// source: e * kk + slot (c_kslot for the 78 stiffness values, k for forces)
__global__ void gl_fill_kernel(long long n, const int* __restrict__ dest, int* __restrict__ cur,
                               int* __restrict__ src, int ne, int kk) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int d = dest[t];
    if (d >= 0) {
      const int k = (int)(t / ne), e = (int)(t - (long long)k * ne);
      src[atomicAdd(&cur[d], 1)] = e * kk + (kk == 78 ? c_kslot[k] : k);
    }
  }
}

// a list's sources (e * kk + slot) sort by perm[e] * kk + slot: an element
// contributes at most once to a destination, so this is the reference's
// order, by original element index
__global__ void gl_sort_kernel(int nd, const int* __restrict__ ptr, int* __restrict__ src,
                               const int* __restrict__ perm, int ne, int kk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nd) return;
  const int a = ptr[i], b = ptr[i + 1];
  for (int j = a + 1; j < b; j++) {
    const int v = src[j];
    const long long key = (long long)perm[v / kk] * kk + v % kk;
    int q = j - 1;
    while (q >= a) {
      const int w = src[q];
      if ((long long)perm[w / kk] * kk + w % kk <= key) break;
      src[q + 1] = w;
      q--;
    }
    src[q + 1] = v;
  }
}

static od_status gather_list(Scene* s, const int* dest, int kk, int nd, int** ptr_out, int** src_out) {
  const int ne = s->n_tets;
  cudaStream_t st = s->ctx->stream;
  const long long n = (long long)kk * ne;
  const int grid = std::max(1, (int)std::min<long long>((n + 255) / 256, 64LL * std::max(1, s->ctx->num_sms)));
  // every buffer is freed on an early error return; ptr and src are handed
  // over on success
  struct Bufs {
    int *ptr = nullptr, *sums = nullptr, *cur = nullptr, *src = nullptr;
    ~Bufs() {
      for (int* p : {ptr, sums, cur, src}) cudaFree(p);
    }
  } b;
  int*& ptr = b.ptr;
  int*& sums = b.sums;
  int*& cur = b.cur;
  int*& src = b.src;
  const int nscan = nd + 1, nb = (nscan + kScanBlock - 1) / kScanBlock;
  OD_CUDA(cudaMalloc(&ptr, sizeof(int) * (size_t)nscan));
  OD_CUDA(cudaMalloc(&sums, sizeof(int) * (size_t)nb));
  OD_CUDA(cudaMemsetAsync(ptr, 0, sizeof(int) * (size_t)nscan, st));
  gl_count_kernel<<<grid, 256, 0, st>>>(n, dest, ptr);
  gl_scan_block_kernel<<<nb, kScanBlock, 0, st>>>(nscan, ptr, sums);
  std::vector<int> hs(nb);
  OD_CUDA(cudaMemcpyAsync(hs.data(), sums, sizeof(int) * (size_t)nb, cudaMemcpyDeviceToHost, st));
  OD_TRY(sync_stream(s));
  long long run = 0;
  for (int b = 0; b < nb; b++) {
    const long long t = hs[b];
    hs[b] = (int)run;
    run += t;
  }
  const int total = (int)run;
  OD_CUDA(cudaMemcpyAsync(sums, hs.data(), sizeof(int) * (size_t)nb, cudaMemcpyHostToDevice, st));
  gl_add_kernel<<<nb, kScanBlock, 0, st>>>(nscan, ptr, sums);
  OD_CUDA(cudaMalloc(&src, sizeof(int) * (size_t)std::max(1, total)));
  OD_CUDA(cudaMalloc(&cur, sizeof(int) * (size_t)std::max(1, nd)));
  if (nd > 0) OD_CUDA(cudaMemcpyAsync(cur, ptr, sizeof(int) * (size_t)nd, cudaMemcpyDeviceToDevice, st));
  gl_fill_kernel<<<grid, 256, 0, st>>>(n, dest, cur, src, ne, kk);
  if (nd > 0) gl_sort_kernel<<<(nd + 255) / 256, 256, 0, st>>>(nd, ptr, src, s->perm, ne, kk);
  OD_CUDA(cudaGetLastError());
  OD_TRY(sync_stream(s));   // hs is read by the copy above; the temporaries go next
  s->device_bytes += (long long)sizeof(int) * ((long long)nscan + std::max(1, total));
  *ptr_out = ptr;
  *src_out = src;
  ptr = src = nullptr;
  return OD_OK;
}

od_status build_gather_lists(Scene* s, int n_pad) {
  if (s->n_tets <= 0 || 78LL * s->n_tets >= (long long)INT32_MAX) return OD_OK;
  OD_TRY(gather_list(s, s->emap, 78, s->nvals, &s->gat_kptr, &s->gat_ksrc));
  OD_TRY(gather_list(s, s->gdof, 12, n_pad, &s->gat_fptr, &s->gat_fsrc));
  return OD_OK;
}

// multi-scene gathered assembly: tile j of scene s covers its destinations
// [256 j, 256 j + 256) (K values, then the padded f_int entries)
__global__ void __launch_bounds__(256) gather_batch_kernel(int n_sc, const int* __restrict__ prefix,
                                                           const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  gather_one((long long)(blockIdx.x - prefix[s]) * 256 + threadIdx.x, D.nvals, D.gat_kptr, D.gat_ksrc, D.stage_k,
             D.K, D.n_pad, D.gat_fptr, D.gat_fsrc, D.stage_f, D.fint, 0);
}

// zero 4096 K values (which 0) or padded f_int entries (which 1) per tile
__global__ void zero_batch_kernel(int n_sc, const int* __restrict__ prefix, int which,
                                  const SceneDev* __restrict__ sd) {
  const int s = dir_scene(prefix, n_sc, blockIdx.x);
  const SceneDev& D = sd[s];
  double* p = which == 0 ? D.K : D.fint;
  const int n = which == 0 ? D.nvals : D.n_pad;
  const int i0 = (blockIdx.x - prefix[s]) * kZeroTileValues, i1 = min(n, i0 + kZeroTileValues);
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) p[i] = 0.0;
}

// ---------------------------------------------------------------- launches
static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

od_status launch_precompute(Scene* s) {
  const int T = 128;
  if (s->n_tets == 0) return OD_OK;
  OD_KL(s);
  precompute_kernel<<<nblk(s->n_tets, T), T, 0, s->ctx->stream>>>(s->n_tets, s->mat.kind, s->tets, s->X, s->D[0],
                                                                   s->D[1], s->D[2], s->pre);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

// ------------------------------------------------------------ linear (Hooke)
// HookeMaterial::generateStiffnessMatrix (material/hooke.cpp:18-60): per
// element and node pair a <= b the block of LinearIsotropicTetElement::
// generateSubStiffnessMatrix (element/tetelement.cpp:98-116) with the Lame
// coefficients D = (lambda + 2 mu, lambda, mu) (hooke.cpp:6-16), written into
// the colour-ordered staging layout (78 values: the element's 12x12 upper
// triangle by rows) that the assembly sums in element order.
__global__ void hooke_stage_kernel(int ne, const int4* __restrict__ tets, const double* __restrict__ X, double D0,
                                   double D1, double D2, double* __restrict__ k78) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int4 t = tets[e];
  const V3t<double> p0 = ld3(X, t.x), p1 = ld3(X, t.y), p2 = ld3(X, t.z), p3 = ld3(X, t.w);
  // shape-function gradients scaled by 6V, oriented as the precomputes
  const V3t<double> da = v_sub(p0, p3), db = v_sub(p1, p3), dc = v_sub(p2, p3), ca = v_sub(p0, p2),
                    cb = v_sub(p1, p2);
  V3t<double> g[4];
  if (v_dot(da, v_cross(db, dc)) > 0.0) {
    g[0] = v_cross(db, dc); g[1] = v_cross(dc, da); g[2] = v_cross(da, db); g[3] = v_cross(cb, ca);
  } else {
    g[0] = v_cross(dc, db); g[1] = v_cross(da, dc); g[2] = v_cross(db, da); g[3] = v_cross(ca, cb);
  }
  const double f = 1.0 / (36.0 * tet_vol(p0, p1, p2, p3));
  for (int a = 0; a < 4; a++) {
    const double Ba[3] = {g[a].x, g[a].y, g[a].z};
    for (int b = a; b < 4; b++) {
      const double Bb[3] = {g[b].x, g[b].y, g[b].z};
      // K_ab(i, j), row i of node a, column j of node b
      double Kab[9];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double v;
          if (i == j) {
            const int j1 = (i + 1) % 3, j2 = (i + 2) % 3;
            const int lo = j1 < j2 ? j1 : j2, hi = j1 < j2 ? j2 : j1;
            v = D0 * Ba[i] * Bb[i] + D2 * (Ba[lo] * Bb[lo] + Ba[hi] * Bb[hi]);
          } else {
            v = D1 * Ba[i] * Bb[j] + D2 * Ba[j] * Bb[i];
          }
          Kab[3 * i + j] = v * f;
        }
      for (int i = 0; i < 3; i++) {
        const int p = 3 * a + i, dp = p * 12 - (p * (p - 1)) / 2;   // packed index of (p, p)
        if (a == b) {
          for (int j = i; j < 3; j++) k78[kst(dp + j - i, e)] = Kab[3 * i + j];
        } else {
          for (int j = 0; j < 3; j++) k78[kst(dp + 3 * b + j - p, e)] = Kab[3 * i + j];
        }
      }
    }
  }
}

od_status launch_hooke(Scene* s, double youngs, double poisson, double* Kh) {
  const int T = 128;
  cudaStream_t st = s->ctx->stream;
  const double lambda = poisson * youngs / ((1.0 + poisson) * (1.0 - 2.0 * poisson));
  const double mu = youngs / (2.0 * (1.0 + poisson));
  OD_CUDA(cudaMemsetAsync(Kh, 0, sizeof(double) * std::max(1, s->nvals), st));
  if (s->n_tets == 0) return OD_OK;
  OD_KL(s);
  hooke_stage_kernel<<<nblk(s->n_tets, T), T, 0, st>>>(s->n_tets, s->tets, s->X, lambda + 2.0 * mu, lambda, mu,
                                                      s->stage_k);
  if (s->gat_kptr) {
    if (s->nvals > 0) {
      OD_KL(s);
      gather_kernel<<<nblk(s->nvals, 256), 256, 0, st>>>(s->nvals, s->gat_kptr, s->gat_ksrc, s->stage_k, Kh, 0,
                                                         nullptr, nullptr, nullptr, nullptr, 0);
    }
  } else {
    for (size_t c = 0; c + 1 < s->color_off.size(); c++) {
      const int e0 = s->color_off[c], e1 = s->color_off[c + 1];
      if (e1 <= e0) continue;
      OD_KL(s);
      scatter_kernel<<<nblk(78LL * (e1 - e0), 256), 256, 0, st>>>(e0, e1 - e0, s->n_tets, s->stage_k, nullptr,
                                                                   s->emap, s->gdof, Kh, nullptr);
    }
  }
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

static int vol_slot(const Scene* s) {
  return s->mat.kind == OD_MATERIAL_COROTATIONAL || s->mat.kind == OD_MATERIAL_COROTATIONAL_PLASTIC ? 99 : 21;
}

od_status launch_mass(Scene* s) {
  const int T = 128;
  OD_CUDA(cudaMemsetAsync(s->M, 0, sizeof(double) * (size_t)s->nvals, s->ctx->stream));
  OD_CUDA(cudaMemsetAsync(s->node_vol4, 0, sizeof(double) * (size_t)s->n_nodes, s->ctx->stream));
  for (size_t c = 0; c + 1 < s->color_off.size(); c++) {
    int e0 = s->color_off[c], e1 = s->color_off[c + 1];
    if (e1 <= e0) continue;
    OD_KL(s);
    mass_kernel<<<nblk(e1 - e0, T), T, 0, s->ctx->stream>>>(e0, e1, s->n_tets, vol_slot(s), s->mat.density, s->pre,
                                                             s->emap, s->M);
    OD_KL(s);
    node_vol_kernel<<<nblk(e1 - e0, T), T, 0, s->ctx->stream>>>(e0, e1, s->n_tets, vol_slot(s), s->tets, s->pre,
                                                                 s->node_vol4);
  }
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status launch_eval(Scene* s, bool zero_first, bool df) {
  const int T = 128;
  cudaStream_t st = s->ctx->stream;
  if (zero_first && (!s->gat_kptr || s->n_tets == 0)) {
    OD_CUDA(cudaMemsetAsync(s->K, 0, sizeof(double) * (size_t)s->nvals, st));
    OD_CUDA(cudaMemsetAsync(s->fint, 0, sizeof(double) * (size_t)s->pcg.n_pad, st));
  }
  if (s->n_tets == 0) return OD_OK;
  // 1) every element at full occupancy into the colour-ordered staging arrays
  OD_KL(s);
  if (s->mat.kind == OD_MATERIAL_COROTATIONAL_PLASTIC)
    plastic_kernel<2><<<nblk(s->n_tets, T), T, 0, st>>>(s->n_tets, s->tets, s->X, s->u, s->pre, s->mat.threshold,
                                                         s->lambda, s->mu, s->mat.yield_criterion,
                                                         s->mat.creep_ratio, s->mat.max_plastic_strain, s->plastic,
                                                         s->stage_k, s->stage_f, nullptr);
  else if (s->mat.kind == OD_MATERIAL_COROTATIONAL && df)
    corot_kernel<2, true><<<nblk(s->n_tets, T), T, 0, st>>>(0, s->n_tets, s->n_tets, s->tets, s->X, s->u, s->pre,
                                                             s->mat.threshold, s->emap, s->gdof, nullptr, nullptr,
                                                             s->stage_k, s->stage_f, nullptr);
  else if (s->mat.kind == OD_MATERIAL_COROTATIONAL)
    corot_kernel<2><<<nblk(s->n_tets, T), T, 0, st>>>(0, s->n_tets, s->n_tets, s->tets, s->X, s->u, s->pre,
                                                       s->mat.threshold, s->emap, s->gdof, nullptr, nullptr, s->stage_k,
                                                       s->stage_f, nullptr);
  else if (df)
    invhyper_kernel<2, true><<<nblk(s->n_tets, T), T, 0, st>>>(0, s->n_tets, s->n_tets,
                                                                s->mat.kind == OD_MATERIAL_STVK, s->tets, s->X, s->u,
                                                                s->pre, s->mat.threshold, s->lambda, s->mu, s->emap,
                                                                s->gdof, nullptr, nullptr, s->stage_k, s->stage_f,
                                                                nullptr);
  else
    invhyper_kernel<2><<<nblk(s->n_tets, T), T, 0, st>>>(0, s->n_tets, s->n_tets, s->mat.kind == OD_MATERIAL_STVK,
                                                          s->tets, s->X, s->u, s->pre, s->mat.threshold, s->lambda,
                                                          s->mu, s->emap, s->gdof, nullptr, nullptr, s->stage_k,
                                                          s->stage_f, nullptr);
  // 2) assembly: one gather launch; one scatter launch per colour for meshes
  //    whose gather lists do not fit 32-bit indices
  if (s->gat_kptr) {
    const long long nd = (long long)s->nvals + s->pcg.n_pad;
    if (nd == 0) return OD_OK;
    OD_KL(s);
    gather_kernel<<<nblk(nd, 256), 256, 0, st>>>(s->nvals, s->gat_kptr, s->gat_ksrc, s->stage_k, s->K, s->pcg.n_pad,
                                                 s->gat_fptr, s->gat_fsrc, s->stage_f, s->fint, zero_first ? 0 : 1);
    OD_CUDA(cudaGetLastError());
    return OD_OK;
  }
  for (size_t c = 0; c + 1 < s->color_off.size(); c++) {
    int e0 = s->color_off[c], e1 = s->color_off[c + 1];
    if (e1 <= e0) continue;
    OD_KL(s);
    scatter_kernel<<<nblk(90LL * (e1 - e0), 256), 256, 0, st>>>(e0, e1 - e0, s->n_tets, s->stage_k, s->stage_f,
                                                                 s->emap, s->gdof, s->K, s->fint);
  }
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

od_status launch_element_values(Scene* s, double* d_k78, double* d_f12) {
  const int T = 128;
  cudaStream_t st = s->ctx->stream;
  if (s->n_tets == 0) return OD_OK;
  OD_KL(s);
  if (s->mat.kind == OD_MATERIAL_COROTATIONAL_PLASTIC)
    plastic_kernel<1><<<nblk(s->n_tets, T), T, 0, st>>>(s->n_tets, s->tets, s->X, s->u, s->pre, s->mat.threshold,
                                                         s->lambda, s->mu, s->mat.yield_criterion,
                                                         s->mat.creep_ratio, s->mat.max_plastic_strain, s->plastic,
                                                         d_k78, d_f12, s->perm);
  else if (s->mat.kind == OD_MATERIAL_COROTATIONAL)
    corot_kernel<1><<<nblk(s->n_tets, T), T, 0, st>>>(0, s->n_tets, s->n_tets, s->tets, s->X, s->u, s->pre,
                                                       s->mat.threshold, s->emap, s->gdof, nullptr, nullptr, d_k78,
                                                       d_f12, s->perm);
  else
    invhyper_kernel<1><<<nblk(s->n_tets, T), T, 0, st>>>(0, s->n_tets, s->n_tets, s->mat.kind == OD_MATERIAL_STVK,
                                                          s->tets, s->X, s->u, s->pre, s->mat.threshold, s->lambda,
                                                          s->mu, s->emap, s->gdof, nullptr, nullptr, d_k78, d_f12,
                                                          s->perm);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

// every (facet, traction) pair of the scene gets the same traction vector
__global__ void fill_traction_kernel(int n, double tx, double ty, double tz, double* __restrict__ tvec) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    tvec[3 * k] = tx;
    tvec[3 * k + 1] = ty;
    tvec[3 * k + 2] = tz;
  }
}

// New load values on the facet list of the scene's last od_scene_set_loads
// (one traction group): the traction vector is written on the device and
// the external forces re-evaluated, no copy and no synchronisation.
od_status scene_set_uniform_loads(Scene* s, const double* body, const double* traction) {
  if (traction && s->n_trac > 0) {
    OD_KL(s);
    fill_traction_kernel<<<nblk(s->n_trac, 128), 128, 0, s->ctx->stream>>>(s->n_trac, traction[0], traction[1],
                                                                            traction[2], s->trac_vec);
  }
  s->has_body = body != nullptr;
  if (body)
    for (int i = 0; i < 3; i++) s->load_body[i] = body[i];
  return launch_loads(s, body, traction ? s->n_trac : 0, 1.0);
}

// body part then traction colours; s->trac_* hold the colour-ordered facets
od_status launch_loads(Scene* s, const double* body, int n_facets_total, double traction_scale) {
  const int T = 128;
  cudaStream_t st = s->ctx->stream;
  const int n = s->pcg.n_pad;
  if (n <= 0) return OD_OK;
  double b[3] = {0, 0, 0};
  if (body) { b[0] = body[0]; b[1] = body[1]; b[2] = body[2]; }
  const bool trac = n_facets_total > 0 && s->load_ptr;
  OD_KL(s);
  loads_kernel<<<nblk(n, T), T, 0, st>>>(n, s->dofs, s->free_pos, s->node_vol4, b[0], b[1], b[2],
                                         trac ? s->load_ptr : nullptr, s->load_src, s->trac_facets, s->trac_vec,
                                         traction_scale, s->facets_dev, s->X, s->u, s->fext);
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

}  // namespace od

namespace od {

od_status launch_eval_batch(Ctx* ctx, int n_sc, const SceneDev* sd, const TileDir& zero_k, const TileDir& zero_f,
                            const TileDir& corot, const TileDir& inv, const TileDir& plastic,
                            const std::vector<TileDir>& scatter, const TileDir& gather) {
  cudaStream_t st = ctx->stream;
  const bool gathered = gather.tiles >= 0;  // every scene has gather lists
  if (!gathered && zero_k.tiles > 0) {
    ctx->launches++;
    zero_batch_kernel<<<zero_k.tiles, 256, 0, st>>>(n_sc, zero_k.prefix, 0, sd);
  }
  if (!gathered && zero_f.tiles > 0) {
    ctx->launches++;
    zero_batch_kernel<<<zero_f.tiles, 256, 0, st>>>(n_sc, zero_f.prefix, 1, sd);
  }
  if (corot.tiles > 0) {
    ctx->launches++;
    corot_batch_kernel<<<corot.tiles, 128, 0, st>>>(n_sc, corot.prefix, sd);
  }
  if (inv.tiles > 0) {
    ctx->launches++;
    invhyper_batch_kernel<<<inv.tiles, 128, 0, st>>>(n_sc, inv.prefix, sd);
  }
  if (plastic.tiles > 0) {
    ctx->launches++;
    plastic_batch_kernel<<<plastic.tiles, 128, 0, st>>>(n_sc, plastic.prefix, sd);
  }
  if (gathered) {
    if (gather.tiles > 0) {
      ctx->launches++;
      gather_batch_kernel<<<gather.tiles, 256, 0, st>>>(n_sc, gather.prefix, sd);
    }
    OD_CUDA(cudaGetLastError());
    return OD_OK;
  }
  for (size_t c = 0; c < scatter.size(); c++) {
    if (scatter[c].tiles <= 0) continue;
    ctx->launches++;
    scatter_batch_kernel<<<scatter[c].tiles, 256, 0, st>>>(n_sc, scatter[c].prefix, (int)c, sd);
  }
  OD_CUDA(cudaGetLastError());
  return OD_OK;
}

}  // namespace od
