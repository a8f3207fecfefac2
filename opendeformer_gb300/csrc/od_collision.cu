// Plane collision damping (collision/penaltyDampingForcer.cpp:8-61,
// collision/intersection.cpp:12-148): MeshPlaneCollisionDampingForcer adds,
// for each element it is given, a damping block to the integrator's external
// damping matrix (the dampMatrix of nonlinearImplicitBackwardEuler.h:86-88;
// in the Newmark step C = alpha_M M + beta_K K + D).
//
// Per element: the deformed tetrahedron is clipped by the plane n.x + c = 0
// (negative side: n.x + c < 1e-6), giving a centroid and a direction whose
// length is six times the clipped volume; w = barycentric coordinates of the
// centroid, u = dir / |dir|, and if the velocity interpolated at the
// centroid approaches the plane (v.u < 0) the element matrix gets
// w_a w_b T in its node block (a, b), T = (coeff dir) u^T.  In the reference
// the diagonal node blocks take T(i, j) for the entry (i, i + j); that is kept.
//
// Compiled without FMA contraction, so every per-element operation rounds
// as the reference's does.
//
// GB300 layout: the given elements are grouped by element colour (the same
// colouring as the assembly), and one launch per colour computes every
// element of the colour (one thread each) and adds its 78 packed values
// into the lower-layout damping values through the element map -- elements
// of one colour share no node, so no two threads touch the same value and
// no atomics are needed.  An element listed k times is added in k rounds.
#include <algorithm>
#include <cmath>
#include <vector>

#include "od_internal.h"

namespace od {
namespace {

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 d3(const double* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double dotp(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 crossp(D3 a, D3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// vector / scalar as the reference divides (by the reciprocal)
__device__ __forceinline__ D3 divs(D3 a, double s) { return a * (1.0 / s); }
__device__ __forceinline__ D3 unitv(D3 a) { return divs(a, sqrt(dotp(a, a))); }
__device__ __forceinline__ double comp(D3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// point where edge (pa, pb) meets the plane, clamped to the edge
__device__ D3 edge_point(D3 n, double c, D3 pa, D3 pb) {
  const D3 ab = pb - pa;
  double t = (-c - dotp(n, pa)) / dotp(n, ab);
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  return pa + ab * t;
}

// clipped part of the tetrahedron on the negative side of the plane
__device__ void clip(D3 n, double c, const D3* P, D3& cen, D3& dir) {
  D3 ng[4], ps[4];
  int nn = 0, np = 0;
  for (int i = 0; i < 4; i++) {
    if (dotp(n, P[i]) + c < 1e-6) ng[nn++] = P[i];
    else ps[np++] = P[i];
  }
  if (nn == 0) {
    double best = 1.7976931348623157e308;
    for (int i = 0; i < 4; i++) {
      const double d = dotp(n, P[i]) + c;
      if (d < best) { best = d; cen = P[i]; }
    }
    dir = {0.0, 0.0, 0.0};
  } else if (nn == 1) {
    const D3 q0 = edge_point(n, c, ng[0], ps[0]), q1 = edge_point(n, c, ng[0], ps[1]),
             q2 = edge_point(n, c, ng[0], ps[2]);
    cen = (((ng[0] + q0) + q1) + q2) * 0.25;
    const D3 ab = q0 - ng[0], ac = q1 - ng[0], ad = q2 - ng[0];
    const double sv = dotp(ab, crossp(ac, ad));
    dir = unitv((crossp(ab, ac) + crossp(ac, ad)) + crossp(ad, ab)) * fabs(sv);
    if (sv < 0.0) dir = dir * -1.0;
  } else if (nn == 2) {
    const D3 q0 = edge_point(n, c, ng[0], ps[0]), q1 = edge_point(n, c, ng[0], ps[1]);
    const D3 q2 = edge_point(n, c, ng[1], ps[0]), q3 = edge_point(n, c, ng[1], ps[1]);
    const D3 ab = ng[1] - ng[0];
    const D3 c0 = ((ng[0] + ng[1]) + q2) + q3;
    const double v0 = fabs(dotp(ng[1] - ng[0], crossp(q2 - ng[0], q3 - ng[0])));
    const D3 c1 = ((ng[0] + q0) + q1) + q2;
    const double v1 = fabs(dotp(q0 - ng[0], crossp(q1 - ng[0], q2 - ng[0])));
    const D3 c2 = ((ng[0] + q1) + q2) + q3;
    const double v2 = fabs(dotp(q1 - ng[0], crossp(q2 - ng[0], q3 - ng[0])));
    cen = divs((c0 * v0 + c1 * v1) + c2 * v2, (v0 + v1) + v2) * 0.25;
    const D3 d = ((((crossp(q0 - ng[0], q1 - ng[0]) + crossp(q3 - ng[1], q2 - ng[1])) + crossp(ab, q2 - ng[0])) +
                   crossp(q2 - ng[0], q0 - ng[0])) +
                  crossp(q3 - ng[0], ab)) +
                 crossp(q1 - ng[0], q3 - ng[0]);
    dir = unitv(d) * ((v0 + v1) + v2);
    if (dotp(ng[1] - ng[0], crossp(ps[0] - ng[0], ps[1] - ng[0])) < 0.0) dir = dir * -1.0;
  } else if (nn == 3) {
    const D3 q0 = edge_point(n, c, ng[0], ps[0]), q1 = edge_point(n, c, ng[1], ps[0]),
             q2 = edge_point(n, c, ng[2], ps[0]);
    const D3 ab = q0 - ps[0], ac = q1 - ps[0], ad = q2 - ps[0];
    const D3 cs = ((P[0] + P[1]) + P[2]) + P[3];
    const double sv = dotp(ng[0] - ps[0], crossp(ng[1] - ps[0], ng[2] - ps[0]));
    const double v = fabs(sv);
    const D3 c0 = ((ps[0] + q0) + q1) + q2;
    const double v0 = fabs(dotp(ab, crossp(ac, ad)));
    cen = divs(cs * v - c0 * v0, v - v0) * 0.25;
    dir = unitv((crossp(ab, ac) + crossp(ac, ad)) + crossp(ad, ab)) * (v - v0);
    if (sv > 0.0) dir = dir * -1.0;
  } else {
    cen = (((P[0] + P[1]) + P[2]) + P[3]) * 0.25;
    const double vol = fabs(dotp(P[1] - P[0], crossp(P[2] - P[0], P[3] - P[0])));
    dir = n * vol;
  }
}

__device__ void bary(const D3* P, D3 p, double w[4]) {
  const D3 ab = P[1] - P[0], ac = P[2] - P[0], ad = P[3] - P[0], bc = P[2] - P[1], bd = P[3] - P[1];
  const D3 ap = p - P[0], bp = p - P[1];
  const double va = fabs(dotp(bp, crossp(bc, bd))), vb = fabs(dotp(ap, crossp(ac, ad)));
  const double vc = fabs(dotp(ap, crossp(ab, ad))), vd = fabs(dotp(ap, crossp(ab, ac)));
  const double vol = fabs(dotp(ab, crossp(ac, ad)));
  if (vol <= 1e-6) {
    w[0] = w[1] = w[2] = w[3] = 0.25;
    return;
  }
  const double inv = 1.0 / vol;
  w[0] = va * inv;
  w[1] = vb * inv;
  w[2] = vc * inv;
  w[3] = vd * inv;
}

struct PlaneArgs {
  double n[3], c, coeff;
};

// one thread per listed element of one colour (pos: colour-order positions)
__global__ void plane_damping_kernel(int cnt, const int* __restrict__ pos, int ne, const int4* __restrict__ tets,
                                     const double* __restrict__ X, const double* __restrict__ u,
                                     const double* __restrict__ node_vel, const double* __restrict__ v_dof,
                                     const int* __restrict__ node_dof, const int* __restrict__ emap, PlaneArgs pa,
                                     double* __restrict__ D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int e = pos[t];
  const int4 tv = tets[e];
  const int nd[4] = {tv.x, tv.y, tv.z, tv.w};
  D3 P[4];
  for (int i = 0; i < 4; i++) P[i] = d3(X + 3 * (size_t)nd[i]) + d3(u + 3 * (size_t)nd[i]);
  const D3 n = {pa.n[0], pa.n[1], pa.n[2]};
  D3 cen = {0.0, 0.0, 0.0}, dir = {0.0, 0.0, 0.0};
  clip(n, pa.c, P, cen, dir);
  double w[4];
  bary(P, cen, w);
  D3 un = {0.0, 0.0, 0.0};
  if (dotp(dir, dir) != 0.0) un = unitv(dir);
  D3 vel = {0.0, 0.0, 0.0};
  for (int i = 0; i < 4; i++) {
    D3 vi;
    if (node_vel) {
      vi = d3(node_vel + 3 * (size_t)nd[i]);
    } else {
      double c3[3];
      for (int a = 0; a < 3; a++) {
        const int g = node_dof[3 * nd[i] + a];
        c3[a] = g >= 0 ? v_dof[g] : 0.0;
      }
      vi = {c3[0], c3[1], c3[2]};
    }
    vel = vel + vi * w[i];
  }
  if (!(dotp(vel, un) < 0.0)) return;
  const D3 cd = dir * pa.coeff;
  double T[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) T[i][j] = comp(cd, i) * comp(un, j);
  // packed row-wise upper triangle of the 12x12: row r starts at diag[r]
  const int diag[12] = {0, 12, 23, 33, 42, 50, 57, 63, 68, 72, 75, 77};
  for (int a = 0; a < 4; a++) {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3 - i; j++) {
        const int idx = emap[(size_t)(diag[3 * a + i] + j) * ne + e];
        if (idx >= 0) D[idx] += w[a] * w[a] * T[i][j];
      }
    for (int b = a + 1; b < 4; b++)
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          const int idx = emap[(size_t)(diag[3 * a + i] + (b - a) * 3 - i + j) * ne + e];
          if (idx >= 0) D[idx] += w[a] * w[b] * T[i][j];
        }
  }
}

}  // namespace
}  // namespace od

using namespace od;

extern "C" od_status od_scene_get_damping(od_scene* scene, double* values) {
  OD_CHECK_ARG(scene && values, "od_scene_get_damping: NULL argument");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  if (s->nvals > 0)
    OD_CUDA(cudaMemcpyAsync(values, s->Dm, sizeof(double) * s->nvals, cudaMemcpyDeviceToHost, s->ctx->stream));
  return sync_stream(s);
}

extern "C" od_status od_scene_clear_damping(od_scene* scene) {
  OD_CHECK_ARG(scene, "od_scene_clear_damping: scene is NULL");
  Scene* s = &scene->s;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  OD_CUDA(cudaMemsetAsync(s->Dm, 0, sizeof(double) * std::max(1, s->nvals), s->ctx->stream));
  s->has_damping = false;
  return sync_stream(s);
}

extern "C" od_status od_scene_add_plane_damping(od_scene* scene, const double* normal, double constant,
                                                double damping, int n_elems, const int* elems,
                                                const double* node_velocities) {
  OD_CHECK_ARG(scene && normal, "od_scene_add_plane_damping: NULL argument");
  OD_CHECK_ARG(n_elems >= 0 && (n_elems == 0 || elems), "od_scene_add_plane_damping: bad element list");
  OD_CHECK_ARG(std::isfinite(constant) && std::isfinite(damping) && std::isfinite(normal[0]) &&
                   std::isfinite(normal[1]) && std::isfinite(normal[2]),
               "od_scene_add_plane_damping: non-finite plane or coefficient");
  Scene* s = &scene->s;
  OD_CHECK_ARG(node_velocities || s->has_integrator,
               "od_scene_add_plane_damping: no node velocities and no integrator to take them from");
  for (int k = 0; k < n_elems; k++)
    OD_CHECK_ARG(elems[k] >= 0 && elems[k] < s->n_tets, "od_scene_add_plane_damping: element id out of range");
  if (n_elems == 0) return OD_OK;
  OD_CUDA(cudaSetDevice(s->ctx->device));
  cudaStream_t strm = s->ctx->stream;
  // colour-order position and colour of every listed element; the k-th
  // listing of an element goes to round k
  std::vector<int> where(s->n_tets);
  for (int p = 0; p < s->n_tets; p++) where[s->elem_perm[p]] = p;
  std::vector<int> seen(s->n_tets, 0);
  int rounds = 0;
  std::vector<int> rnd(n_elems), col(n_elems);
  for (int k = 0; k < n_elems; k++) {
    const int p = where[elems[k]];
    rnd[k] = seen[elems[k]]++;
    rounds = std::max(rounds, rnd[k] + 1);
    col[k] = (int)(std::upper_bound(s->color_off.begin(), s->color_off.end(), p) - s->color_off.begin()) - 1;
  }
  std::vector<int> order(n_elems);
  for (int k = 0; k < n_elems; k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return rnd[a] != rnd[b] ? rnd[a] < rnd[b] : col[a] < col[b];
  });
  std::vector<int> pos(n_elems), group_off(1, 0);
  for (int k = 0; k < n_elems; k++) {
    pos[k] = where[elems[order[k]]];
    if (k > 0 && (rnd[order[k]] != rnd[order[k - 1]] || col[order[k]] != col[order[k - 1]]))
      group_off.push_back(k);
  }
  group_off.push_back(n_elems);
  int* d_pos = nullptr;
  double* d_vel = nullptr;
  OD_CUDA(cudaMalloc(&d_pos, sizeof(int) * n_elems));
  od_status rc = OD_OK;
  do {
    if (cudaMemcpyAsync(d_pos, pos.data(), sizeof(int) * n_elems, cudaMemcpyHostToDevice, strm) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "od_scene_add_plane_damping: upload");
      break;
    }
    if (node_velocities) {
      const size_t nb = sizeof(double) * 3 * (size_t)s->n_nodes;
      if (cudaMalloc(&d_vel, nb) != cudaSuccess ||
          cudaMemcpyAsync(d_vel, node_velocities, nb, cudaMemcpyHostToDevice, strm) != cudaSuccess) {
        rc = cuda_fail(cudaGetLastError(), "od_scene_add_plane_damping: velocities");
        break;
      }
    }
    PlaneArgs pa{{normal[0], normal[1], normal[2]}, constant, damping};
    for (size_t gi = 0; gi + 1 < group_off.size(); gi++) {
      const int g0 = group_off[gi], cnt = group_off[gi + 1] - g0;
      OD_KL(s);
      plane_damping_kernel<<<(cnt + 127) / 128, 128, 0, strm>>>(cnt, d_pos + g0, s->n_tets, s->tets, s->X, s->u, d_vel,
                                                                 s->v, s->node_dof, s->emap, pa, s->Dm);
    }
    if (cudaGetLastError() != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "od_scene_add_plane_damping: launch");
      break;
    }
    rc = sync_stream(s);
  } while (0);
  cudaFree(d_pos);
  cudaFree(d_vel);
  if (rc == OD_OK) s->has_damping = true;
  return rc;
}
