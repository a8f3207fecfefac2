// End-to-end check of the C++ drop-in classes (include/od_gb300_dropin.hpp)
// inside the reference's own time loop: the same mesh stepped by the
// reference's backward Euler (intergrator/nonlinearImplicitBackwardEuler.h)
//   A  as shipped (reference material, CGSolver with Jacobi),
//   B  with GpuMaterial in place of the reference material,
//   C  with GpuCGSolver in place of CGSolver,
//   D  GpuIntergrator in place of the whole integrator,
//   E  as shipped with InCholeskyPreconditioner,
//   F  CGSolver with GpuInCholeskyPreconditioner,
//   G  as shipped with InLDLTPreconditioner,
//   H  CGSolver with GpuInLDLTPreconditioner,
//   I  as shipped with plane collision damping (MeshPlaneCollisionDampingForcer
//      on every element, the integrator's velocities, before every step), and
//   J  GpuIntergrator with the same damping;
// prints the relative displacement differences B, C, D against A, F against
// E, H against G and J against I, and exits 0 when all are within the given
// tolerance.
//
// usage: dropin_check <dir> <tolerance>; <dir> holds params.txt (n_nodes
// n_tets n_facets n_cdofs rho youngs poisson threshold dt alpha_m beta_k tol
// max_iter steps gx gy gz), X.bin (double), tets.bin, facets.bin, cdofs.bin
// (int32).  Test infrastructure: compiled and run by tests/test_gpu_dropin.py
// against the compiled reference (oracle/_ref) and libodgpu.so.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <climits>
#include <cstdint>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "od_gb300_dropin.hpp"

#include "cgSolver.h"
#include "constrainer.h"
#include "inCholeskyPreconditioner.h"
#include "inLDLTPreconditioner.h"
#include "invertibleNeoHookean.h"
#include "jacobiPreconditioner.h"
#include "nonlinearImplicitBackwardEuler.h"
#include "tetmesh.h"

using namespace ODER;
using Mat = BlockedSymSpMatrix;

namespace {

struct Params {
  int n_nodes, n_tets, n_facets, n_cdofs;
  double rho, youngs, poisson, thr, dt, alpha_m, beta_k, tol;
  int max_iter, steps;
  double g[3];
};

template <class T>
std::vector<T> read_bin(const std::string& path, size_t n) {
  std::vector<T> v(n);
  FILE* f = fopen(path.c_str(), "rb");
  if (!f || fread(v.data(), sizeof(T), n, f) != n) {
    fprintf(stderr, "cannot read %s\n", path.c_str());
    exit(2);
  }
  fclose(f);
  return v;
}

struct Input {
  Params p;
  std::vector<double> X;
  std::vector<int> tets, facets, cdofs;
};

struct RefSetup {
  Reference<Mesh> mesh;
  Reference<NodeIndexer> indexer;
  int dofs = 0;
};

RefSetup make_setup(const Input& in) {
  RefSetup s;
  TetMesh* m = new TetMesh(in.p.n_nodes, in.p.n_tets, in.p.n_facets);
  s.mesh = m;
  for (int i = 0; i < in.p.n_nodes; i++) m->setVertex(i, Vector3(in.X[3 * i], in.X[3 * i + 1], in.X[3 * i + 2]));
  for (int e = 0; e < in.p.n_tets; e++) m->setElement(e, const_cast<int*>(in.tets.data() + 4 * e));
  for (int f = 0; f < in.p.n_facets; f++) m->setFacet(f, const_cast<int*>(in.facets.data() + 3 * f));
  // whole-node constraints through the public API (Constrainer::setConstrains
  // with no types fixes every axis, core/constrainer.cpp:43-50)
  std::vector<int> nodes;
  for (size_t k = 0; k + 2 < in.cdofs.size(); k += 3) {
    if (in.cdofs[k] % 3 != 0 || in.cdofs[k + 1] != in.cdofs[k] + 1 || in.cdofs[k + 2] != in.cdofs[k] + 2) {
      fprintf(stderr, "constrained DOFs must be whole nodes\n");
      exit(2);
    }
    nodes.push_back(in.cdofs[k] / 3);
  }
  Constrainer c(s.mesh);
  c.setConstrains((int)nodes.size(), nodes.data());
  s.indexer = new NodeIndexer(c);
  s.dofs = s.indexer->getMatrixOrder(s.mesh);
  return s;
}

std::vector<double> displacements(const RefSetup& s, int n_nodes) {
  std::vector<double> u(3 * (size_t)n_nodes);
  for (int i = 0; i < n_nodes; i++) {
    const Vector3& d = s.mesh->getVertexDisplacementConst(i);
    u[3 * i] = d.x;
    u[3 * i + 1] = d.y;
    u[3 * i + 2] = d.z;
  }
  return u;
}

double rel_diff(const std::vector<double>& a, const std::vector<double>& b) {
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < a.size(); i++) {
    num += (a[i] - b[i]) * (a[i] - b[i]);
    den += b[i] * b[i];
  }
  return den > 0.0 ? sqrt(num / den) : sqrt(num);
}

// wall-clock time spent in one seam (a material or solver call) over a loop
struct SeamClock {
  double ms = 0.0;
  int calls = 0;
  double per_call() const { return calls ? ms / calls : 0.0; }
};

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// forwards every call to the material it wraps and times
// generateMatrixAndVirtualWorks, the seam a drop-in material replaces
class TimedMaterial : public FullOrderNonlinearMaterial<Mat> {
 public:
  TimedMaterial(const Reference<FullOrderNonlinearMaterial<Mat>>& m, Scalar rho, SeamClock* c)
      : FullOrderNonlinearMaterial(rho, MarterialType(Marterial_Isotropic | Marterial_Invertible)), inner(m),
        clock(c) {}
  FullOrderNonlinearMaterialCache getPrecomputes(const Reference<Mesh>& mesh) const override {
    return inner->getPrecomputes(mesh);
  }
  void generateMatrixAndVirtualWorks(const Reference<Mesh>& mesh, const Reference<NodeIndexer>& indexer,
                                     const FullOrderNonlinearMaterialCache& cache,
                                     const SparseSymMatrixIndicesPerElementCache& matrixIndices, Mat& matrix,
                                     Scalar* vws) const override {
    const double t0 = now_ms();
    inner->generateMatrixAndVirtualWorks(mesh, indexer, cache, matrixIndices, matrix, vws);
    clock->ms += now_ms() - t0;
    clock->calls++;
  }
  Reference<FullOrderNonlinearMaterial<Mat>> inner;
  SeamClock* clock;
};

// forwards to the solver it wraps and times solveLinearSystem
class TimedSolver : public LinearSolver<Mat> {
 public:
  TimedSolver(const Reference<LinearSolver<Mat>>& s, SeamClock* c) : inner(s), clock(c) {}
  void resetLinearSystem(const Mat* m) override {
    mat = m;
    inner->resetLinearSystem(m);
  }
  void solveLinearSystem(const Scalar* rhs, Scalar* result) override {
    const double t0 = now_ms();
    inner->solveLinearSystem(rhs, result);
    clock->ms += now_ms() - t0;
    clock->calls++;
  }
  Reference<LinearSolver<Mat>> inner;
  SeamClock* clock;
};

// times of one loop: the whole steps, and the material and solver seams
struct LoopTimes {
  SeamClock step, material, solver;
};

// the reference's backward Euler with the given material and solver
std::vector<double> run_reference_loop(const Input& in, RefSetup& s,
                                       const Reference<FullOrderNonlinearMaterial<Mat>>& material,
                                       const Reference<LinearSolver<Mat>>& solver, LoopTimes* times = nullptr) {
  LoopTimes scratch;
  LoopTimes& t = times ? *times : scratch;
  Reference<FullOrderNonlinearMaterial<Mat>> tm(new TimedMaterial(material, in.p.rho, &t.material));
  Reference<LinearSolver<Mat>> ts(new TimedSolver(solver, &t.solver));
  NonlinearImplicitBackwardEuler<Mat> be(s.dofs, in.p.alpha_m, in.p.beta_k, in.p.dt, s.mesh, s.indexer, tm, ts);
  Forcer f;
  Scalar g[3] = {in.p.g[0], in.p.g[1], in.p.g[2]};
  f.addBodyForce(s.mesh, g, s.indexer);
  be.setExternalVirtualWork(f);
  for (int k = 0; k < in.p.steps; k++) {
    const double t0 = now_ms();
    be.runOneTimeStep();
    be.updateMeshVerticesDisplacements(s.indexer, s.mesh);
    t.step.ms += now_ms() - t0;
    t.step.calls++;
  }
  return displacements(s, in.p.n_nodes);
}

// any integrator (the reference's or the drop-in, through the base class)
// with plane damping on every element, set up before every step as a
// collision loop does (odref_be_plane_damping in oracle/ref_harness.cpp)
std::vector<double> damped_loop(const Input& in, RefSetup& s, Intergrator& it) {
  Forcer f;
  Scalar g[3] = {in.p.g[0], in.p.g[1], in.p.g[2]};
  f.addBodyForce(s.mesh, g, s.indexer);
  it.setExternalVirtualWork(f);
  std::vector<Vector3> vel((size_t)in.p.n_nodes);
  Collision::StaticPlaneShape plane;
  plane.planeNormal = Vector3(0.0, 0.0, 1.0);
  plane.planeConstant = 0.0;
  for (int k = 0; k < in.p.steps; k++) {
    it.clearExternalDampingForceMatrix();
    it.getMeshVerticesVelocities(s.indexer, s.mesh, vel.data());
    Collision::MeshPlaneCollisionDampingForcer fd(100.0, s.mesh, s.indexer, vel.data());
    for (int e = 0; e < in.p.n_tets; e++) {
      fd.setCollisionPair(plane, e);
      it.addExternalDampingForceMatrix(fd);
    }
    it.runOneTimeStep();
    it.updateMeshVerticesDisplacements(s.indexer, s.mesh);
  }
  return displacements(s, in.p.n_nodes);
}

Reference<FullOrderNonlinearMaterial<Mat>> reference_material(const Input& in) {
  return Reference<FullOrderNonlinearMaterial<Mat>>(
      new InvertibleNeoHookeanMaterial(in.p.rho, in.p.youngs, in.p.poisson, in.p.thr));
}

od_scene* new_scene(od_ctx* ctx, const Input& in) {
  od_material mat{};
  mat.kind = OD_MATERIAL_NEOHOOKEAN;
  mat.density = in.p.rho;
  mat.youngs = in.p.youngs;
  mat.poisson = in.p.poisson;
  mat.threshold = in.p.thr;
  od_scene* scene = nullptr;
  if (od_scene_create(ctx, in.p.n_nodes, in.X.data(), in.p.n_tets, in.tets.data(), in.p.n_facets, in.facets.data(),
                      in.p.n_cdofs, in.cdofs.data(), &mat, &scene) != OD_OK) {
    fprintf(stderr, "od_scene_create failed\n");
    exit(3);
  }
  return scene;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: dropin_check <dir> <tolerance> [seams]\n");
    return 2;
  }
  const std::string dir = argv[1];
  const double tol_ok = atof(argv[2]);
  // "seams": only A-D, whose times are the cost of each seam at this size
  const bool seams_only = argc > 3 && std::string(argv[3]) == "seams";
  Input in;
  {
    FILE* f = fopen((dir + "/params.txt").c_str(), "r");
    Params& p = in.p;
    if (!f || fscanf(f, "%d %d %d %d %lf %lf %lf %lf %lf %lf %lf %lf %d %d %lf %lf %lf", &p.n_nodes, &p.n_tets,
                     &p.n_facets, &p.n_cdofs, &p.rho, &p.youngs, &p.poisson, &p.thr, &p.dt, &p.alpha_m, &p.beta_k,
                     &p.tol, &p.max_iter, &p.steps, &p.g[0], &p.g[1], &p.g[2]) != 17) {
      fprintf(stderr, "cannot read params.txt\n");
      return 2;
    }
    fclose(f);
  }
  in.X = read_bin<double>(dir + "/X.bin", 3 * (size_t)in.p.n_nodes);
  in.tets = read_bin<int>(dir + "/tets.bin", 4 * (size_t)in.p.n_tets);
  in.facets = read_bin<int>(dir + "/facets.bin", 3 * (size_t)in.p.n_facets);
  in.cdofs = read_bin<int>(dir + "/cdofs.bin", (size_t)in.p.n_cdofs);

  od_ctx* ctx = nullptr;
  if (od_ctx_create(0, &ctx) != OD_OK) {
    fprintf(stderr, "od_ctx_create failed\n");
    return 3;
  }
  int bad = 0;
  auto check = [&](od_status st, const char* what) {
    if (st != OD_OK) {
      fprintf(stderr, "%s: status %d\n", what, (int)st);
      bad = 1;
    }
  };
  auto jacobi_cg = [&]() {
    return Reference<LinearSolver<Mat>>(new CGSolver(in.p.tol, in.p.max_iter, Reference<Preconditioner>(new JacobiPreconditioner())));
  };

  // A: the reference as shipped
  LoopTimes ta, tb, tc, td;
  RefSetup sa = make_setup(in);
  const std::vector<double> ua = run_reference_loop(in, sa, reference_material(in), jacobi_cg(), &ta);

  // B: GpuMaterial inside the reference integrator
  od_scene* sb_scene = new_scene(ctx, in);
  RefSetup sb = make_setup(in);
  // the reference's intrusive Reference owns each drop-in; the handles
  // below keep them alive until their statuses are read
  auto* gm = new od_dropin::GpuMaterial(sb_scene, in.p.rho, MarterialType(Marterial_Isotropic | Marterial_Invertible));
  Reference<FullOrderNonlinearMaterial<Mat>> gm_ref(gm);
  const std::vector<double> ub = run_reference_loop(in, sb, gm_ref, jacobi_cg(), &tb);

  // C: GpuCGSolver inside the reference integrator
  od_scene* sc_scene = new_scene(ctx, in);
  RefSetup sc = make_setup(in);
  auto* gcg = new od_dropin::GpuCGSolver(sc_scene, in.p.tol, in.p.max_iter, OD_PRECOND_JACOBI);
  Reference<LinearSolver<Mat>> gcg_ref(gcg);
  const std::vector<double> uc = run_reference_loop(in, sc, reference_material(in), gcg_ref, &tc);

  // D: GpuIntergrator in place of the integrator
  od_scene* sd_scene = new_scene(ctx, in);
  RefSetup sd = make_setup(in);
  od_integrator_params ip{};
  ip.kind = OD_INTEGRATOR_BACKWARD_EULER;
  ip.dt = in.p.dt;
  ip.alpha_m = in.p.alpha_m;
  ip.beta_k = in.p.beta_k;
  ip.solver.tol = in.p.tol;
  ip.solver.max_iter = in.p.max_iter;
  ip.solver.precond = OD_PRECOND_JACOBI;
  ip.solver.precision = OD_PRECISION_FP64;
  std::vector<double> ud;
  {
    od_dropin::GpuIntergrator gi(sd_scene, sd.dofs, ip);
    check(gi.last_status, "GpuIntergrator setup");
    Forcer f;
    Scalar g[3] = {in.p.g[0], in.p.g[1], in.p.g[2]};
    f.addBodyForce(sd.mesh, g, sd.indexer);
    gi.setExternalVirtualWork(f);
    check(gi.last_status, "setExternalVirtualWork");
    for (int k = 0; k < in.p.steps; k++) {
      const double t0 = now_ms();
      gi.runOneTimeStep();
      check(gi.last_status, "runOneTimeStep");
      gi.updateMeshVerticesDisplacements(sd.indexer, sd.mesh);
      td.step.ms += now_ms() - t0;
      td.step.calls++;
    }
    ud = displacements(sd, in.p.n_nodes);
  }
  // per step: the whole step, the material call and the solver call (ms)
  printf("seams_ms reference step %.3f material %.3f solver %.3f | GpuMaterial step %.3f material %.3f | "
         "GpuCGSolver step %.3f solver %.3f (%d iterations) | GpuIntergrator step %.3f\n",
         ta.step.per_call(), ta.material.per_call(), ta.solver.per_call(), tb.step.per_call(),
         tb.material.per_call(), tc.step.per_call(), tc.solver.per_call(),
         tc.solver.calls ? gcg->stats.iterations : 0, td.step.per_call());
  if (seams_only) {
    check(gm->last_status, "GpuMaterial");
    check(gcg->last_status, "GpuCGSolver");
    const double eb = rel_diff(ub, ua), ec = rel_diff(uc, ua), ed = rel_diff(ud, ua);
    printf("material %.3e solver %.3e integrator %.3e\n", eb, ec, ed);
    for (od_scene* s : {sb_scene, sc_scene, sd_scene}) od_scene_destroy(s);
    od_ctx_destroy(ctx);
    return !bad && eb <= tol_ok && ec <= tol_ok && ed <= tol_ok ? 0 : 1;
  }

  // E, F: threshold incomplete Cholesky, the reference's and the drop-in
  RefSetup se = make_setup(in);
  const std::vector<double> ue = run_reference_loop(
      in, se, reference_material(in),
      Reference<LinearSolver<Mat>>(
          new CGSolver(in.p.tol, in.p.max_iter, Reference<Preconditioner>(new InCholeskyPreconditioner(1e-3, 0.0)))));
  od_scene* sf_scene = new_scene(ctx, in);
  RefSetup sf = make_setup(in);
  auto* gic = new od_dropin::GpuInCholeskyPreconditioner(sf_scene, 1e-3, 0.0);
  Reference<Preconditioner> gic_ref(gic);
  const std::vector<double> uf = run_reference_loop(
      in, sf, reference_material(in), Reference<LinearSolver<Mat>>(new CGSolver(in.p.tol, in.p.max_iter, gic_ref)));

  // G, H: incomplete LDL^T, the reference's and the drop-in
  RefSetup sg = make_setup(in);
  const std::vector<double> ug = run_reference_loop(
      in, sg, reference_material(in),
      Reference<LinearSolver<Mat>>(
          new CGSolver(in.p.tol, in.p.max_iter, Reference<Preconditioner>(new InLDLTPreconditioner(0.1, 0.01)))));
  od_scene* sh_scene = new_scene(ctx, in);
  RefSetup sh = make_setup(in);
  auto* gld = new od_dropin::GpuInLDLTPreconditioner(sh_scene, 0.1, 0.01);
  Reference<Preconditioner> gld_ref(gld);
  const std::vector<double> uh = run_reference_loop(
      in, sh, reference_material(in), Reference<LinearSolver<Mat>>(new CGSolver(in.p.tol, in.p.max_iter, gld_ref)));

  // I, J: plane collision damping through the integrator seam
  RefSetup si = make_setup(in);
  std::vector<double> ui;
  {
    NonlinearImplicitBackwardEuler<Mat> be(si.dofs, in.p.alpha_m, in.p.beta_k, in.p.dt, si.mesh, si.indexer,
                                           reference_material(in), jacobi_cg());
    ui = damped_loop(in, si, be);
  }
  od_scene* sj_scene = new_scene(ctx, in);
  RefSetup sj = make_setup(in);
  std::vector<double> uj;
  {
    od_dropin::GpuIntergrator gi(sj_scene, sj.dofs, ip);
    uj = damped_loop(in, sj, gi);
    check(gi.last_status, "GpuIntergrator with damping");
  }

  check(gm->last_status, "GpuMaterial");
  check(gld->last_status, "GpuInLDLTPreconditioner");
  check(gcg->last_status, "GpuCGSolver");
  check(gic->last_status, "GpuInCholeskyPreconditioner");
  const double eb = rel_diff(ub, ua), ec = rel_diff(uc, ua), ed = rel_diff(ud, ua), ef = rel_diff(uf, ue);
  const double eh = rel_diff(uh, ug), ej = rel_diff(uj, ui), edamp = rel_diff(ui, ua);
  double umax = 0.0;
  for (double x : ua) umax = std::max(umax, fabs(x));
  printf("umax %.6e material %.3e solver %.3e integrator %.3e ic_preconditioner %.3e ldlt_preconditioner %.3e "
         "damped_integrator %.3e (damping changes the reference's motion by %.3e)\n",
         umax, eb, ec, ed, ef, eh, ej, edamp);
  for (od_scene* s : {sb_scene, sc_scene, sd_scene, sf_scene, sh_scene, sj_scene}) od_scene_destroy(s);
  od_ctx_destroy(ctx);
  const bool ok = !bad && umax > 0.0 && edamp > 10.0 * tol_ok && eb <= tol_ok && ec <= tol_ok && ed <= tol_ok &&
                  ef <= tol_ok && eh <= tol_ok && ej <= tol_ok;
  return ok ? 0 : 1;
}
