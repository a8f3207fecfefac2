// Drop-in implementations of OpenDeformer's seams on the GB300 C ABI.
//
// Each class implements one of the reference's virtual interfaces and
// forwards to include/od_gb300.h, so a reference-based program switches to
// the GPU step by constructing these instead of the reference's own
// classes.  Compile inside such a program: the reference's core/, material/,
// solver/, intergrator/ and collision/ directories on the include path
// (with the reference's own build defines), and link libodgpu.so.
//
//   GpuMaterial                 FullOrderNonlinearMaterial<BlockedSymSpMatrix>
//                               (material/fullOrderNonlinear.h:36-44)
//   GpuCGSolver                 LinearSolver<BlockedSymSpMatrix> (core/linearSolver.h:12-20),
//                               the CGSolver of solver/cgSolver.cpp:13-57
//   GpuInCholeskyPreconditioner Preconditioner (core/preconditioner.h:12-22),
//                               solver/inCholeskyPreconditioner.cpp
//   GpuInLDLTPreconditioner     Preconditioner, solver/inLDLTPreconditioner.cpp
//   GpuIntergrator              Intergrator (core/intergrator.h:13-35): the whole
//                               time step (backward Euler or Newmark, as set up
//                               on the scene) on the device
//
// Every class holds an od_scene created from the same mesh, constraints and
// material as the reference objects it replaces (od_scene_create); the
// value layout, pattern and element map are the reference's own, so values
// cross the seam without permutation.  The reference has no error channel;
// each class keeps the status of its last C ABI call in last_status.
#pragma once

#include <cstring>
#include <type_traits>
#include <vector>

#include "od_gb300.h"

#include "oder.h"
#include "mesh.h"
#include "nodeIndexer.h"
#include "sparseMatrix.h"
#include "forcer.h"
#include "linearSolver.h"
#include "preconditioner.h"
#include "intergrator.h"
#include "fullOrderNonlinear.h"
#include "penaltyDampingForcer.h"

namespace od_dropin {

static_assert(std::is_same<ODER::Scalar, double>::value, "the C ABI takes FP64 arrays");

// The reference keeps the matrix values and the plane forcer's pair private
// and offers no getter.  An explicit instantiation may name a private member
// (the language does not check access there), which lets these accessors
// read them without changing the reference.
template <class Tag, typename Tag::type M>
struct Expose {
  friend typename Tag::type member(Tag) { return M; }
};
struct MatValues {
  using type = ODER::Scalar* ODER::BlockedSymSpMatrix::*;
  friend type member(MatValues);
};
struct PlaneOf {
  using type = ODER::Collision::StaticPlaneShape ODER::Collision::MeshPlaneCollisionDampingForcer::*;
  friend type member(PlaneOf);
};
struct ElementOf {
  using type = int ODER::Collision::MeshPlaneCollisionDampingForcer::*;
  friend type member(ElementOf);
};
struct CoeffOf {
  using type = ODER::Scalar ODER::Collision::PenaltyDampingForcer::*;
  friend type member(CoeffOf);
};
template struct Expose<MatValues, &ODER::BlockedSymSpMatrix::values>;
template struct Expose<PlaneOf, &ODER::Collision::MeshPlaneCollisionDampingForcer::plane>;
template struct Expose<ElementOf, &ODER::Collision::MeshPlaneCollisionDampingForcer::elementIndex>;
template struct Expose<CoeffOf, &ODER::Collision::PenaltyDampingForcer::dampingCoeff>;

inline const double* values_of(const ODER::BlockedSymSpMatrix& m) { return m.*member(MatValues{}); }

// mesh displacement (Mesh::getVertexDisplacement, core/mesh.h:38-39) <-> scene
inline od_status upload_displacements(od_scene* scene, const ODER::Mesh& mesh) {
  const int n = mesh.getNodeCount();
  std::vector<double> u(3 * (size_t)n);
  for (int i = 0; i < n; i++) {
    const ODER::Vector3& d = mesh.getVertexDisplacementConst(i);
    u[3 * (size_t)i] = d.x;
    u[3 * (size_t)i + 1] = d.y;
    u[3 * (size_t)i + 2] = d.z;
  }
  return od_scene_set_displacements(scene, u.data());
}

inline od_status download_displacements(od_scene* scene, ODER::Mesh& mesh) {
  const int n = mesh.getNodeCount();
  std::vector<double> u(3 * (size_t)n);
  const od_status st = od_scene_get_displacements(scene, u.data());
  if (st != OD_OK) return st;
  for (int i = 0; i < n; i++) {
    ODER::Vector3& d = mesh.getVertexDisplacement(i);
    d.x = u[3 * (size_t)i];
    d.y = u[3 * (size_t)i + 1];
    d.z = u[3 * (size_t)i + 2];
  }
  return OD_OK;
}

// generateMatrixAndVirtualWorks accumulates into matrix and vws, which the
// caller zeroes (material/fullOrderNonlinear.h:40-41): the scene evaluates its
// elements at the mesh's displacement and the values are added in the
// reference layout.  The material law is the scene's (od_material).
class GpuMaterial : public ODER::FullOrderNonlinearMaterial<ODER::BlockedSymSpMatrix> {
 public:
  GpuMaterial(od_scene* s, ODER::Scalar rho, ODER::MarterialType type)
      : FullOrderNonlinearMaterial(rho, type), scene(s) {}
  void generateMatrixAndVirtualWorks(const ODER::Reference<ODER::Mesh>& mesh,
                                     const ODER::Reference<ODER::NodeIndexer>& indexer,
                                     const ODER::FullOrderNonlinearMaterialCache& cache,
                                     const ODER::SparseSymMatrixIndicesPerElementCache& matrixIndices,
                                     ODER::BlockedSymSpMatrix& matrix, ODER::Scalar* vws) const override {
    (void)indexer;
    (void)cache;
    (void)matrixIndices;
    last_status = upload_displacements(scene, *mesh);
    if (last_status != OD_OK) return;
    std::vector<double> values((size_t)matrix.getNumEntries()), fint((size_t)matrix.getNumColumns());
    last_status = od_scene_evaluate(scene, values.data(), fint.data());
    if (last_status != OD_OK) return;
    for (int i = 0; i < (int)values.size(); i++) matrix.addEntry(i, values[i]);
    for (int i = 0; i < (int)fint.size(); i++) vws[i] += fint[i];
  }
  od_scene* scene;
  mutable od_status last_status = OD_OK;
};

// CGSolver::solveLinearSystem: PCG on the matrix last passed to
// resetLinearSystem; result is the warm start and the solution
class GpuCGSolver : public ODER::LinearSolver<ODER::BlockedSymSpMatrix> {
 public:
  GpuCGSolver(od_scene* s, double tol, int max_iter, int precond, const ODER::BlockedSymSpMatrix* m = nullptr)
      : LinearSolver(m), scene(s) {
    std::memset(&params, 0, sizeof(params));
    params.tol = tol;
    params.max_iter = max_iter;
    params.precond = precond;
    params.precision = OD_PRECISION_FP64;
  }
  void solveLinearSystem(const ODER::Scalar* rhs, ODER::Scalar* result) override {
    last_status = od_scene_pcg(scene, values_of(*mat), rhs, result, &params, &stats);
  }
  od_scene* scene;
  od_solver_params params;
  od_solve_stats stats{};
  od_status last_status = OD_OK;
};

// Preprocess (inCholeskyPreconditioner.cpp:76-130) factors on the host,
// bit-identical to the reference's; solvePreconditionerSystem (:132-162)
// runs the two triangular sweeps on the device
class GpuInCholeskyPreconditioner : public ODER::Preconditioner {
 public:
  GpuInCholeskyPreconditioner(od_scene* s, ODER::Scalar epsilon, ODER::Scalar relaxedScale)
      : scene(s), eps(epsilon), relax(relaxedScale) {}
  using Preconditioner::Preprocess;
  void Preprocess(const ODER::BlockedSymSpMatrix& mat) override {
    last_status = od_scene_ic_factor(scene, values_of(mat), eps, relax, nullptr);
  }
  void solvePreconditionerSystem(int width, const ODER::Scalar* rhs, ODER::Scalar* result) const override {
    (void)width;
    last_status = od_scene_ic_apply(scene, rhs, result);
  }
  od_scene* scene;
  ODER::Scalar eps, relax;
  mutable od_status last_status = OD_OK;
};

// InLDLTPreconditioner(sainvEpsilon, ldltEpsilon) (inLDLTPreconditioner.cpp)
class GpuInLDLTPreconditioner : public ODER::Preconditioner {
 public:
  GpuInLDLTPreconditioner(od_scene* s, ODER::Scalar sainvEpsilon, ODER::Scalar ldltEpsilon)
      : scene(s), sainv_eps(sainvEpsilon), ldlt_eps(ldltEpsilon) {}
  using Preconditioner::Preprocess;
  void Preprocess(const ODER::BlockedSymSpMatrix& mat) override {
    last_status = od_scene_ldlt_factor(scene, values_of(mat), sainv_eps, ldlt_eps, nullptr);
  }
  void solvePreconditionerSystem(int width, const ODER::Scalar* rhs, ODER::Scalar* result) const override {
    (void)width;
    last_status = od_scene_ldlt_apply(scene, rhs, result);
  }
  od_scene* scene;
  ODER::Scalar sainv_eps, ldlt_eps;
  mutable od_status last_status = OD_OK;
};

// The integrator seam: the step (integrator, solver and preconditioner as
// given in params) runs on the device; loads, displacements, velocities and
// the plane collision damping cross the seam.
class GpuIntergrator : public ODER::Intergrator {
 public:
  GpuIntergrator(od_scene* s, int dofs, const od_integrator_params& params)
      : Intergrator(dofs, params.alpha_m, params.beta_k, params.dt), scene(s) {
    last_status = od_integrator_setup(scene, &params);
  }
  void setExternalVirtualWork(const ODER::Forcer& forcer) override {   // forcer.cpp:80-96
    std::vector<double> vws((size_t)dofs, 0.0);
    forcer.getVirtualWorks(dofs, dofs, nullptr, vws.data());
    last_status = od_scene_set_external_forces(scene, vws.data());
  }
  // MeshPlaneCollisionDampingForcer (collision/penaltyDampingForcer.cpp:8-61):
  // its plane, coefficient and element go to the device, which forms the
  // damping block from the integrator's own velocities
  void addExternalDampingForceMatrix(const ODER::StaDampingForcer& forcer) override {
    const auto* p = dynamic_cast<const ODER::Collision::MeshPlaneCollisionDampingForcer*>(&forcer);
    if (!p) {
      last_status = OD_ERR_UNSUPPORTED;
      return;
    }
    const ODER::Collision::StaticPlaneShape& plane = p->*member(PlaneOf{});
    const int elem = p->*member(ElementOf{});
    const double coeff = static_cast<const ODER::Collision::PenaltyDampingForcer*>(p)->*member(CoeffOf{});
    const double n[3] = {plane.planeNormal.x, plane.planeNormal.y, plane.planeNormal.z};
    last_status = od_scene_add_plane_damping(scene, n, plane.planeConstant, coeff, 1, &elem, nullptr);
  }
  void clearExternalDampingForceMatrix() override { last_status = od_scene_clear_damping(scene); }
  void runOneTimeStep() override { last_status = od_step(scene, 1, &stats); }
  void updateMeshVerticesDisplacements(const ODER::Reference<ODER::NodeIndexer>& indexer,
                                       ODER::Reference<ODER::Mesh>& mesh) const override {
    (void)indexer;
    last_status = download_displacements(scene, *mesh);
  }
  // free-DOF velocities mapped to nodes by the indexer (constrained axes 0)
  void getMeshVerticesVelocities(const ODER::Reference<ODER::NodeIndexer>& indexer,
                                 const ODER::Reference<ODER::Mesh>& mesh, ODER::Vector3* velocities) const override {
    std::vector<double> d((size_t)dofs), v((size_t)dofs), a((size_t)dofs);
    last_status = od_get_state(scene, d.data(), v.data(), a.data());
    if (last_status != OD_OK) return;
    for (int i = 0; i < mesh->getNodeCount(); i++) {
      double c[3];
      for (int ax = 0; ax < 3; ax++) {
        const int g = indexer->getGlobalIndex(i, ax);
        c[ax] = g >= 0 ? v[(size_t)g] : 0.0;
      }
      velocities[i] = ODER::Vector3(c[0], c[1], c[2]);
    }
  }
  od_scene* scene;
  od_step_stats stats{};
  mutable od_status last_status = OD_OK;
};

// LinearNewmark (intergrator/linearNewmark.h:13-41), the modal integrator.
// Its constructor's mesh and indexer are the scene's mesh and constraints;
// HookeMaterial keeps its moduli private, so youngs and poisson are passed
// here (the density is the scene's).  The eigenpairs come from the device
// Lanczos solve (od_modal_create) instead of ARPACK.
class GpuLinearNewmark : public ODER::Intergrator {
 public:
  GpuLinearNewmark(od_scene* s, ODER::Scalar beta, ODER::Scalar gamma, int DOFS, ODER::Scalar massDamp,
                   ODER::Scalar stiffDamp, ODER::Scalar ts, ODER::Scalar youngs, ODER::Scalar poisson)
      : Intergrator(DOFS, massDamp, stiffDamp, ts), scene(s) {
    od_scene_info info{};
    last_status = od_scene_get_info(scene, &info);
    totalDofs = info.dofs;
    nodes = info.n_nodes;
    if (last_status != OD_OK) return;
    od_modal_params p{};
    p.n_modes = DOFS;
    p.beta = beta;
    p.gamma = gamma;
    p.alpha_m = massDamp;
    p.beta_k = stiffDamp;
    p.dt = ts;
    p.youngs = youngs;
    p.poisson = poisson;
    last_status = od_modal_create(scene, &p, &modal);
  }
  ~GpuLinearNewmark() override { od_modal_destroy(modal); }
  GpuLinearNewmark(const GpuLinearNewmark&) = delete;
  GpuLinearNewmark& operator=(const GpuLinearNewmark&) = delete;
  // the forcer's full-order virtual works (forcer.cpp:80-96), projected on
  // the modes on the device (linearNewmark.cpp:52-55)
  void setExternalVirtualWork(const ODER::Forcer& forcer) override {
    std::vector<double> vws((size_t)totalDofs, 0.0);
    forcer.getVirtualWorks(totalDofs, totalDofs, nullptr, vws.data());
    last_status = od_modal_set_external_forces(modal, vws.data());
  }
  void runOneTimeStep() override { last_status = od_modal_step(modal, 1); }
  // free DOFs only; constrained axes keep the mesh's value (linearNewmark.cpp:94-108)
  void updateMeshVerticesDisplacements(const ODER::Reference<ODER::NodeIndexer>& indexer,
                                       ODER::Reference<ODER::Mesh>& mesh) const override {
    std::vector<double> u(3 * (size_t)nodes);
    last_status = od_modal_get_displacements(modal, u.data());
    if (last_status != OD_OK) return;
    for (int i = 0; i < nodes; i++)
      for (int ax = 0; ax < 3; ax++)
        if (indexer->getGlobalIndex(i, ax) >= 0) mesh->getVertexDisplacement(i)[ax] = u[3 * (size_t)i + ax];
  }
  void getMeshVerticesVelocities(const ODER::Reference<ODER::NodeIndexer>& indexer,
                                 const ODER::Reference<ODER::Mesh>& mesh, ODER::Vector3* velocities) const override {
    (void)indexer;
    (void)mesh;
    std::vector<double> v(3 * (size_t)nodes);
    last_status = od_modal_get_velocities(modal, v.data());
    if (last_status != OD_OK) return;
    for (int i = 0; i < nodes; i++)
      velocities[i] = ODER::Vector3(v[3 * (size_t)i], v[3 * (size_t)i + 1], v[3 * (size_t)i + 2]);
  }
  od_scene* scene;
  od_modal* modal = nullptr;
  int totalDofs = 0, nodes = 0;
  mutable od_status last_status = OD_OK;
};

}  // namespace od_dropin
