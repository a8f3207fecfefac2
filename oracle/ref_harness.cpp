// C API around the compiled reference (test infrastructure only).
//
// This file is compiled together with the patched copy of the reference's
// hot-path sources by oracle/build_ref.py.  It drives the reference's own
// classes -- TetMesh, Constrainer/NodeIndexer, the full-order materials,
// BlockedSymSparseMatrix, SpMDV, CGSolver with its preconditioners and
// NonlinearImplicitBackwardEuler -- and exposes them to Python (ctypes) so the
// oracle restatement and the GPU path can be compared against the reference
// on identical inputs.  It also holds a full-order Newmark integrator written
// for this project from the reference's modal Newmark formulas
// (intergrator/linearNewmark.cpp:27-30,57-79) with a Newton loop, built only
// from reference components (material, Scale/Add, SpMDV, CGSolver), because
// the reference has no full-order Newmark.
//
// Access to private members (pattern arrays, private material helpers) is by
// compiling the reference headers with private/protected mapped to public in
// this translation unit only.
#include <math.h>
#include <string.h>
#include <stdio.h>
#include <algorithm>
#include <array>
#include <atomic>
#include <climits>
#include <cstdint>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>
#include <malloc.h>

#define private public
#define protected public
#include "oder.h"
#include "memory.h"
#include "latool.h"
#include "sparseMatrix.h"
#include "numerMethod.h"
#include "mesh.h"
#include "tetmesh.h"
#include "tetelement.h"
#include "constrainer.h"
#include "nodeIndexer.h"
#include "forcer.h"
#include "fullOrderNonlinear.h"
#include "corotationalHyperelastic.h"
#include "invertibleHyperelastic.h"
#include "invertibleNeoHookean.h"
#include "invertibleStVK.h"
#include "corotationalPlastic.h"
#include "hooke.h"
#include "preconditioner.h"
#include "linearSolver.h"
#include "cgSolver.h"
#include "jacobiPreconditioner.h"
#include "inCholeskyPreconditioner.h"
#include "inLDLTPreconditioner.h"
#include "penaltyDampingForcer.h"
#include "meshRelabeler.h"
#include "intergrator.h"
#include "nonlinearImplicitBackwardEuler.h"
#undef private
#undef protected

using namespace ODER;
using Mat = BlockedSymSpMatrix;
using Material = FullOrderNonlinearMaterial<Mat>;

namespace {

// Forwards to a real preconditioner and counts applications, so the number of
// CG iterations (applications - 1) can be reported without touching CGSolver.
struct CountingPreconditioner : public Preconditioner {
  Reference<Preconditioner> inner;
  mutable int applications = 0;
  explicit CountingPreconditioner(Preconditioner* p) : inner(p) {}
  void solvePreconditionerSystem(int width, const Scalar* rhs, Scalar* result) const override {
    applications++;
    inner->solvePreconditionerSystem(width, rhs, result);
  }
  void resetPreconditionerSystem(const BlockedSymSpMatrix& mat) override { inner->resetPreconditionerSystem(mat); }
  void Preprocess(const BlockedSymSpMatrix& mat) override { inner->Preprocess(mat); }
};

Preconditioner* make_preconditioner(int kind, double eps, double relax) {
  switch (kind) {
    case 1: return new JacobiPreconditioner();
    case 2: return new InCholeskyPreconditioner(eps, relax);
    case 3: return new InLDLTPreconditioner(eps, relax);  // (sainvEpsilon, ldltEpsilon)
    default: return new Preconditioner();
  }
}

// Full-order Newmark (beta, gamma) with a Newton loop on the acceleration:
//   predictor  d~ = d + h v + (1/2 - beta) h^2 a,   v~ = v + (1 - gamma) h a
//   iterate    d_k = d~ + beta h^2 a_k,  v_k = v~ + gamma h a_k
//              r   = f_ext - f_int(d_k) - (alpha M + beta_K K) v_k - M a_k
//              [(1 + gamma h alpha) M + (gamma h beta_K + beta h^2) K] da = r
//              a_k += da        (a_0 = a of the previous step, da starts at 0)
//   corrector  d = d~ + beta h^2 a,  v = v~ + gamma h a
struct RefNewmark {
  int dofs;
  double beta, gamma, alphaM, betaK, h;
  int newton;
  std::vector<double> d, v, a, dp, vp, fint, fext, r, tmp, y, da;
  Mat* K = nullptr;
  Mat* M = nullptr;
  Reference<LinearSolver<Mat>> solver;
  int last_pcg_iterations = 0;
};

}  // namespace

struct RefScene {
  Reference<Mesh> mesh;
  Reference<NodeIndexer> indexer;
  Reference<Material> material;
  int n_nodes = 0, n_tets = 0, dofs = 0;
  int mat_kind = 0;
  Mat* pattern = nullptr;
  Mat* mass = nullptr;
  SparseSymMatrixIndicesPerElementCache indices;
  FullOrderNonlinearMaterialCache cache;
  Forcer forcer;
  std::vector<int> cdofs;
  // backward Euler
  NonlinearImplicitBackwardEuler<Mat>* be = nullptr;
  CountingPreconditioner* be_precond = nullptr;
  // Newmark
  RefNewmark* nm = nullptr;
  CountingPreconditioner* nm_precond = nullptr;
  // a stand-alone incomplete LDL^T factor (odref_ldlt_*)
  InLDLTPreconditioner* ldlt = nullptr;
  // a stand-alone threshold incomplete Cholesky factor (odref_ic_*)
  InCholeskyPreconditioner* ic = nullptr;
};

static void write_free_dofs_to_mesh(RefScene* s, const double* d) {
  auto it = s->indexer->getConstrainIterBegin();
  auto end = s->indexer->getConstrainIterEnd();
  int k = 0;
  for (int n = 0; n < s->n_nodes; n++)
    for (int ax = 0; ax < 3; ax++) {
      if (it != end && 3 * n + ax == *it) it++;
      else s->mesh->getVertexDisplacement(n)[ax] = d[k++];
    }
}

// CorotationalPlasticMaterial parameters for the next scene of kind 3
// (yieldCriterion, creepRatio, maxPlasticStrain)
static double g_plastic[3] = {1e-3, 0.5, 0.05};

extern "C" {

void odref_plastic_params(double yield, double creep, double max_strain) {
  g_plastic[0] = yield;
  g_plastic[1] = creep;
  g_plastic[2] = max_strain;
}

void* odref_scene_create(int n_nodes, const double* X, int n_tets, const int* tets,
                         int n_facets, const int* facets, int n_cdofs, const int* cdofs,
                         int mat_kind, double rho, double youngs, double poisson, double threshold) {
  RefScene* s = new RefScene();
  TetMesh* m = new TetMesh(n_nodes, n_tets, n_facets);
  s->mesh = m;
  for (int i = 0; i < n_nodes; i++) m->setVertex(i, Vector3(X[3 * i], X[3 * i + 1], X[3 * i + 2]));
  for (int e = 0; e < n_tets; e++) m->setElement(e, const_cast<int*>(tets + 4 * e));
  for (int f = 0; f < n_facets; f++) m->setFacet(f, const_cast<int*>(facets + 3 * f));
  Constrainer c(s->mesh);
  for (int i = 0; i < n_cdofs; i++) c.constrains.insert(cdofs[i]);
  s->indexer = new NodeIndexer(c);
  s->cdofs.assign(cdofs, cdofs + n_cdofs);
  s->n_nodes = n_nodes;
  s->n_tets = n_tets;
  s->dofs = s->indexer->getMatrixOrder(s->mesh);
  s->mat_kind = mat_kind;
  if (mat_kind == 0) s->material = new CorotationalHyperelasticMaterial(rho, youngs, poisson, threshold);
  else if (mat_kind == 1) s->material = new InvertibleNeoHookeanMaterial(rho, youngs, poisson, threshold);
  else if (mat_kind == 3)
    s->material = new CorotationalPlasticMaterial(rho, youngs, poisson, g_plastic[0], g_plastic[1], g_plastic[2],
                                                  threshold);
  else s->material = new InvertibleStVKMaterial(rho, youngs, poisson, threshold);

  Mat::Assembler assembler(s->dofs);
  s->material->getMatrixStructure(s->mesh, s->indexer, assembler);
  s->pattern = new Mat(assembler);
  s->mass = new Mat(assembler);
  s->indices = s->material->getMatrixIndicesPerElement(s->mesh, s->indexer, *s->pattern);
  s->material->generateMassMatrix(s->mesh, s->indexer, s->indices, *s->mass);
  s->cache = s->material->getPrecomputes(s->mesh);
  return s;
}

void odref_scene_destroy(void* p) {
  RefScene* s = (RefScene*)p;
  delete s->be;
  if (s->nm) { delete s->nm->K; delete s->nm; }
  delete s->pattern;
  delete s->mass;
  delete s->ldlt;
  delete s->ic;
  delete s;
}

int odref_dofs(void* p) { return ((RefScene*)p)->dofs; }

// sizes[0..4] = numColumns, numBlockColumn, numRemainedColumn, row-index count, value count
void odref_pattern_sizes(void* p, int* sizes) {
  Mat* m = ((RefScene*)p)->pattern;
  sizes[0] = m->numColumns;
  sizes[1] = m->numBlockColumn;
  sizes[2] = m->numRemainedColumn;
  sizes[3] = m->blockPcol[m->numBlockColumn + m->numRemainedColumn];
  sizes[4] = m->blockColumnOris[m->numBlockColumn + m->numRemainedColumn];
}

void odref_pattern(void* p, int* blockPcol, int* blockRows, int* blockColumnOris, int* elem_map) {
  RefScene* s = (RefScene*)p;
  Mat* m = s->pattern;
  int nc = m->numBlockColumn + m->numRemainedColumn;
  memcpy(blockPcol, m->blockPcol, sizeof(int) * (nc + 1));
  memcpy(blockRows, m->blockRows, sizeof(int) * m->blockPcol[nc]);
  memcpy(blockColumnOris, m->blockColumnOris, sizeof(int) * (nc + 1));
  if (elem_map) {
    for (int e = 0; e < s->n_tets; e++) {
      // entries for constrained rows/columns are left unset by the reference
      // (getMatrixIndicesPerElement writes -1 there); copy all 78
      memcpy(elem_map + 78 * e, s->indices.getElementMatIndices(e), sizeof(int) * 78);
    }
  }
}

void odref_set_displacements(void* p, const double* u) {
  RefScene* s = (RefScene*)p;
  for (int i = 0; i < s->n_nodes; i++)
    s->mesh->getVertexDisplacement(i) = Vector3(u[3 * i], u[3 * i + 1], u[3 * i + 2]);
}

void odref_get_displacements(void* p, double* u) {
  RefScene* s = (RefScene*)p;
  for (int i = 0; i < s->n_nodes; i++) {
    const Vector3& d = s->mesh->getVertexDisplacementConst(i);
    u[3 * i] = d.x; u[3 * i + 1] = d.y; u[3 * i + 2] = d.z;
  }
}

// Per-element packed 78 stiffness values and 12 nodal forces at the current
// mesh displacement, computed by the reference's element routines exactly as
// the material loops do (corotationalHyperelastic.cpp:92-98,
// invertibleHyperelastic.cpp:231-270).
void odref_element_values(void* p, double* K78, double* f12) {
  RefScene* s = (RefScene*)p;
  int ne = s->n_tets;
  if (s->mat_kind == 3) {  // the plastic material has no per-element entry; compare assembled values
    memset(K78, 0, sizeof(double) * 78 * (size_t)ne);
    memset(f12, 0, sizeof(double) * 12 * (size_t)ne);
    return;
  }
  if (s->mat_kind == 0) {
    auto* mat = (CorotationalHyperelasticMaterial*)&*s->material;
    auto* el = dynamic_cast<CorotationalHyperelasticElement*>(s->mesh->getMaterialElement(mat->type));
    const double* pre = (const double*)s->cache.getMemoryBlock();
    const double* K0 = pre;
    const double* Dm = pre + (size_t)ne * 90;
    double R[9];
    for (int e = 0; e < ne; e++) {
      el->setNodeIndices(e);
      el->generateProperOrthoMats(Dm + 9 * (size_t)e, mat->threshold, R);
      el->generateSubStiffnessMatrixNodalVirtualWorks(R, K0 + 90 * (size_t)e, K78 + 78 * (size_t)e, f12 + 12 * (size_t)e);
    }
    delete el;
  } else {
    auto* mat = (InvertibleHyperelasticMaterial*)&*s->material;
    auto* el = dynamic_cast<InvertibleHyperelasticElement*>(s->mesh->getMaterialElement(mat->type));
    const double* pre = (const double*)s->cache.getMemoryBlock();
    const double* dN = pre;
    const double* Dm = pre + (size_t)ne * 12;
    for (int e = 0; e < ne; e++) {
      double F[9], diags[3], U[9], VT[9], g[3], H[6], P[9], inv[3];
      el->setNodeIndices(e);
      el->generateDeformationGradient(Dm + 9 * (size_t)e, F);
      mat->modifiedDeformGradient(F, diags, U, VT);
      mat->getInvariants(diags, inv);
      mat->getEnergyGradient(inv, g);
      mat->getEnergyHassian(inv, H);
      mat->getPiolaKirchhoffStress(diags, U, VT, inv, g, P);
      double* k = K78 + 78 * (size_t)e;
      memset(k, 0, sizeof(double) * 78);
      el->generateSubStiffnessMatrix(dN + 12 * (size_t)e, diags, U, VT, g, H, k);
      el->generateNodalVirtualWorks(dN + 12 * (size_t)e, P, f12 + 12 * (size_t)e);
    }
    delete el;
  }
}

// values (value count) and f_int (dofs) assembled by the reference material loop
void odref_assemble(void* p, double* values, double* fint) {
  RefScene* s = (RefScene*)p;
  s->pattern->setZeros();
  memset(fint, 0, sizeof(double) * s->dofs);
  s->material->generateMatrixAndVirtualWorks(s->mesh, s->indexer, s->cache, s->indices, *s->pattern, fint);
  memcpy(values, s->pattern->values, sizeof(double) * s->pattern->getNumEntries());
}

// plastic strain state of a kind-3 scene: 9 per element (the cache block
// after 90 K0 + 9 Dm^-1 + 12 shape derivatives per element,
// corotationalPlastic.cpp:24-51)
void odref_plastic_state(void* p, double* out) {
  RefScene* s = (RefScene*)p;
  // the backward-Euler integrator evaluates the material with its own cache
  // (nonlinearImplicitBackwardEuler.h:72); the other paths use the scene's
  const double* pre = (const double*)(s->be ? s->be->materialCache.getMemoryBlock() : s->cache.getMemoryBlock());
  memcpy(out, pre + (size_t)s->n_tets * (90 + 9 + 12), sizeof(double) * 9 * (size_t)s->n_tets);
}

// The modal path's matrices (LinearNewmark::LinearNewmark,
// linearNewmark.cpp:33-38): which == 0 the Hooke stiffness
// (HookeMaterial::generateStiffnessMatrix, hooke.cpp:18-60), which == 1 the
// consistent mass (MechMaterial::generateMassMatrix into the scalar
// assembler), both the lower triangle by columns from the reference's
// assembler; returns the entry count (NULL arrays: count only).
int odref_linear_csc(void* p, int which, double youngs, double poisson, int* pcol, int* rows, double* values) {
  RefScene* s = (RefScene*)p;
  SparseMatrixAssembler a(s->dofs);
  HookeMaterial h(s->material->getDensity(), youngs, poisson);
  if (which == 0) h.generateStiffnessMatrix(s->mesh, s->indexer, a);
  else h.generateMassMatrix(s->mesh, s->indexer, a);
  int nnz = 0;
  for (int c = 0; c < s->dofs; c++) {
    if (pcol) pcol[c] = nnz;
    for (const auto& e : a.rowEntries[c]) {
      if (rows) rows[nnz] = e.first;
      if (values) values[nnz] = e.second;
      nnz++;
    }
  }
  if (pcol) pcol[s->dofs] = nnz;
  return nnz;
}

void odref_mass(void* p, double* values) {
  RefScene* s = (RefScene*)p;
  memcpy(values, s->mass->values, sizeof(double) * s->mass->getNumEntries());
}

// y += A x for A with the scene's pattern and the given values (SpMDV)
void odref_spmdv(void* p, const double* values, const double* x, double* y) {
  RefScene* s = (RefScene*)p;
  memcpy(s->pattern->values, values, sizeof(double) * s->pattern->getNumEntries());
  SpMDV(*s->pattern, x, y);
}

// CGSolver on A (scene pattern, given values); x is the warm start and result.
// precond: 0 identity, 1 Jacobi, 2 reference threshold IC(eps, relax).
// Returns the iteration count.
int odref_cg(void* p, const double* values, const double* b, double* x, double tol, int maxit,
             int precond, double eps, double relax) {
  RefScene* s = (RefScene*)p;
  memcpy(s->pattern->values, values, sizeof(double) * s->pattern->getNumEntries());
  CountingPreconditioner* cp = new CountingPreconditioner(make_preconditioner(precond, eps, relax));
  Reference<Preconditioner> pre(cp);
  CGSolver solver(tol, maxit, pre);
  solver.resetLinearSystem(s->pattern);
  solver.solveLinearSystem(b, x);
  return cp->applications - 1;
}

// InLDLTPreconditioner::Preprocess on A (scene pattern, given values) with
// (sainvEpsilon, ldltEpsilon); returns the number of stored L entries.  The
// factor is kept for odref_ldlt_get / odref_ldlt_apply.
int odref_ldlt_factor(void* p, const double* values, double sainv_eps, double ldlt_eps) {
  RefScene* s = (RefScene*)p;
  memcpy(s->pattern->values, values, sizeof(double) * s->pattern->getNumEntries());
  delete s->ldlt;
  s->ldlt = new InLDLTPreconditioner(sainv_eps, ldlt_eps);
  s->ldlt->resetPreconditionerSystem(*s->pattern);
  s->ldlt->Preprocess(*s->pattern);
  return (int)s->ldlt->values.size();
}

// the factor in the reference's storage: L columns 0..dofs-2 (pcol has
// dofs entries; rows in each column in the order they were produced) and
// the inverted diagonal (dofs entries)
void odref_ldlt_get(void* p, double* values, int* rows, int* pcol, double* inv_diag) {
  RefScene* s = (RefScene*)p;
  const InLDLTPreconditioner* f = s->ldlt;
  memcpy(values, f->values.data(), sizeof(double) * f->values.size());
  memcpy(rows, f->rows.data(), sizeof(int) * f->rows.size());
  memcpy(pcol, f->pcol.data(), sizeof(int) * f->pcol.size());
  memcpy(inv_diag, f->invDiagonal.data(), sizeof(double) * f->invDiagonal.size());
}

// result = (L D L^T)^-1 rhs with the kept factor (solvePreconditionerSystem)
void odref_ldlt_apply(void* p, const double* rhs, double* result) {
  RefScene* s = (RefScene*)p;
  s->ldlt->solvePreconditionerSystem(s->dofs, rhs, result);
}

// MeshPlaneCollisionDampingForcer (collision/penaltyDampingForcer.cpp:8-61):
// the damping-matrix values (reference layout) the forcer adds for each
// element of elems against the plane normal.x + constant = 0, with node
// velocities vel (3 per node), at the scene's current displacements.
void odref_plane_damping(void* p, const double* vel, const double* normal, double constant, double coeff, int n,
                         const int* elems, double* values) {
  RefScene* s = (RefScene*)p;
  std::vector<Vector3> v(s->n_nodes);
  for (int i = 0; i < s->n_nodes; i++) v[i] = Vector3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
  Collision::StaticPlaneShape plane;
  plane.planeNormal = Vector3(normal[0], normal[1], normal[2]);
  plane.planeConstant = constant;
  Collision::MeshPlaneCollisionDampingForcer f(coeff, s->mesh, s->indexer, v.data());
  s->pattern->setZeros();
  for (int k = 0; k < n; k++) {
    f.setCollisionPair(plane, elems[k]);
    f.addDampingMatrix(s->indices, *s->pattern);
  }
  memcpy(values, s->pattern->values, sizeof(double) * s->pattern->getNumEntries());
}

// backward Euler: clearExternalDampingForceMatrix, then the plane forcer for
// each element with the integrator's current node velocities
// (getMeshVerticesVelocities) through addExternalDampingForceMatrix
void odref_be_plane_damping(void* p, const double* normal, double constant, double coeff, int n, const int* elems) {
  RefScene* s = (RefScene*)p;
  s->be->clearExternalDampingForceMatrix();
  std::vector<Vector3> v(s->n_nodes);
  s->be->getMeshVerticesVelocities(s->indexer, s->mesh, v.data());
  Collision::StaticPlaneShape plane;
  plane.planeNormal = Vector3(normal[0], normal[1], normal[2]);
  plane.planeConstant = constant;
  Collision::MeshPlaneCollisionDampingForcer f(coeff, s->mesh, s->indexer, v.data());
  for (int k = 0; k < n; k++) {
    f.setCollisionPair(plane, elems[k]);
    s->be->addExternalDampingForceMatrix(f);
  }
}

// InCholeskyPreconditioner::Preprocess (inCholeskyPreconditioner.cpp:76-130)
// on A (scene pattern, given values) with (epsilon, relaxedScale); returns
// the number of stored L entries (diagonals included)
int odref_ic_factor(void* p, const double* values, double eps, double relax) {
  RefScene* s = (RefScene*)p;
  memcpy(s->pattern->values, values, sizeof(double) * s->pattern->getNumEntries());
  delete s->ic;
  s->ic = new InCholeskyPreconditioner(eps, relax);
  s->ic->resetPreconditionerSystem(*s->pattern);
  s->ic->Preprocess(*s->pattern);
  return (int)s->ic->values.size();
}

// the factor in the reference's storage: column c holds its diagonal first,
// then its rows below in ascending order; pcol has dofs + 1 entries
void odref_ic_get(void* p, double* values, int* rows, int* pcol) {
  RefScene* s = (RefScene*)p;
  const InCholeskyPreconditioner* f = s->ic;
  memcpy(values, f->values.data(), sizeof(double) * f->values.size());
  memcpy(rows, f->rows.data(), sizeof(int) * f->rows.size());
  memcpy(pcol, f->pcol.data(), sizeof(int) * f->pcol.size());
}

void odref_ic_apply(void* p, const double* rhs, double* result) {
  RefScene* s = (RefScene*)p;
  s->ic->solvePreconditionerSystem(s->dofs, rhs, result);
}

// MeshRelabeler::getNewLables(elementCount, nodePerElementCount,
// newNodeLables, elements) (core/meshRelabler.cpp:482-505): labels[old] =
// new node label; elems rewritten with the new labels and reordered
void odref_relabel(int n_nodes, int n_elems, int per, int* elems, int* labels) {
  MeshRelabeler r(n_nodes);
  r.getNewLables(n_elems, per, labels, elems);
}

// Loads: body force density (N/m^3) over all elements, then uniform
// tractions (Pa) over facet lists, as Forcer::addBodyForce /
// addSurfaceForceByElement do; odref_loads_clear starts a new Forcer.
void odref_loads_clear(void* p) { ((RefScene*)p)->forcer = Forcer(); }
void odref_loads_body(void* p, const double* b) {
  RefScene* s = (RefScene*)p;
  double bb[3] = {b[0], b[1], b[2]};
  s->forcer.addBodyForce(s->mesh, bb, s->indexer);
}
void odref_loads_surface(void* p, const double* t, int n, const int* facets) {
  RefScene* s = (RefScene*)p;
  double tt[3] = {t[0], t[1], t[2]};
  s->forcer.addSurfaceForceByElement(s->mesh, tt, n, facets, s->indexer);
}
void odref_loads_get(void* p, double* fext) {
  RefScene* s = (RefScene*)p;
  s->forcer.getVirtualWorks(s->dofs, s->dofs, NULL, fext);
}

// ---- backward Euler (reference integrator as shipped) ----
void odref_be_setup(void* p, double massDamp, double stiffDamp, double dt, double tol, int maxit,
                    int precond, double eps, double relax) {
  RefScene* s = (RefScene*)p;
  delete s->be;
  s->be_precond = new CountingPreconditioner(make_preconditioner(precond, eps, relax));
  Reference<Preconditioner> pre(s->be_precond);
  Reference<LinearSolver<Mat>> solver(new CGSolver(tol, maxit, pre));
  s->be = new NonlinearImplicitBackwardEuler<Mat>(s->dofs, massDamp, stiffDamp, dt, s->mesh, s->indexer,
                                                 s->material, solver);
}

void odref_be_apply_loads(void* p) {
  RefScene* s = (RefScene*)p;
  s->be->setExternalVirtualWork(s->forcer);
}

// Runs n steps, each followed by the displacement write-back a render loop
// performs (Simulator::getVertexPositions -> updateMeshVerticesDisplacements).
// Returns the total CG iteration count.
int odref_be_step(void* p, int nsteps) {
  RefScene* s = (RefScene*)p;
  int before = s->be_precond->applications;
  for (int i = 0; i < nsteps; i++) {
    s->be->runOneTimeStep();
    s->be->updateMeshVerticesDisplacements(s->indexer, s->mesh);
  }
  return s->be_precond->applications - before - nsteps;
}

void odref_be_velocity(void* p, double* v) {
  RefScene* s = (RefScene*)p;
  memcpy(v, s->be->v, sizeof(double) * s->dofs);
}

// ---- full-order Newmark restatement from reference components ----
void odref_nm_setup(void* p, double beta, double gamma, double alphaM, double betaK, double dt, int newton,
                    double tol, int maxit, int precond, double eps, double relax) {
  RefScene* s = (RefScene*)p;
  if (s->nm) { delete s->nm->K; delete s->nm; }
  RefNewmark* nm = new RefNewmark();
  int n = s->dofs;
  nm->dofs = n; nm->beta = beta; nm->gamma = gamma; nm->alphaM = alphaM; nm->betaK = betaK; nm->h = dt;
  nm->newton = newton;
  for (auto* v : {&nm->d, &nm->v, &nm->a, &nm->dp, &nm->vp, &nm->fint, &nm->fext, &nm->r, &nm->tmp, &nm->y, &nm->da})
    v->assign(n, 0.0);
  Mat::Assembler assembler(n);
  s->material->getMatrixStructure(s->mesh, s->indexer, assembler);
  nm->K = new Mat(assembler);
  nm->M = s->mass;
  s->nm_precond = new CountingPreconditioner(make_preconditioner(precond, eps, relax));
  Reference<Preconditioner> pre(s->nm_precond);
  nm->solver = new CGSolver(tol, maxit, pre);
  nm->solver->resetLinearSystem(nm->K);
  s->nm = nm;
}

void odref_nm_apply_loads(void* p) {
  RefScene* s = (RefScene*)p;
  s->forcer.getVirtualWorks(s->dofs, s->dofs, NULL, s->nm->fext.data());
}

int odref_nm_step(void* p, int nsteps) {
  RefScene* s = (RefScene*)p;
  RefNewmark* nm = s->nm;
  const int n = nm->dofs;
  const double h = nm->h, b = nm->beta, g = nm->gamma;
  const double bh2 = b * h * h, gh = g * h;
  int before = s->nm_precond->applications, solves = 0;
  for (int step = 0; step < nsteps; step++) {
    for (int i = 0; i < n; i++) {
      nm->dp[i] = nm->d[i] + h * nm->v[i] + (0.5 - b) * h * h * nm->a[i];
      nm->vp[i] = nm->v[i] + (1.0 - g) * h * nm->a[i];
    }
    for (int it = 0; it < nm->newton; it++) {
      for (int i = 0; i < n; i++) nm->tmp[i] = nm->dp[i] + bh2 * nm->a[i];
      write_free_dofs_to_mesh(s, nm->tmp.data());
      nm->K->setZeros();
      std::fill(nm->fint.begin(), nm->fint.end(), 0.0);
      s->material->generateMatrixAndVirtualWorks(s->mesh, s->indexer, s->cache, s->indices, *nm->K, nm->fint.data());
      // y = M (alpha v_k + a_k) + beta_K K v_k
      for (int i = 0; i < n; i++) {
        double vk = nm->vp[i] + gh * nm->a[i];
        nm->tmp[i] = nm->alphaM * vk + nm->a[i];
        nm->r[i] = vk;
      }
      std::fill(nm->y.begin(), nm->y.end(), 0.0);
      SpMDV(*nm->M, nm->tmp.data(), nm->y.data());
      std::fill(nm->tmp.begin(), nm->tmp.end(), 0.0);
      SpMDV(*nm->K, nm->r.data(), nm->tmp.data());
      for (int i = 0; i < n; i++)
        nm->r[i] = nm->fext[i] - nm->fint[i] - (nm->y[i] + nm->betaK * nm->tmp[i]);
      nm->K->Scale(gh * nm->betaK + bh2);
      nm->K->Add(1.0 + gh * nm->alphaM, *nm->M);
      std::fill(nm->da.begin(), nm->da.end(), 0.0);
      nm->solver->solveLinearSystem(nm->r.data(), nm->da.data());
      solves++;
      for (int i = 0; i < n; i++) nm->a[i] += nm->da[i];
    }
    for (int i = 0; i < n; i++) {
      nm->d[i] = nm->dp[i] + bh2 * nm->a[i];
      nm->v[i] = nm->vp[i] + gh * nm->a[i];
    }
    write_free_dofs_to_mesh(s, nm->d.data());
  }
  return s->nm_precond->applications - before - solves;
}

void odref_nm_state(void* p, double* d, double* v, double* a) {
  RefScene* s = (RefScene*)p;
  int n = s->dofs;
  if (d) memcpy(d, s->nm->d.data(), sizeof(double) * n);
  if (v) memcpy(v, s->nm->v.data(), sizeof(double) * n);
  if (a) memcpy(a, s->nm->a.data(), sizeof(double) * n);
}

// ---- math kernels exposed directly for known-answer tests ----
void odref_polar(const double* F, double* R, double* S) {
  double A[9];
  memcpy(A, F, sizeof(A));
  polarDecompostion3x3(A, R, S);
}
void odref_qr(const double* F, double* Q, double* R) { properQRDecompostion3x3(F, Q, R); }
void odref_eigsym(const double* tri6, double* vals, double* vecs) { eigenSym3x3(tri6, vals, vecs); }

}  // extern "C"
