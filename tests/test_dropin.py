"""The C++ drop-in classes (include/od_gb300_dropin.hpp) compile against the
reference's own interfaces: every override matches a virtual of the
reference's Material / LinearSolver / Preconditioner / Intergrator seams
(the modal LinearNewmark's included),
and the private-member accessors resolve.  Compiled against the patched
copy of the reference headers that oracle/build_ref.py makes (skipped where
that copy is absent); nothing runs, so no GPU is needed.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")

TU = r"""
#include "od_gb300_dropin.hpp"
// instantiate every class through its reference base
void use(od_scene* s, const od_integrator_params& p, ODER::BlockedSymSpMatrix& A, const ODER::Forcer& f,
         ODER::Reference<ODER::NodeIndexer>& ix, ODER::Reference<ODER::Mesh>& mesh, ODER::Vector3* vel,
         const ODER::StaDampingForcer& damper) {
  od_dropin::GpuMaterial m(s, 1000.0, ODER::MarterialType(ODER::Marterial_Isotropic | ODER::Marterial_Invertible));
  ODER::FullOrderNonlinearMaterial<ODER::BlockedSymSpMatrix>* mat = &m;
  (void)mat;
  od_dropin::GpuCGSolver cg(s, 1e-8, 100, OD_PRECOND_BLOCK_JACOBI, &A);
  ODER::LinearSolver<ODER::BlockedSymSpMatrix>* ls = &cg;
  ls->solveLinearSystem(nullptr, nullptr);
  od_dropin::GpuInCholeskyPreconditioner ic(s, 1e-3, 0.0);
  od_dropin::GpuInLDLTPreconditioner ldlt(s, 0.1, 0.01);
  ODER::Preconditioner* pc[2] = {&ic, &ldlt};
  for (ODER::Preconditioner* q : pc) {
    q->Preprocess(A);
    q->solvePreconditionerSystem(0, nullptr, nullptr);
  }
  od_dropin::GpuIntergrator it(s, 3, p);
  ODER::Intergrator* in = &it;
  in->setExternalVirtualWork(f);
  in->addExternalDampingForceMatrix(damper);
  in->runOneTimeStep();
  in->updateMeshVerticesDisplacements(ix, mesh);
  in->getMeshVerticesVelocities(ix, mesh, vel);
  in->clearExternalDampingForceMatrix();
  od_dropin::GpuLinearNewmark lm(s, 0.25, 0.5, 8, 0.01, 0.001, 1.0 / 60, 1e5, 0.4);
  ODER::Intergrator* modal = &lm;
  modal->setExternalVirtualWork(f);
  modal->runOneTimeStep();
  modal->updateMeshVerticesDisplacements(ix, mesh);
  modal->getMeshVerticesVelocities(ix, mesh, vel);
}
"""


def test_dropin_classes_compile_against_reference_interfaces():
    if not os.path.isdir(REF_SRC):
        pytest.skip("patched reference headers not built here (oracle/build_ref.py)")
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    inc = ["-I", os.path.join(ROOT, "include")]
    for d in sorted(os.listdir(REF_SRC)):
        if os.path.isdir(os.path.join(REF_SRC, d)):
            inc += ["-I", os.path.join(REF_SRC, d)]
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "dropin_tu.cpp")
        with open(src, "w") as f:
            f.write(TU)
        r = subprocess.run([gxx, "-std=c++17", "-O0", "-DNDEBUG", "-DODER_CORE_DATASTRUCTURE_H", *inc,
                            "-c", src, "-o", os.path.join(tmp, "dropin_tu.o")],
                           capture_output=True, text=True)
    errors = [ln for ln in r.stderr.splitlines() if "error" in ln]
    assert r.returncode == 0, "\n".join(errors[:20])
