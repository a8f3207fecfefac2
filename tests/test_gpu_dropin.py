"""The C++ drop-in classes run inside the reference's own time loop and give
the reference's results: tests/dropin/dropin_check.cpp steps one
Neo-Hookean cantilever with the reference's backward Euler as shipped, then
with GpuMaterial, GpuCGSolver, GpuInCholeskyPreconditioner and
GpuInLDLTPreconditioner swapped in, and with GpuIntergrator in place of the
integrator, with and without plane collision damping handed over the
integrator seam; every variant's displacements stay within 1e-8 of the
reference's (and the damping does change the motion).  On the 98,304-tet
beam the same program times each seam inside the reference's loop (the
material call with its host round trip of the values, the solver call, the
whole step), printed as its "seams_ms" line.  Needs the compiled reference
(oracle/_ref, made by oracle/build_ref.py) and a GPU.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from opendeformer_gb300 import meshgen

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
LIB = os.path.join(ROOT, "opendeformer_gb300", "_lib")


def run_dropin_check(g, cd, params, tol, *mode):
    """Compile tests/dropin/dropin_check.cpp against the compiled reference
    and libodgpu.so, write the mesh, run it; returns the finished process."""
    if not (os.path.isdir(os.path.join(REF, "src")) and os.path.exists(os.path.join(REF, "libodref.so"))):
        pytest.skip("compiled reference not available (oracle/build_ref.py)")
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    inc = ["-I", os.path.join(ROOT, "include")]
    for d in sorted(os.listdir(os.path.join(REF, "src"))):
        if os.path.isdir(os.path.join(REF, "src", d)):
            inc += ["-I", os.path.join(REF, "src", d)]
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "dropin_check")
        r = subprocess.run([gxx, "-std=c++17", "-O2", "-DNDEBUG", "-DODER_CORE_DATASTRUCTURE_H", "-ffp-contract=off",
                            "-w", *inc, os.path.join(ROOT, "tests", "dropin", "dropin_check.cpp"),
                            "-L", REF, "-lodref", "-L", LIB, "-lodgpu", f"-Wl,-rpath,{REF}:{LIB}", "-o", exe],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        np.ascontiguousarray(g.X, dtype=np.float64).tofile(os.path.join(tmp, "X.bin"))
        np.ascontiguousarray(g.tets, dtype=np.int32).tofile(os.path.join(tmp, "tets.bin"))
        np.ascontiguousarray(g.facets, dtype=np.int32).tofile(os.path.join(tmp, "facets.bin"))
        np.ascontiguousarray(cd, dtype=np.int32).tofile(os.path.join(tmp, "cdofs.bin"))
        with open(os.path.join(tmp, "params.txt"), "w") as f:
            # nodes tets facets cdofs | rho E nu threshold | dt alpha_m beta_k tol | max_iter steps | body force
            f.write(f"{g.n_nodes} {g.n_tets} {g.facets.shape[0]} {cd.size} " + params + "\n")
        run = subprocess.run([exe, tmp, str(tol), *mode], capture_output=True, text=True, timeout=900)
    print(run.stdout, run.stderr)
    return run


def test_dropins_match_the_reference_loop():
    g = meshgen.tet_grid(12, 3, 3, h=0.05, jitter=0.1, seed=11)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    run = run_dropin_check(g, cd, f"1000 98640 0.4506 0.1 {1 / 60} 0.01 0.001 1e-10 3000 10 0 0 -9800", 1e-8)
    assert run.returncode == 0, run.stdout + run.stderr


def test_dropin_seam_costs_on_the_beam():
    """The 98,304-tet beam, two backward Euler steps under gravity with Jacobi
    PCG to 1e-8: the drop-ins stay within 1e-6 of the reference's loop (the
    solver tolerance bounds the difference) and each seam's time per call is
    printed."""
    g = meshgen.beam_98k()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    run = run_dropin_check(g, cd, f"1000 98640 0.4506 0.1 {1 / 120} 0.01 0.001 1e-8 20000 2 0 0 -9800", 1e-6,
                           "seams")
    assert run.returncode == 0, run.stdout + run.stderr
    assert "seams_ms" in run.stdout
