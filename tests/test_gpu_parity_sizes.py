"""Displacement parity at the benchmarked sizes, against the oracle.

* The 98,304-tet Neo-Hookean beam (64x16x16 cubes x 6 tets, jitter 0.15 h),
  Newmark dt 1/120 s with 3 Newton iterations per step, a 500 Pa traction
  along -y scaled by sin(2 pi 2 t) and re-evaluated on the deformed facets
  every step, PCG to 1e-8: the plain FP64 path with block-Jacobi and with
  IC(0) after several steps within 1e-8 relative of the oracle's
  restatement of the same steps.
* The 2,621,440-tet Neo-Hookean block (128x64x64 cubes x 5 tets, jitter
  0.2 h, bottom fixed, a seeded 20% of the top nodes prescribed to
  -0.05 height), one Newmark step with one Newton iteration, block-Jacobi
  PCG to 1e-10: the mixed-precision path within 1e-6 relative of the oracle
  (the precision form's error bound) and the FP64 path within 1e-8.

The oracle is single-threaded: about 0.6 s per beam step and 30 s per block
step on one core, so the block case runs one step.
"""
import math

import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, rel_err

pytestmark = pytest.mark.gpu

NH_MU, NH_LAMBDA = 3.4e4, 3.1e5
NH_E = NH_MU * (3 * NH_LAMBDA + 2 * NH_MU) / (NH_LAMBDA + NH_MU)
NH_NU = NH_LAMBDA / (2 * (NH_LAMBDA + NH_MU))
BEAM_DT, BEAM_FREQ, BEAM_TRACTION = 1 / 120, 2.0, 500.0


def beam_oracle_steps(g, cd, precond, steps):
    from oracle import restated as O
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "neohookean", 1000.0, NH_E, NH_NU, 0.1)
    o.integrator_setup(BEAM_DT, 0.01, 0.001, newton=3, tol=1e-8, maxit=5000, precond=precond)
    facets = g.face_facets(0, 1)
    t, iters = 0.0, 0
    for _ in range(steps):
        t += BEAM_DT
        scale = math.sin(2 * math.pi * BEAM_FREQ * t)
        o.set_fext(o.loads(tractions=[(np.array([0.0, -BEAM_TRACTION, 0.0]) * scale, facets)]))
        iters += o.nm_step(1)
    u = o.displacements()
    o.close()
    return u, iters


@pytest.mark.parametrize("precond,steps", [("block_jacobi", 10), ("ic0", 5)])
def test_beam98k_newmark_matches_oracle(precond, steps):
    g = meshgen.beam_98k()
    assert g.n_tets == 98304
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.InvertibleNeoHookeanMaterial(1000.0, NH_E, NH_NU, 0.1))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, BEAM_DT,
                                             api.CGSolver(1e-8, 5000, api.Preconditioner(precond)), 3))
    s.set_loads(tractions=[([0.0, -BEAM_TRACTION, 0.0], g.face_facets(0, 1))])
    s.set_traction_schedule(BEAM_FREQ)
    st = s.step(steps)
    assert st.status == 0
    ug = s.displacements()
    s.close()
    uo, iters_o = beam_oracle_steps(g, cd, precond, steps)
    assert np.abs(uo).max() > 1e-4  # the beam has moved
    assert abs(st.pcg_iterations - iters_o) <= 0.03 * iters_o + 2
    assert rel_err(ug, uo) <= 1e-8


@pytest.fixture(scope="module")
def block_case():
    g = meshgen.block_2m6()
    bottom, top = g.face_nodes(2, 0), g.face_nodes(2, 1)
    rng = np.random.default_rng(4)
    presc = np.sort(rng.choice(top, size=int(0.2 * top.size), replace=False))
    cd = meshgen.constrained_dofs_for_nodes(np.concatenate([bottom, presc]))
    u0 = np.zeros((g.n_nodes, 3))
    u0[presc, 2] = -0.05 * g.dims[2] * g.h
    from oracle import restated as O
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "neohookean", 1000.0, NH_E, NH_NU, 0.1)
    o.set_displacements(u0)
    o.integrator_setup(1 / 120, 0.01, 0.001, newton=1, tol=1e-10, maxit=20000, precond="block_jacobi")
    o.nm_step(1)
    uo = o.displacements()
    o.close()
    return g, cd, u0, uo


@pytest.mark.parametrize("precision,bound", [("mixed", 1e-6), ("fp64", 1e-8)])
def test_block2m6_one_step_matches_oracle(block_case, precision, bound):
    g, cd, u0, uo = block_case
    assert g.n_tets == 2621440
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.InvertibleNeoHookeanMaterial(1000.0, NH_E, NH_NU, 0.1))
    s.set_displacements(u0)
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 120,
                                             api.CGSolver(1e-10, 20000, api.BlockJacobiPreconditioner(),
                                                          precision=precision), 1))
    st = s.step(1)
    assert st.status == 0
    ug = s.displacements()
    s.close()
    assert rel_err(ug, uo) <= bound
