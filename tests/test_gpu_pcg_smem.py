"""The one-launch FP64 PCG with the matrix rows staged in shared memory
(scenes whose rows fit: every CTA's share of the blocks and block-Jacobi
rows in one CTA's shared memory) gives bit for bit the displacements of the
same kernel reading the matrix from L2 (OD_GB300_PCG_SMEM=0): the products
take the same operations in the same order."""
import os

import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx

pytestmark = pytest.mark.gpu

NH = api.InvertibleNeoHookeanMaterial(1000.0, 98640.0, 0.4506, 0.1)


def run(g, cd, precond, steps, staged):
    old = os.environ.get("OD_GB300_PCG_SMEM")
    os.environ["OD_GB300_PCG_SMEM"] = "1" if staged else "0"
    try:
        s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, NH)
    finally:
        if old is None:
            os.environ.pop("OD_GB300_PCG_SMEM", None)
        else:
            os.environ["OD_GB300_PCG_SMEM"] = old
    smem = s.info.pcg_smem_bytes
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 120,
                                             api.CGSolver(1e-8, 5000, api.Preconditioner(precond)), 3))
    s.set_loads(tractions=[([0.0, -500.0, 0.0], g.face_facets(0, 1))])
    s.set_traction_schedule(2.0)
    st = s.step(steps)
    assert st.status == 0
    u = s.displacements()
    s.close()
    return u, st.pcg_iterations, smem


@pytest.mark.parametrize("precond", ["block_jacobi", "jacobi"])
@pytest.mark.parametrize("mesh", ["beam98k", "grid"])
def test_staged_pcg_is_bitwise_the_l2_pcg(mesh, precond):
    g = meshgen.beam_98k() if mesh == "beam98k" else meshgen.tet_grid(12, 4, 4, h=0.05, jitter=0.1, seed=3)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    u1, it1, smem1 = run(g, cd, precond, 4, True)
    u0, it0, smem0 = run(g, cd, precond, 4, False)
    assert smem1 > 0 and smem0 == 0
    assert np.abs(u1).max() > 1e-5
    assert it1 == it0
    assert np.array_equal(u1, u0)
