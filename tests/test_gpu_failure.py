"""Failure detection without a GPU fault: every device wait of the library
is bounded.  od_selftest_bounded_waits runs the production grid barrier with
one CTA that never arrives and the triangular sweeps' cooperative wait on a
value nobody writes; both waits must run out, raise the timeout flag the
library turns into OD_ERR_DEVICE_TIMEOUT, and leave the context usable."""
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx

pytestmark = pytest.mark.gpu


def test_bounded_waits_run_out_and_report():
    c = ctx()
    barrier, value = c.selftest_bounded_waits()
    assert barrier, "the grid barrier's wait did not report its timeout"
    assert value, "the sweep's value wait did not report its timeout"
    # the context still runs a step afterwards
    g = meshgen.tet_grid(4, 2, 2, h=0.05, jitter=0.1, seed=3)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(c, g.X, g.tets, g.facets, cd, api.InvertibleNeoHookeanMaterial(1000.0, 1e5, 0.45, 0.1))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                             api.CGSolver(1e-10, 500, api.BlockJacobiPreconditioner()), 2))
    s.set_loads(body=[0.0, 0.0, -9800.0])
    assert s.step(2).status == 0
