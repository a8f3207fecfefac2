"""The oracle's plane collision damping (collision/penaltyDampingForcer.cpp,
collision/intersection.cpp) pinned against the reference's own outputs: the
golden fixture (forcer values for two planes covering every clipping case,
backward-Euler steps with the forcer re-applied each step) and, where the
compiled reference is present, a live comparison on another mesh."""
import numpy as np
import pytest

from opendeformer_gb300 import meshgen
from oracle import reforacle as R
from oracle import restated as O


def oracle_scene(d):
    rho, E, nu, thr = d["material"]
    return O.OracleScene(d["X"], d["tets"], d["facets"], d["cdofs"], "corotational", rho, E, nu, thr)


def test_forcer_values_bit_identical(golden):
    d = golden("damping")
    o = oracle_scene(d)
    o.set_displacements(d["u"])
    for k, pl in enumerate(d["planes"]):
        v = o.plane_damping(d["vel"], pl[:3], pl[3], float(d["coeff"]), d["elems"])
        assert np.array_equal(v, d[f"values_{k}"])
        assert np.count_nonzero(v) > 0


def test_every_clipping_case_is_covered(golden):
    d = golden("damping")
    P = d["X"] + d["u"]
    seen = set()
    for pl in d["planes"]:
        below = ((P[d["tets"]] @ pl[:3] + pl[3]) < 1e-6).sum(axis=1)
        seen |= set(below.tolist())
    assert seen == {0, 1, 2, 3, 4}


def test_backward_euler_with_damping(golden):
    d = golden("damping")
    o = oracle_scene(d)
    dt, am, bk, tol = d["be_params"]
    o.integrator_setup(dt, am, bk, tol=tol, maxit=2000, precond="jacobi")
    o.set_fext(d["be_fext"])
    its = 0
    for _ in range(int(d["be_steps"])):
        o.integrator_plane_damping([0.0, 0.0, 1.0], 0.0, float(d["be_coeff"]), np.arange(d["tets"].shape[0]))
        its += o.be_step(1)
    assert abs(its - int(d["be_iters"])) <= int(d["be_steps"])
    assert np.abs(o.displacements() - d["be_u"]).max() <= 1e-8 * np.abs(d["be_u"]).max()


def test_no_contribution_away_from_the_plane(golden):
    d = golden("damping")
    o = oracle_scene(d)
    o.set_displacements(d["u"])
    v = o.plane_damping(d["vel"], [0.0, 0.0, 1.0], 10.0, 50.0, d["elems"])   # plane far below the mesh
    assert not np.any(v)


@pytest.mark.skipif(not R.available(), reason="compiled reference not built")
def test_restatement_matches_compiled_reference_live():
    g = meshgen.tet_grid(6, 3, 3, h=0.05, jitter=0.15, seed=9)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    r = R.RefScene(g.X, g.tets, g.facets, cd, "neohookean", 1000, 1e5, 0.45, 0.1)
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "neohookean", 1000, 1e5, 0.45, 0.1)
    rng = np.random.default_rng(12)
    u = rng.normal(scale=0.005, size=(g.n_nodes, 3))
    vel = rng.normal(size=(g.n_nodes, 3))
    r.set_displacements(u)
    o.set_displacements(u)
    n = np.array([0.3, -0.2, 1.0]) / np.linalg.norm([0.3, -0.2, 1.0])
    el = rng.permutation(g.n_tets)[: g.n_tets // 2]
    assert np.array_equal(r.plane_damping(vel, n, -0.08, 75.0, el), o.plane_damping(vel, n, -0.08, 75.0, el))
