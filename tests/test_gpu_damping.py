"""Plane collision damping (collision/penaltyDampingForcer.cpp) on the GPU
through the C ABI.

Tolerances:
* damping values: 1e-13 relative to the largest (each element's block is
  computed with the reference's operation order and rounding; values that
  several elements share are summed colour by colour instead of in list
  order);
* backward-Euler / Newmark steps with the forcer: displacements within 1e-8.
"""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, material, rel_err

pytestmark = pytest.mark.gpu


def golden_scene(golden):
    d = golden("damping")
    s = api.Scene(ctx(), d["X"], d["tets"], d["facets"], d["cdofs"], material("corotational", *d["material"]))
    return s, d


def test_forcer_values_match_reference(golden):
    s, d = golden_scene(golden)
    s.set_displacements(d["u"])
    for k, pl in enumerate(d["planes"]):
        s.clear_damping()
        assert not np.any(s.damping_values())
        s.add_plane_damping(pl[:3], pl[3], float(d["coeff"]), d["elems"], node_velocities=d["vel"])
        assert rel_err(s.damping_values(), d[f"values_{k}"]) <= 1e-13


def test_additions_accumulate(golden):
    """Two calls add up like one call with both lists (addEntry accumulates)."""
    s, d = golden_scene(golden)
    s.set_displacements(d["u"])
    pl = d["planes"][0]
    el = d["elems"]
    s.clear_damping()
    s.add_plane_damping(pl[:3], pl[3], 50.0, el[:40], node_velocities=d["vel"])
    s.add_plane_damping(pl[:3], pl[3], 50.0, el[40:], node_velocities=d["vel"])
    assert rel_err(s.damping_values(), d["values_0"]) <= 1e-13


def test_backward_euler_with_damping_matches_reference(golden):
    s, d = golden_scene(golden)
    dt, am, bk, tol = d["be_params"]
    s.setup_integrator(api.NonlinearImplicitBackwardEuler(am, bk, dt, api.CGSolver(tol, 2000, api.JacobiPreconditioner())))
    s.set_external_forces(d["be_fext"])
    all_el = np.arange(d["tets"].shape[0])
    its = 0
    for _ in range(int(d["be_steps"])):
        s.clear_damping()
        s.add_plane_damping([0.0, 0.0, 1.0], 0.0, float(d["be_coeff"]), all_el)   # integrator velocities
        st = s.step(1)
        assert st.status == 0
        its += st.pcg_iterations
    assert abs(its - int(d["be_iters"])) <= 0.02 * int(d["be_iters"])
    assert rel_err(s.displacements(), d["be_u"]) <= 1e-8


def test_newmark_with_damping_vs_oracle():
    from oracle import restated as O
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    o.integrator_setup(1 / 60, 0.01, 0.001, newton=2, tol=1e-10, maxit=2000, precond="jacobi")
    o.set_fext(o.loads(body=[0, 0, -9800.0 * 5]))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                             api.CGSolver(1e-10, 2000, api.JacobiPreconditioner()), 2))
    s.set_loads(body=[0, 0, -9800.0 * 5])
    # a floor just under the beam's free end, tilted a little
    n = np.array([0.05, 0.0, 1.0]) / np.linalg.norm([0.05, 0.0, 1.0])
    c = 0.02
    el = np.arange(g.n_tets)
    for _ in range(10):
        o.integrator_plane_damping(n, c, 500.0, el)
        s.clear_damping()
        s.add_plane_damping(n, c, 500.0, el)
        o.nm_step(1)
        assert s.step(1).status == 0
    assert rel_err(s.displacements(), o.displacements()) <= 1e-8


def test_given_velocities_equal_integrator_velocities(golden):
    s, d = golden_scene(golden)
    dt, am, bk, tol = d["be_params"]
    s.setup_integrator(api.NonlinearImplicitBackwardEuler(am, bk, dt, api.CGSolver(tol, 2000, api.JacobiPreconditioner())))
    s.set_external_forces(d["be_fext"])
    s.step(3)
    _, v, _ = s.state()
    vel = np.zeros((s.n_nodes, 3))
    free = np.ones(3 * s.n_nodes, bool)
    free[d["cdofs"]] = False
    vel.reshape(-1)[free] = v
    all_el = np.arange(d["tets"].shape[0])
    s.clear_damping()
    s.add_plane_damping([0.0, 0.0, 1.0], 0.0, 100.0, all_el)
    a = s.damping_values()
    s.clear_damping()
    s.add_plane_damping([0.0, 0.0, 1.0], 0.0, 100.0, all_el, node_velocities=vel)
    assert np.array_equal(a, s.damping_values())


def test_bad_arguments(golden):
    s, d = golden_scene(golden)
    with pytest.raises(api.ODError):   # no integrator and no velocities
        s.add_plane_damping([0.0, 0.0, 1.0], 0.0, 1.0, [0, 1])
    with pytest.raises(api.ODError):
        s.add_plane_damping([0.0, 0.0, 1.0], 0.0, 1.0, [d["tets"].shape[0]], node_velocities=d["vel"])
    with pytest.raises(api.ODError):
        s.add_plane_damping([0.0, 0.0, float("nan")], 0.0, 1.0, [0], node_velocities=d["vel"])
