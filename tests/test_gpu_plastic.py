"""Corotational plastic material on the GPU (CorotationalPlasticMaterial,
material/corotationalPlastic.cpp:53-183, element tetelement.cpp:654-729).

The plastic strain is state that changes at every evaluation of the element
forces, as in the reference; the tests replay the reference's sequence of
evaluations (golden fixture from the compiled reference) and its
backward-Euler run, compare per-element values with the restated oracle, and
check that checkpoints and batches carry the plastic strain."""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, rel_err

pytestmark = pytest.mark.gpu


def plastic_scene(d):
    rho, E, nu, thr = d["material"]
    y, c, m = d["plastic_params"]
    mat = api.CorotationalPlasticMaterial(rho, E, nu, y, c, m, thr)
    return api.Scene(ctx(), d["X"], d["tets"], d["facets"], d["cdofs"], mat)


def test_plastic_evaluations_match_reference(golden):
    d = golden("plastic")
    s = plastic_scene(d)
    for k, scale in enumerate(d["scales"]):
        s.set_displacements(d["u"] * scale)
        vals, fint = s.evaluate()
        assert rel_err(vals, d[f"values_{k}"]) <= 1e-12
        assert rel_err(fint, d[f"fint_{k}"]) <= 1e-12
        assert rel_err(s.plastic_strain(), d[f"plastic_{k}"]) <= 1e-12


def test_plastic_element_values_match_oracle(golden):
    from oracle import restated as O
    d = golden("plastic")
    rho, E, nu, thr = d["material"]
    o = O.OracleScene(d["X"], d["tets"], d["facets"], d["cdofs"], "corotational_plastic", rho, E, nu, thr,
                      plastic=tuple(d["plastic_params"]))
    s = plastic_scene(d)
    for scale in (0.2, 0.6):
        s.set_displacements(d["u"] * scale)
        o.set_displacements(d["u"] * scale)
        K, f = s.element_values()
        Ko, fo = o.element_values()
        assert rel_err(K, Ko) <= 1e-12
        assert rel_err(f, fo) <= 1e-12
        assert rel_err(s.plastic_strain(), o.plastic_state()) <= 1e-12


def test_plastic_backward_euler_matches_reference(golden):
    d = golden("plastic")
    dt, am, bk, tol = d["be_params"]
    s = plastic_scene(d)
    s.setup_integrator(api.NonlinearImplicitBackwardEuler(am, bk, dt, api.CGSolver(tol, 2000,
                                                                                  api.JacobiPreconditioner())))
    s.set_external_forces(d["be_fext"])
    st = s.step(int(d["be_steps"]))
    assert st.status == 0
    assert abs(st.pcg_iterations - int(d["be_iters"])) <= 0.01 * int(d["be_iters"])
    assert rel_err(s.displacements(), d["be_u"]) <= 1e-8
    assert rel_err(s.plastic_strain(), d["be_plastic"]) <= 1e-8


def test_plastic_checkpoint_carries_plastic_strain():
    g = meshgen.tet_grid(6, 2, 2, h=0.05, jitter=0.1, seed=5)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    mat = api.CorotationalPlasticMaterial(1000.0, 1e5, 0.45, 2e-3, 0.5, 0.02, 0.1)
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, mat)
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                             api.CGSolver(1e-10, 2000, api.BlockJacobiPreconditioner()), 2))
    s.set_loads(body=[0.0, 0.0, -9800.0 * 4])
    s.step(5)
    blob = s.save()
    p5 = s.plastic_strain()
    assert np.abs(p5).max() > 0
    s.step(3)
    u8, p8 = s.displacements(), s.plastic_strain()
    s.load(blob)
    assert np.array_equal(s.plastic_strain(), p5)
    s.step(3)
    assert np.array_equal(s.displacements(), u8)
    assert np.array_equal(s.plastic_strain(), p8)


def test_plastic_scene_in_batch_matches_alone():
    g = meshgen.tet_grid(6, 2, 2, h=0.05, jitter=0.1, seed=5)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    g2 = meshgen.tet_grid(5, 3, 2, h=0.05, jitter=0.1, seed=6, tets_per_cube=5)
    cd2 = meshgen.constrained_dofs_for_nodes(g2.face_nodes(0, 0))

    def scenes():
        a = api.Scene(ctx(), g.X, g.tets, g.facets, cd,
                      api.CorotationalPlasticMaterial(1000.0, 1e5, 0.45, 2e-3, 0.5, 0.02, 0.1))
        b = api.Scene(ctx(), g2.X, g2.tets, g2.facets, cd2, api.InvertibleNeoHookeanMaterial(1000.0, 5e4, 0.4, 0.1))
        for s in (a, b):
            s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                                     api.CGSolver(1e-10, 2000, api.BlockJacobiPreconditioner(),
                                                                  precision="mixed"), 1))
            s.set_loads(body=[0.0, 0.0, -9800.0 * 4])
        return a, b

    a1, b1 = scenes()
    a2, b2 = scenes()
    api.Batch(ctx(), [a1, b1]).step(6)
    a2.step(6)
    b2.step(6)
    assert rel_err(a1.displacements(), a2.displacements()) <= 1e-7
    assert rel_err(a1.plastic_strain(), a2.plastic_strain()) <= 1e-7
    assert rel_err(b1.displacements(), b2.displacements()) <= 1e-7
