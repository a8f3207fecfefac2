"""Batched stepping (od_batch_*): many uneven scenes advanced together.

Every scene of a batch follows the od_step sequence (Newmark, full-order
restatement of linearNewmark.cpp:27-30, 57-79) with the mixed-precision
solver.  The checks: a batch gives each scene the same displacements as
stepping it alone (the solves of both reach the same FP64 residual
tolerance, 1e-10, so the tolerance on the displacements is 1e-7
relative), stays within 1e-6 of the plain FP64 path, does not depend on
the order or company of the scenes, and rejects scenes it cannot batch.
"""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, rel_err

pytestmark = pytest.mark.gpu

# (grid, tets per cube, material kind, E, nu, dt, body force, traction Pa)
SPECS = [
    ((6, 3, 3), 6, "corotational", 1e5, 0.45, 1 / 60, (0.0, 0.0, -9800.0), 0.0),
    ((10, 4, 4), 5, "neohookean", 98640.0, 0.4506, 1 / 120, None, 500.0),
    ((8, 5, 3), 6, "stvk", 3e5, 0.35, 1 / 90, (0.0, -9800.0, 0.0), 0.0),
    ((4, 4, 4), 5, "corotational", 2e4, 0.3, 1 / 60, (9800.0, 0.0, 0.0), 200.0),
]
MAT = {"corotational": api.CorotationalHyperelasticMaterial, "neohookean": api.InvertibleNeoHookeanMaterial,
       "stvk": api.InvertibleStVKMaterial}


def make_scene(k, precision="mixed", newton=2, precond="block_jacobi"):
    (nx, ny, nz), tpc, kind, E, nu, dt, body, trac = SPECS[k]
    g = meshgen.tet_grid(nx, ny, nz, h=0.05, jitter=0.1, seed=10 + k, tets_per_cube=tpc)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, MAT[kind](1000.0, E, nu, 0.1))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, dt,
                                             api.CGSolver(1e-10, 5000, api.Preconditioner(precond),
                                                          precision=precision), newton))
    tr = [([0.0, -trac, 0.0], g.face_facets(0, 1))] if trac else []
    s.set_loads(body=body, tractions=tr)
    if trac:
        s.set_traction_schedule(2.0)
    return s


def test_batch_matches_scenes_stepped_alone():
    alone = [make_scene(k) for k in range(len(SPECS))]
    fp64 = [make_scene(k, precision="fp64") for k in range(len(SPECS))]
    batched = [make_scene(k) for k in range(len(SPECS))]
    for s in alone + fp64:
        st = s.step(12)
        assert st.status == 0
    b = api.Batch(ctx(), batched)
    stats = b.step(12)
    assert len(stats) == len(SPECS)
    for k, st in enumerate(stats):
        assert st.status == 0 and st.steps == 12 and st.solves == 24
        assert st.max_rel_residual <= 1e-10
        ub, ua, u64 = batched[k].displacements(), alone[k].displacements(), fp64[k].displacements()
        assert np.abs(ua).max() > 0
        assert rel_err(ub, ua) <= 1e-7, k
        assert rel_err(ub, u64) <= 1e-6, k
        db, va, _ = batched[k].state()
        da, vb, _ = alone[k].state()
        assert rel_err(db, da) <= 1e-7


def test_batch_results_do_not_depend_on_company_or_order():
    a = [make_scene(k) for k in (0, 1, 2, 3)]
    b = [make_scene(k) for k in (3, 1)]
    api.Batch(ctx(), a).step(8)
    api.Batch(ctx(), b).step(8)
    assert rel_err(a[1].displacements(), b[1].displacements()) <= 1e-7
    assert rel_err(a[3].displacements(), b[0].displacements()) <= 1e-7


def test_batch_then_alone_continues_the_same_trajectory():
    s1, s2 = make_scene(1), make_scene(1)
    bt = api.Batch(ctx(), [s1, make_scene(0)])
    bt.step(5)
    s1.step(5)        # the scene keeps its state outside the batch
    s2.step(10)
    assert rel_err(s1.displacements(), s2.displacements()) <= 1e-7


@pytest.mark.parametrize("precond", ["jacobi", "none"])
def test_batch_other_preconditioners(precond):
    sc = [make_scene(k, precond=precond) for k in (0, 2)]
    al = [make_scene(k, precond=precond) for k in (0, 2)]
    stats = api.Batch(ctx(), sc).step(4)
    for k in range(2):
        al[k].step(4)
        assert stats[k].status == 0
        assert rel_err(sc[k].displacements(), al[k].displacements()) <= 1e-7


def test_batch_rejects_what_it_cannot_batch():
    with pytest.raises(RuntimeError):
        api.Batch(ctx(), [make_scene(0), make_scene(1, precision="fp64")])
    with pytest.raises(RuntimeError):
        api.Batch(ctx(), [make_scene(0, newton=1), make_scene(1, newton=2)])
    with pytest.raises(RuntimeError):
        api.Batch(ctx(), [make_scene(0), make_scene(1, precond="jacobi")])
    with pytest.raises(RuntimeError):   # mixed IC(0) steps scene by scene
        api.Batch(ctx(), [make_scene(0, precond="ic0"), make_scene(1, precond="ic0")])
    s = make_scene(0)
    with pytest.raises(RuntimeError):
        api.Batch(ctx(), [s, s])


def test_colour_scatter_assembly_matches_the_gather(monkeypatch):
    """OD_GB300_ASSEMBLY=scatter keeps the per-colour scatter (the assembly of
    meshes whose gather lists would overflow 32-bit indices) for every scene:
    the same element values summed in colour order instead of element order
    give the same steps within rounding, for a scene alone (plastic material
    included) and for a batch."""
    g = meshgen.tet_grid(10, 4, 4, h=0.05, jitter=0.1, seed=21)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    out = {}
    for mode in ("gather", "scatter"):
        if mode == "scatter":
            monkeypatch.setenv("OD_GB300_ASSEMBLY", "scatter")
        else:
            monkeypatch.delenv("OD_GB300_ASSEMBLY", raising=False)
        res = []
        for mat in (api.InvertibleNeoHookeanMaterial(1000.0, 98640.0, 0.45, 0.1),
                    api.CorotationalPlasticMaterial(1000.0, 1e5, 0.45, 1e-3, 0.5, 0.05, 0.1)):
            s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, mat)
            s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                                   api.CGSolver(1e-10, 3000, api.BlockJacobiPreconditioner()), 2))
            s.set_loads(body=[0.0, 0.0, -9800.0])
            assert s.step(8).status == 0
            res.append(s.displacements())
        batched = [make_scene(k) for k in range(len(SPECS))]
        b = api.Batch(ctx(), batched)
        st = b.step(4)
        b.close()
        assert all(x.status == 0 for x in st)
        res += [s.displacements() for s in batched]
        out[mode] = res
    for a, b in zip(out["scatter"], out["gather"]):
        assert rel_err(a, b) <= 1e-8


def test_autotune_keeps_state_and_results(tmp_path):
    """The autotuner re-solves the last Newton system with every candidate
    tile shape: the scenes' state is unchanged by it, the fastest shape stays
    set (or comes back from the cache file), and the tuned batch steps every
    scene as the untuned one does (1e-7, both solves reach 1e-10)."""
    tuned = [make_scene(k) for k in range(len(SPECS))]
    plain = [make_scene(k) for k in range(len(SPECS))]
    bt, bp = api.Batch(ctx(), tuned), api.Batch(ctx(), plain)
    with pytest.raises(api.ODError):
        bt.autotune()                       # nothing to tune on before a step
    bt.step(3)
    bp.step(3)
    before = [(s.displacements(), *s.state()) for s in tuned]
    cache = str(tmp_path / "tune.json")
    rep = bt.autotune(repeats=1, cache=cache)
    assert not rep["cached"] and rep["candidates"] == 20
    assert (rep["piece_steps"], rep["consumer_warps"]) in ((12, 12), (16, 12), (20, 12), (12, 15), (16, 15))
    assert rep["slice_cost"] in (2.0, 4.0, 8.0, 16.0)
    assert rep["best_ms"] <= rep["default_ms"]
    shape = {k: rep[k] for k in ("piece_steps", "consumer_warps", "slice_cost")}
    assert bt.tuning() == shape
    for s, b in zip(tuned, before):
        assert all(np.array_equal(x, y) for x, y in zip((s.displacements(), *s.state()), b))
    bt.step(4)
    bp.step(4)
    for k in range(len(SPECS)):
        assert rel_err(tuned[k].displacements(), plain[k].displacements()) <= 1e-7, k
    # a second batch of the same scenes finds the choice in the cache
    bt.close()
    again = api.Batch(ctx(), tuned)
    again.step(1)
    rep2 = again.autotune(cache=cache)
    assert rep2["cached"] and rep2["key"] == rep["key"]
    assert again.tuning() == shape
    with pytest.raises(api.ODError):
        again.set_tuning(14, 8.0)
    with pytest.raises(api.ODError):
        again.set_tuning(20, 8.0, consumer_warps=15)   # 15 warps of 20-step rings exceed the shared memory


def test_batch_of_many_small_scenes_after_large_ones():
    """A batch whose first scenes hold most of the work and whose tail is
    thousands of one-cube scenes: the partition of the inner solve gives no
    CTA more than its scene capacity (32) and still covers every scene, and
    each tiny scene moves as it does alone."""
    big = [make_scene(1, newton=1) for _ in range(6)]
    tiny = []
    for k in range(2400):
        g = meshgen.tet_grid(1, 1, 1, h=0.05, jitter=0.0, seed=k, tets_per_cube=6)
        cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
        s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000.0, 1e5, 0.4, 0.1))
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                                 api.CGSolver(1e-10, 5000, api.BlockJacobiPreconditioner(),
                                                              precision="mixed"), 1))
        s.set_loads(body=(0.0, 0.0, -9800.0 * (1 + k % 7)))
        tiny.append(s)
    b = api.Batch(ctx(), big + tiny)
    stats = b.step(2)
    assert all(st.status == 0 for st in stats)
    probe = tiny[-1]
    g = meshgen.tet_grid(1, 1, 1, h=0.05, jitter=0.0, seed=2399, tets_per_cube=6)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    alone = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000.0, 1e5, 0.4, 0.1))
    alone.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                                 api.CGSolver(1e-10, 5000, api.BlockJacobiPreconditioner(),
                                                              precision="mixed"), 1))
    alone.set_loads(body=(0.0, 0.0, -9800.0 * (1 + 2399 % 7)))
    assert alone.step(2).status == 0
    ua = alone.displacements()
    assert np.abs(ua).max() > 0
    assert rel_err(probe.displacements(), ua) <= 1e-7
    b.close()
    for s in big + tiny + [alone]:
        s.close()
