"""Serving (opendeformer_gb300.serving): step requests for many scenes,
continuous batching, admission by a device-memory budget (scenes built on
the library's admission thread while ticks run, or inside the tick), LRU
eviction through checkpoints.  Each scene's result through the server, in the mix and
across evictions, equals the same request sequence applied to the scene
alone (both mixed-precision solves reach 1e-10, so the tolerance on the
displacements is 1e-7 relative)."""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen, serving
from tests.gpu_util import ctx, rel_err

pytestmark = pytest.mark.gpu

POOL = [dict(dims=(6, 2, 2), h=1 / 6, kind="corotational", E=2e5, nu=0.4, seed=1),
        dict(dims=(4, 4, 3), h=1 / 4, kind="neohookean", E=5e4, nu=0.45, seed=2),
        dict(dims=(8, 3, 2), h=1 / 8, kind="corotational", E=1e6, nu=0.3, seed=3),
        dict(dims=(5, 5, 5), h=1 / 5, kind="neohookean", E=2e4, nu=0.35, seed=4),
        dict(dims=(7, 2, 3), h=1 / 7, kind="neohookean", E=3e5, nu=0.48, seed=5),
        dict(dims=(3, 3, 9), h=1 / 9, kind="corotational", E=8e4, nu=0.42, seed=6)]


def build(inst):
    g = meshgen.pool_grid(inst)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    return g.X, g.tets, g.facets, cd, g.face_facets(0, 1)


def spec(inst):
    return serving.SceneSpec(build=lambda inst=inst: build(inst),
                             material=api.Material(inst["kind"], 1000.0, inst["E"], inst["nu"], 0.1), tol=1e-10)


def requests(seed, n_per_scene):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_per_scene):
        for sid in range(len(POOL)):
            gdir = rng.normal(size=3)
            out.append(serving.StepRequest(scene=sid, arrival=0.0, dt=float(rng.uniform(1 / 120, 1 / 30)),
                                           gravity=tuple(gdir / np.linalg.norm(gdir)),
                                           traction=float(np.exp(rng.uniform(np.log(10), np.log(1000))))))
    rng.shuffle(out)
    return out


def alone(sid, reqs):
    X, tets, facets, cd, lf = build(POOL[sid])
    sp = spec(POOL[sid])
    s = api.Scene(ctx(), X, tets, facets, cd, sp.material)
    first = True
    for r in reqs:
        integ = api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, r.dt,
                                      api.CGSolver(1e-10, 5000, api.BlockJacobiPreconditioner(), precision="mixed"), 1)
        if first:
            s.setup_integrator(integ)
            first = False
        else:
            s.update_integrator(integ)
        s.set_loads(body=np.asarray(r.gravity) * 9800.0, tractions=[([0.0, -r.traction, 0.0], lf)])
        assert s.step(1).status == 0
    return s.displacements()


def run_server(reqs, budget, admission_thread=True):
    import time
    sv = serving.Server(ctx(), budget_bytes=budget, admission_thread=admission_thread)
    for inst in POOL:
        sv.add_scene(spec(inst))
    for r in reqs:
        sv.submit(r)
    done = []
    peak = 0
    t_end = time.time() + 120
    while sv.pending() and time.time() < t_end:
        done += sv.tick()
        peak = max(peak, sv.stats["resident_bytes"])
    assert not sv.pending()
    out = {sid: sv.displacements(sid) for sid in range(len(POOL))}
    stats = sv.stats
    sv.close()
    return done, out, peak, stats


@pytest.mark.parametrize("admission_thread", [True, False])
def test_server_results_equal_each_scene_alone(admission_thread):
    reqs = requests(7, 3)
    done, out, _, stats = run_server(reqs, budget=1 << 40, admission_thread=admission_thread)
    assert len(done) == len(reqs) and all(r.status == 0 for r in done)
    assert stats["evictions"] == 0
    for sid in range(len(POOL)):
        mine = [r for r in reqs if r.scene == sid]   # submission order = the scene's order
        ua = alone(sid, mine)
        assert np.abs(ua).max() > 0
        assert rel_err(out[sid], ua) <= 1e-7, sid


@pytest.mark.parametrize("admission_thread", [True, False])
def test_server_evicts_within_budget_and_restores_state(admission_thread):
    reqs = requests(11, 3)
    # about half of the pool fits
    budget = int(0.5 * 2600 * sum(6 * np.prod(i["dims"]) for i in POOL))
    done, out, peak, stats = run_server(reqs, budget=budget, admission_thread=admission_thread)
    assert stats["evictions"] > 0 and stats["restores"] > 0
    assert peak <= budget
    assert all(r.status == 0 for r in done) and len(done) == len(reqs)
    for sid in range(len(POOL)):
        mine = [r for r in reqs if r.scene == sid]
        assert rel_err(out[sid], alone(sid, mine)) <= 1e-7, sid
