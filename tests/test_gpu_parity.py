"""GPU parity through the C ABI against the reference's golden vectors and
the oracle restatement.

Tolerances (from the project's parity contract):
* sparsity pattern and element->value map: bit-exact;
* per-element stiffness / forces and assembled values: 1e-12 relative to the
  largest magnitude (summation order and FMA contraction differ);
* displacements after N steps: 1e-8 relative (plain FP64 path).
"""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, material, rel_err

pytestmark = pytest.mark.gpu

MATS = ["corotational", "neohookean", "stvk"]


def gpu_scene(golden, mat, case):
    p = golden(f"pattern_{case}")
    e = golden(f"elements_{mat}_{case}")
    s = api.Scene(ctx(), p["X"], p["tets"], p["facets"], p["cdofs"], material(mat, *e["material"]))
    return s, p, e


@pytest.mark.parametrize("case", ["full", "partial"])
def test_pattern_bit_exact(golden, case):
    s, p, _ = gpu_scene(golden, "corotational", case)
    assert s.dofs == int(p["dofs"])
    pcol, rows, oris, emap = s.pattern()
    assert np.array_equal(pcol, p["pcol"])
    assert np.array_equal(rows, p["rows"])
    assert np.array_equal(oris, p["oris"])
    assert np.array_equal(emap, p["emap"])


@pytest.mark.parametrize("mat", MATS)
@pytest.mark.parametrize("case", ["full", "partial"])
def test_elements_assembly_mass_loads(golden, mat, case):
    s, p, e = gpu_scene(golden, mat, case)
    s.set_displacements(e["u"])
    K, f = s.element_values()
    assert rel_err(K, e["K78"]) <= 1e-12
    assert rel_err(f, e["f12"]) <= 1e-12
    vals, fint = s.evaluate()
    assert rel_err(vals, e["values"]) <= 1e-12
    assert rel_err(fint, e["fint"]) <= 1e-12
    assert rel_err(s.mass(), e["mass"]) <= 1e-13
    y = s.spmdv(e["values"], e["spmv_x"])
    assert rel_err(y, e["spmv_y"]) <= 1e-12
    g = meshgen.tet_grid(4, 2, 2, h=0.05, jitter=0.1, seed=11, tets_per_cube=6)
    s.set_loads(body=[0, 0, -9800.0], tractions=[([0, -500.0, 0], g.face_facets(0, 1))])
    assert rel_err(s.external_forces(), e["fext"]) <= 1e-12


@pytest.mark.parametrize("mat", MATS)
@pytest.mark.parametrize("case", ["full", "partial"])
def test_jacobi_pcg_matches_reference(golden, mat, case):
    s, p, e = gpu_scene(golden, mat, case)
    A = e["values"] * (1.0 / 3600.0) + e["mass"]
    x, st = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-10, 2000, api.JacobiPreconditioner()))
    assert st.status == 0
    assert abs(st.iterations - int(e["cg_iters"])) <= 2
    assert rel_err(x, e["cg_x"]) <= 1e-8


@pytest.mark.parametrize("precond", ["none", "jacobi", "block_jacobi", "ic0"])
def test_preconditioners_converge(golden, precond):
    s, p, e = gpu_scene(golden, "neohookean", "partial")
    A = e["values"] * (1.0 / 3600.0) + e["mass"]
    x, st = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-11, 5000, api.Preconditioner(precond)))
    assert st.status == 0
    assert st.rel_residual <= 1e-10
    assert rel_err(x, e["cg_x"]) <= 1e-7


@pytest.mark.parametrize("precond", ["block_jacobi", "ic0", "ic0_natural"])
def test_preconditioner_iterations_match_oracle(golden, precond, monkeypatch):
    """Partial constraints (DOF blocks straddling nodes, a short last block).
    IC(0) factors its blocks in colour order by default and in the DOF order
    with OD_GB300_IC0_ORDER=natural; the oracle orders the same way."""
    from oracle import restated as O
    natural = precond == "ic0_natural"
    if natural:
        monkeypatch.setenv("OD_GB300_IC0_ORDER", "natural")
        precond = "ic0"
    p = golden("pattern_partial")
    e = golden("elements_stvk_partial")
    s, _, _ = gpu_scene(golden, "stvk", "partial")
    A = e["values"] * (1.0 / 3600.0) + e["mass"]
    o = O.OracleScene(p["X"], p["tets"], p["facets"], p["cdofs"], "stvk", *e["material"])
    o.set_ic0_natural(natural)
    xo, ito = o.pcg(A, e["cg_b"], tol=1e-10, maxit=2000, precond=precond)
    x, st = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-10, 2000, api.Preconditioner(precond)))
    assert abs(st.iterations - ito) <= 2
    assert rel_err(x, xo) <= 1e-8


@pytest.mark.parametrize("mat", MATS)
def test_backward_euler_matches_reference(golden, mat):
    p = golden("pattern_full")
    e = golden(f"elements_{mat}_full")
    be = golden(f"be_{mat}")
    s = api.Scene(ctx(), p["X"], p["tets"], p["facets"], p["cdofs"], material(mat, *e["material"]))
    dt, am, bk, tol = be["params"]
    s.setup_integrator(api.NonlinearImplicitBackwardEuler(am, bk, dt, api.CGSolver(tol, 2000, api.JacobiPreconditioner())))
    s.set_external_forces(be["fext"])
    st = s.step(int(be["steps"]))
    assert st.steps == int(be["steps"]) and st.status == 0
    assert rel_err(s.displacements(), be["u"]) <= 1e-8
    _, v, _ = s.state()
    assert rel_err(v, be["v"]) <= 1e-8


@pytest.mark.parametrize("mat", MATS)
def test_newmark_matches_reference_restatement(golden, mat):
    p = golden("pattern_full")
    e = golden(f"elements_{mat}_full")
    nm = golden(f"nm_{mat}")
    s = api.Scene(ctx(), p["X"], p["tets"], p["facets"], p["cdofs"], material(mat, *e["material"]))
    dt, am, bk, beta, gamma, newton, tol = nm["params"]
    s.setup_integrator(api.NewmarkIntegrator(beta, gamma, am, bk, dt, api.CGSolver(tol, 2000, api.JacobiPreconditioner()),
                                             int(newton)))
    s.set_external_forces(nm["fext"])
    s.step(int(nm["steps"]))
    d, v, a = s.state()
    assert rel_err(d, nm["d"]) <= 1e-8
    assert rel_err(s.displacements(), nm["u"]) <= 1e-8


def test_cantilever_3000_backward_euler_vs_oracle():
    from oracle import restated as O
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    o.integrator_setup(1 / 60, 0.01, 0.001, tol=1e-8, maxit=1000, precond="jacobi")
    o.set_fext(o.loads(body=[0, 0, -9800.0]))
    s.setup_integrator(api.NonlinearImplicitBackwardEuler(0.01, 0.001, 1 / 60, api.CGSolver(1e-8, 1000, api.JacobiPreconditioner())))
    s.set_loads(body=[0, 0, -9800.0])
    its_o = o.be_step(100)
    st = s.step(100)
    assert abs(st.pcg_iterations - its_o) <= 0.01 * its_o
    assert rel_err(s.displacements(), o.displacements()) <= 1e-8


@pytest.mark.parametrize("precond", ["jacobi", "block_jacobi", "ic0"])
def test_cantilever_3000_newmark_vs_oracle(precond):
    """Newmark on the soft cantilever stays within 1e-8 of the oracle for the
    first 15 steps (afterwards the large-rotation trajectory is chaotic: two
    CPU implementations of the same algorithm also separate)."""
    from oracle import restated as O
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    o.integrator_setup(1 / 60, 0.01, 0.001, newton=1, tol=1e-8, maxit=1000, precond=precond)
    o.set_fext(o.loads(body=[0, 0, -9800.0]))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                             api.CGSolver(1e-8, 1000, api.Preconditioner(precond)), 1))
    s.set_loads(body=[0, 0, -9800.0])
    o.nm_step(15)
    s.step(15)
    assert rel_err(s.displacements(), o.displacements()) <= 1e-8


def test_checkpoint_resume_is_bitwise():
    g = meshgen.tet_grid(6, 3, 3, h=0.05, jitter=0.1, seed=3)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    mat = api.InvertibleNeoHookeanMaterial(1000, 98640.0, 0.4506, 0.1)
    integ = api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 120, api.CGSolver(1e-8, 1000, api.BlockJacobiPreconditioner()), 2)
    a = api.Scene(ctx(), g.X, g.tets, g.facets, cd, mat)
    a.setup_integrator(integ)
    a.set_loads(body=[0, 0, -9800.0])
    a.step(6)
    blob = a.save()
    a.step(4)
    b = api.Scene(ctx(), g.X, g.tets, g.facets, cd, mat)
    b.setup_integrator(integ)
    b.load(blob)
    b.step(4)
    assert np.array_equal(a.displacements(), b.displacements())
    assert all(np.array_equal(x, y) for x, y in zip(a.state(), b.state()))


def test_invalid_arguments_are_rejected():
    g = meshgen.tet_grid(2, 1, 1)
    bad = g.tets.copy()
    bad[0, 0] = 10_000
    with pytest.raises(api.ODError) as ei:
        api.Scene(ctx(), g.X, bad, g.facets, [], api.CorotationalHyperelasticMaterial(1000, 1e5, 0.3, 0.1))
    assert ei.value.status == 1
    s = api.Scene(ctx(), g.X, g.tets, g.facets, [], api.CorotationalHyperelasticMaterial(1000, 1e5, 0.3, 0.1))
    with pytest.raises(api.ODError):
        s.step(1)  # no integrator yet
    with pytest.raises(api.ODError):
        s.setup_integrator(api.NonlinearImplicitBackwardEuler(0.01, 0.001, -1.0, api.CGSolver()))


@pytest.mark.parametrize("precond", ["none", "jacobi", "block_jacobi"])
def test_persistent_and_multikernel_pcg_agree(golden, precond, monkeypatch):
    """The one-launch cooperative PCG and the multi-kernel PCG are the same
    algorithm with different reduction orders: iteration counts within 3% and
    solutions within 1e-8 on this badly conditioned matrix."""
    p = golden("pattern_full")
    e = golden("elements_neohookean_full")
    A = e["values"] * (1.0 / 3600.0) + e["mass"]
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("OD_GB300_PCG_PERSISTENT", flag)
        s = api.Scene(ctx(), p["X"], p["tets"], p["facets"], p["cdofs"], material("neohookean", *e["material"]))
        out[flag] = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-10, 3000, api.Preconditioner(precond)))
    (x1, s1), (x0, s0) = out["1"], out["0"]
    assert s1.status == 0 and s0.status == 0
    assert abs(s1.iterations - s0.iterations) <= max(2, 0.03 * s0.iterations)
    assert rel_err(x1, x0) <= 1e-8


@pytest.mark.parametrize("precond", ["none", "jacobi", "block_jacobi", "ic0"])
def test_mixed_precision_solve_reaches_fp64_tolerance(golden, precond):
    """FP32 inner PCG + FP64 refinement reaches the same true-residual
    tolerance as the FP64 solve and the same solution."""
    _mixed_vs_fp64(golden, precond)


@pytest.mark.parametrize("layout", ["lower", "full"])
@pytest.mark.parametrize("precond", ["none", "block_jacobi"])
def test_mixed_precision_matrix_layouts(golden, precond, layout, monkeypatch):
    """The inner FP32 SpMV streams the lower triangle (each stored block
    applied with its transpose, the transposed products summed by reductions)
    by default, and both triangles with OD_GB300_MIXED_SPMV=full: the two
    operators are the same matrix, and both solves reach the FP64 solution."""
    if layout == "full":
        monkeypatch.setenv("OD_GB300_MIXED_SPMV", "full")
    else:
        monkeypatch.delenv("OD_GB300_MIXED_SPMV", raising=False)
    _mixed_vs_fp64(golden, precond)


def _mixed_vs_fp64(golden, precond):
    p = golden("pattern_full")
    e = golden("elements_stvk_full")
    A = e["values"] * (1.0 / 3600.0) + e["mass"]
    s = api.Scene(ctx(), p["X"], p["tets"], p["facets"], p["cdofs"], material("stvk", *e["material"]))
    x64, s64 = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-10, 3000, api.Preconditioner(precond)))
    xm, sm = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-10, 3000, api.Preconditioner(precond), precision="mixed"))
    assert sm.status == 0 and sm.refinements >= 1
    assert sm.rel_residual <= 1e-10
    assert rel_err(xm, x64) <= 1e-8


@pytest.mark.parametrize("kind,precond", [("neohookean", "block_jacobi"), ("stvk", "block_jacobi"),
                                           ("neohookean", "ic0")])
def test_mixed_precision_newmark_within_1e6_of_fp64(kind, precond):
    """20 Newmark steps (3 Newton iterations each) with the mixed solver stay
    within 1e-6 of the FP64 solver; IC(0) mixed = FP64 factor, FP32 sweeps."""
    g = meshgen.tet_grid(12, 4, 4, h=0.05, jitter=0.15, seed=2)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    mat = material(kind, 1000.0, 98640.0, 0.4506, 0.1)
    out = {}
    for prec in ("fp64", "mixed"):
        s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, mat)
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 120,
                                                 api.CGSolver(1e-10, 3000, api.Preconditioner(precond),
                                                              precision=prec), 3))
        s.set_loads(tractions=[([0.0, -500.0, 0.0], g.face_facets(0, 1))])
        s.set_traction_schedule(2.0)
        st = s.step(20)
        assert st.status == 0
        out[prec] = s.displacements()
    assert rel_err(out["mixed"], out["fp64"]) <= 1e-6


def test_relabeled_mesh_gives_the_same_motion():
    """The physics does not depend on node numbering: a shuffled beam and its
    relabeling (od_mesh_relabel) step to the same displacements, node for node."""
    g = meshgen.tet_grid(16, 4, 4, h=0.05, jitter=0.15, seed=3)
    perm = np.random.default_rng(1).permutation(g.n_nodes)          # old node -> shuffled id
    X = np.empty_like(g.X)
    X[perm] = g.X
    tets = perm[g.tets].astype(np.int32)
    facets = perm[g.facets].astype(np.int32)
    cd = meshgen.constrained_dofs_for_nodes(perm[g.face_nodes(0, 0)])
    X2, t2, f2, cd2, labels = api.relabel_mesh(X, tets, facets, cd)
    load = np.where(np.isin(facets, perm[g.face_nodes(0, 1)]).all(axis=1))[0]
    mat = api.InvertibleNeoHookeanMaterial(1000.0, 98640.0, 0.4506, 0.1)
    out = []
    for (XX, TT, FF, CC, lf) in ((X, tets, facets, cd, load), (X2, t2, f2, cd2, load)):
        s = api.Scene(ctx(), XX, TT, FF, CC, mat)
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 120,
                                                 api.CGSolver(1e-10, 2000, api.BlockJacobiPreconditioner()), 2))
        s.set_loads(body=[0.0, 0.0, -9800.0], tractions=[([0.0, -500.0, 0.0], lf)])
        assert s.step(5).status == 0
        out.append(s.displacements())
    # facet ids keep their meaning (facets are permuted node-wise, not reordered)
    assert rel_err(out[1][labels], out[0]) <= 1e-8


def test_ic0_factor_paths_agree(golden, monkeypatch):
    """The one-launch IC(0) factorisation and the one-launch-per-level one
    (OD_GB300_IC0_FACTOR=levels, kept for rows too long for the warp) give
    the same PCG: iterations within 1, solutions within 1e-10."""
    out = {}
    for mode in ("coop", "levels"):
        if mode == "levels":
            monkeypatch.setenv("OD_GB300_IC0_FACTOR", "levels")
        else:
            monkeypatch.delenv("OD_GB300_IC0_FACTOR", raising=False)
        s, p, e = gpu_scene(golden, "neohookean", "full")
        A = e["values"] * (1.0 / 3600.0) + e["mass"]
        out[mode] = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-11, 5000, api.Preconditioner("ic0")))
    (x1, s1), (x0, s0) = out["coop"], out["levels"]
    assert s1.status == 0 and s0.status == 0
    assert abs(s1.iterations - s0.iterations) <= 1
    assert rel_err(x1, x0) <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ic0_sweeps_by_colour_agree(golden, monkeypatch, precision):
    """IC(0) sweeps one launch per colour (OD_GB300_IC0_SWEEP=levels; the
    default when colours hold far more block rows than the one-launch
    sweep has warps) and the one-launch sweep apply the same factor: PCG
    iterations within 1, solutions within 1e-9 (FP64) or 1e-8 (mixed)."""
    out = {}
    for mode in ("one_launch", "levels"):
        monkeypatch.setenv("OD_GB300_IC0_SWEEP", "levels" if mode == "levels" else "one")
        s, p, e = gpu_scene(golden, "neohookean", "full")
        A = e["values"] * (1.0 / 3600.0) + e["mass"]
        out[mode] = s.pcg(A, e["cg_b"], solver=api.CGSolver(1e-11, 5000, api.Preconditioner("ic0"),
                                                             precision=precision))
    (x1, s1), (x0, s0) = out["levels"], out["one_launch"]
    assert s1.status == 0 and s0.status == 0
    assert abs(s1.iterations - s0.iterations) <= 1 + (2 if precision == "mixed" else 0)
    assert rel_err(x1, x0) <= (1e-9 if precision == "fp64" else 1e-8)


def test_degenerate_scenes_step():
    """Edge cases of the setup and assembly paths: a single tetrahedron, and
    a mesh with every DOF constrained (no free DOF, empty force lists); both
    evaluate and step with status OK, the single element matching the
    oracle's values."""
    from oracle import restated as O
    X = np.array([[0.0, 0.0, 0.0], [0.1, 0.0, 0.0], [0.0, 0.1, 0.0], [0.0, 0.0, 0.1]])
    tets = np.array([[0, 1, 2, 3]], dtype=np.int32)
    facets = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]], dtype=np.int32)
    cd = meshgen.constrained_dofs_for_nodes(np.array([0]))
    mat = api.InvertibleNeoHookeanMaterial(1000.0, 1e5, 0.45, 0.1)
    s = api.Scene(ctx(), X, tets, facets, cd, mat)
    u = np.zeros((4, 3))
    u[1:, :] = [[0.002, -0.001, 0.0], [0.0, 0.003, 0.001], [-0.001, 0.0, 0.002]]
    s.set_displacements(u)
    vals, f = s.evaluate()
    o = O.OracleScene(X, tets, facets, cd, "neohookean", 1000.0, 1e5, 0.45, 0.1)
    o.set_displacements(u)
    ov, of = o.assemble()
    assert rel_err(vals, ov) <= 1e-12 and rel_err(f, of) <= 1e-12
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                             api.CGSolver(1e-10, 100, api.BlockJacobiPreconditioner()), 2))
    s.set_loads(body=[0.0, 0.0, -9800.0])
    assert s.step(3).status == 0
    g = meshgen.tet_grid(2, 2, 2, h=0.05)
    all_dofs = np.arange(3 * g.n_nodes, dtype=np.int32)
    s2 = api.Scene(ctx(), g.X, g.tets, g.facets, all_dofs, mat)
    assert s2.dofs == 0
    v2, f2 = s2.evaluate()
    assert f2.size == 0
    s2.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                              api.CGSolver(1e-10, 100, api.BlockJacobiPreconditioner()), 1))
    assert s2.step(2).status == 0
