"""The oracle restatement pinned against the reference's own outputs.

The golden fixtures were produced by the compiled reference
(tests/golden/make_golden.py); when the compiled reference is present
(oracle/_ref) the restatement is also compared with it live.
"""
import numpy as np
import pytest

from opendeformer_gb300 import meshgen
from oracle import restated as O
from oracle import reforacle as R

MATS = ["corotational", "neohookean", "stvk"]


def scene_from(golden, mat, case):
    p = golden(f"pattern_{case}")
    e = golden(f"elements_{mat}_{case}")
    rho, E, nu, thr = e["material"]
    s = O.OracleScene(p["X"], p["tets"], p["facets"], p["cdofs"], mat, rho, E, nu, thr)
    return s, p, e


@pytest.mark.parametrize("case", ["full", "partial"])
def test_pattern_bit_exact(golden, case):
    s, p, _ = scene_from(golden, "corotational", case)
    assert s.dofs == int(p["dofs"])
    assert np.array_equal(s.sizes, p["sizes"])
    pcol, rows, oris, emap = s.pattern()
    assert np.array_equal(pcol, p["pcol"])
    assert np.array_equal(rows, p["rows"])
    assert np.array_equal(oris, p["oris"])
    assert np.array_equal(emap, p["emap"])


@pytest.mark.parametrize("mat", MATS)
@pytest.mark.parametrize("case", ["full", "partial"])
def test_elements_and_assembly(golden, mat, case):
    s, p, e = scene_from(golden, mat, case)
    s.set_displacements(e["u"])
    K, f = s.element_values()
    # restatement follows the reference's operation order: bit-exact on x86
    # and within 1e-12 relative on any IEEE build
    np.testing.assert_allclose(K, e["K78"], rtol=0, atol=1e-12 * np.abs(e["K78"]).max())
    np.testing.assert_allclose(f, e["f12"], rtol=0, atol=1e-12 * np.abs(e["f12"]).max())
    vals, fint = s.assemble()
    np.testing.assert_allclose(vals, e["values"], rtol=0, atol=1e-12 * np.abs(e["values"]).max())
    np.testing.assert_allclose(fint, e["fint"], rtol=0, atol=1e-12 * np.abs(e["fint"]).max())
    np.testing.assert_allclose(s.mass(), e["mass"], rtol=1e-14, atol=0)
    y = s.spmdv(e["values"], e["spmv_x"])
    np.testing.assert_allclose(y, e["spmv_y"], rtol=0, atol=1e-12 * np.abs(e["spmv_y"]).max())
    g = meshgen.tet_grid(4, 2, 2, h=0.05, jitter=0.1, seed=11, tets_per_cube=6)
    fext = s.loads(body=[0, 0, -9800.0], tractions=[([0, -500.0, 0], g.face_facets(0, 1))])
    np.testing.assert_allclose(fext, e["fext"], rtol=0, atol=1e-12 * np.abs(e["fext"]).max())


@pytest.mark.parametrize("mat", MATS)
def test_jacobi_cg(golden, mat):
    s, p, e = scene_from(golden, mat, "partial")
    A = e["values"] * (1.0 / 3600.0) + e["mass"]
    x, it = s.pcg(A, e["cg_b"], tol=1e-10, maxit=2000, precond="jacobi")
    assert abs(it - int(e["cg_iters"])) <= 2
    np.testing.assert_allclose(x, e["cg_x"], rtol=0, atol=1e-8 * np.abs(e["cg_x"]).max())


@pytest.mark.parametrize("precond", ["none", "jacobi", "block_jacobi", "ic0"])
def test_preconditioners_converge_to_same_solution(golden, precond):
    s, p, e = scene_from(golden, "neohookean", "partial")
    A = e["values"] * (1.0 / 3600.0) + e["mass"]
    x, it = s.pcg(A, e["cg_b"], tol=1e-11, maxit=5000, precond=precond)
    r = e["cg_b"] - s.spmdv(A, x)
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(e["cg_b"])
    np.testing.assert_allclose(x, e["cg_x"], rtol=0, atol=1e-7 * np.abs(e["cg_x"]).max())


@pytest.mark.parametrize("mat", MATS)
def test_backward_euler(golden, mat):
    p = golden("pattern_full")
    e = golden(f"elements_{mat}_full")
    be = golden(f"be_{mat}")
    rho, E, nu, thr = e["material"]
    s = O.OracleScene(p["X"], p["tets"], p["facets"], p["cdofs"], mat, rho, E, nu, thr)
    dt, am, bk, tol = be["params"]
    s.integrator_setup(dt, am, bk, tol=tol, maxit=2000, precond="jacobi")
    s.set_fext(be["fext"])
    s.be_step(int(be["steps"]))
    u = s.displacements()
    np.testing.assert_allclose(u, be["u"], rtol=0, atol=1e-8 * np.abs(be["u"]).max())


@pytest.mark.parametrize("mat", MATS)
def test_newmark(golden, mat):
    p = golden("pattern_full")
    e = golden(f"elements_{mat}_full")
    nm = golden(f"nm_{mat}")
    rho, E, nu, thr = e["material"]
    s = O.OracleScene(p["X"], p["tets"], p["facets"], p["cdofs"], mat, rho, E, nu, thr)
    dt, am, bk, beta, gamma, newton, tol = nm["params"]
    s.integrator_setup(dt, am, bk, beta=beta, gamma=gamma, newton=int(newton), tol=tol, maxit=2000,
                       precond="jacobi")
    s.set_fext(nm["fext"])
    s.nm_step(int(nm["steps"]))
    d, v, a = s.state()
    np.testing.assert_allclose(d, nm["d"], rtol=0, atol=1e-8 * np.abs(nm["d"]).max())
    np.testing.assert_allclose(s.displacements(), nm["u"], rtol=0, atol=1e-8 * np.abs(nm["u"]).max())


def test_math_kats(golden):
    k = golden("kat_math")
    for i in range(k["F"].shape[0]):
        Rm, S = O.polar(k["F"][i])
        np.testing.assert_allclose(Rm, k["polar_R"][i], rtol=0, atol=1e-12)
        Q, Rr = O.qr(k["F"][i])
        np.testing.assert_allclose(Q, k["qr_Q"][i], rtol=0, atol=1e-12)
        vals, vecs = O.eigsym(k["tri"][i])
        scale = max(1.0, np.abs(k["eig_vals"][i]).max())
        np.testing.assert_allclose(vals, k["eig_vals"][i], rtol=0, atol=1e-12 * scale)


def test_polar_properties():
    rng = np.random.default_rng(3)
    for _ in range(300):
        F = rng.normal(size=(3, 3))
        Rm, S = O.polar(F)
        # orthogonal factor with det = sign(det F) (numerMethod.h:707-711,1004)
        assert abs(np.linalg.det(Rm) - np.sign(np.linalg.det(F))) < 1e-12
        np.testing.assert_allclose(Rm @ Rm.T, np.eye(3), atol=1e-12)
        np.testing.assert_allclose(S, S.T, atol=1e-10 * np.abs(S).max())
        assert np.linalg.eigvalsh(0.5 * (S + S.T)).min() > -1e-10
        np.testing.assert_allclose(Rm @ S, F, atol=1e-10 * np.abs(F).max())


def test_rigid_motion_gives_zero_force():
    g = meshgen.tet_grid(2, 2, 2, h=0.1, jitter=0.1, seed=5)
    th = 0.7
    Rz = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    u = g.X @ Rz.T + np.array([0.3, -0.2, 0.1]) - g.X
    for mat in MATS:
        s = O.OracleScene(g.X, g.tets, g.facets, np.zeros(0, np.int32), mat, 1000, 1e5, 0.3, 0.1)
        s.set_displacements(u)
        K, f = s.element_values()
        assert np.abs(f).max() < 1e-9 * np.abs(K).max()


def test_mass_and_body_force_totals():
    g = meshgen.tet_grid(3, 2, 2, h=0.1, jitter=0.1, seed=5)
    s = O.OracleScene(g.X, g.tets, g.facets, np.zeros(0, np.int32), "corotational", 800, 1e5, 0.3, 0.1)
    ones_x = np.zeros(s.dofs)
    ones_x[0::3] = 1.0
    total = ones_x @ s.spmdv(s.mass(), ones_x)
    assert abs(total - 800 * 0.3 * 0.2 * 0.2) < 1e-10
    f = s.loads(body=[0, 0, -9800.0])
    assert abs(f.sum() + 9800.0 * 0.3 * 0.2 * 0.2) < 1e-9


@pytest.mark.skipif(not R.available(), reason="compiled reference not built")
def test_restatement_matches_compiled_reference_live():
    g = meshgen.tet_grid(6, 3, 3, h=0.05, jitter=0.15, seed=9)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    u = np.random.default_rng(1).normal(scale=0.003, size=(g.n_nodes, 3))
    for mat in MATS:
        r = R.RefScene(g.X, g.tets, g.facets, cd, mat, 1000, 1e5, 0.45, 0.1)
        o = O.OracleScene(g.X, g.tets, g.facets, cd, mat, 1000, 1e5, 0.45, 0.1)
        for a, b in zip(r.pattern(), o.pattern()):
            assert np.array_equal(a, b)
        r.set_displacements(u)
        o.set_displacements(u)
        Kr, fr = r.element_values()
        Ko, fo = o.element_values()
        np.testing.assert_allclose(Ko, Kr, rtol=0, atol=1e-12 * np.abs(Kr).max())
        np.testing.assert_allclose(fo, fr, rtol=0, atol=1e-12 * np.abs(fr).max())


def test_plastic_restatement_matches_reference(golden):
    """Corotational plastic material: assembled values, f_int and the plastic
    strain after three evaluations at growing displacements (each evaluation
    updates the plastic strain, corotationalPlastic.cpp:129-183)."""
    d = golden("plastic")
    rho, E, nu, thr = d["material"]
    o = O.OracleScene(d["X"], d["tets"], d["facets"], d["cdofs"], "corotational_plastic", rho, E, nu, thr,
                      plastic=tuple(d["plastic_params"]))
    for k, scale in enumerate(d["scales"]):
        o.set_displacements(d["u"] * scale)
        vals, fint = o.assemble()
        assert np.abs(vals - d[f"values_{k}"]).max() <= 1e-13 * np.abs(d[f"values_{k}"]).max()
        assert np.abs(fint - d[f"fint_{k}"]).max() <= 1e-12 * np.abs(d[f"fint_{k}"]).max()
        p = o.plastic_state()
        assert np.abs(p - d[f"plastic_{k}"]).max() <= 1e-13 * np.abs(d[f"plastic_{k}"]).max()


def test_plastic_backward_euler_restatement_matches_reference(golden):
    d = golden("plastic")
    rho, E, nu, thr = d["material"]
    dt, am, bk, tol = d["be_params"]
    o = O.OracleScene(d["X"], d["tets"], d["facets"], d["cdofs"], "corotational_plastic", rho, E, nu, thr,
                      plastic=tuple(d["plastic_params"]))
    o.integrator_setup(dt, am, bk, tol=tol, maxit=2000, precond="jacobi")
    o.set_fext(d["be_fext"])
    its = o.be_step(int(d["be_steps"]))
    assert abs(its - int(d["be_iters"])) <= 0.01 * int(d["be_iters"])
    assert np.abs(o.displacements() - d["be_u"]).max() <= 1e-8 * np.abs(d["be_u"]).max()
    assert np.abs(o.plastic_state() - d["be_plastic"]).max() <= 1e-8 * np.abs(d["be_plastic"]).max()
