"""The oracle's threshold incomplete Cholesky with fill
(solver/inCholeskyPreconditioner.cpp) pinned against the reference's own
outputs: the golden fixtures (factor arrays, apply, CG with it,
backward-Euler steps with it) and, where the compiled reference is present,
a live comparison on the 3000-tet cantilever."""
import numpy as np
import pytest

from opendeformer_gb300 import meshgen
from oracle import reforacle as R
from oracle import restated as O

CASES = [(m, c) for m in ("corotational", "neohookean") for c in ("full", "partial")]


def oracle_scene(d, mat):
    rho, E, nu, thr = d["material"]
    return O.OracleScene(d["X"], d["tets"], d["facets"], d["cdofs"], mat, rho, E, nu, thr)


@pytest.mark.parametrize("mat,case", CASES)
def test_ic_factor_and_apply_bit_identical(golden, mat, case):
    d = golden(f"ic_{mat}_{case}")
    o = oracle_scene(d, mat)
    for k, (eps, relax) in enumerate(d["eps"]):
        o.set_ic(eps, relax)
        lv, lr, pc = o.ic(d["A"])
        assert np.array_equal(lv, d[f"l_values_{k}"])
        assert np.array_equal(lr, d[f"l_rows_{k}"])
        assert np.array_equal(pc, d[f"l_pcol_{k}"])
        assert np.array_equal(o.ic_apply(d[f"apply_r_{k}"]), d[f"apply_z_{k}"])


@pytest.mark.parametrize("mat,case", CASES)
def test_ic_cg(golden, mat, case):
    d = golden(f"ic_{mat}_{case}")
    o = oracle_scene(d, mat)
    for k, (eps, relax) in enumerate(d["eps"]):
        o.set_ic(eps, relax)
        x, its = o.pcg(d["A"], d[f"cg_b_{k}"], tol=1e-10, maxit=2000, precond="ic")
        assert its == int(d[f"cg_iters_{k}"])
        ref = d[f"cg_x_{k}"]
        assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("mat,case", CASES)
def test_ic_backward_euler(golden, mat, case):
    d = golden(f"ic_{mat}_{case}")
    o = oracle_scene(d, mat)
    o.set_ic(*d["eps"][0])
    dt, am, bk, tol = d["be_params"]
    o.integrator_setup(dt, am, bk, tol=tol, maxit=2000, precond="ic")
    o.set_fext(d["be_fext"])
    its = o.be_step(int(d["be_steps"]))
    assert abs(its - int(d["be_iters"])) <= 1
    assert np.abs(o.displacements() - d["be_u"]).max() <= 1e-8 * np.abs(d["be_u"]).max()


def test_ic_fill_and_drop_behaviour(golden):
    """A larger epsilon keeps fewer entries and needs more iterations; every
    column stores its diagonal first and its rows below in ascending order."""
    d = golden("ic_corotational_full")
    assert d["l_values_1"].size < d["l_values_0"].size
    assert int(d["cg_iters_1"]) > int(d["cg_iters_0"])
    rows, pc = d["l_rows_0"], d["l_pcol_0"]
    for c in range(pc.size - 1):
        col = rows[pc[c]:pc[c + 1]]
        assert col[0] == c and np.all(np.diff(col) > 0)


@pytest.mark.skipif(not R.available(), reason="compiled reference not built")
def test_ic_restatement_matches_compiled_reference_live():
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    r = R.RefScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    u = np.random.default_rng(8).normal(scale=0.002, size=(g.n_nodes, 3))
    r.set_displacements(u)
    K, _ = r.assemble()
    h = 1.0 / 60.0
    A = (1 + h * 0.01) * r.mass() + (h * h + h * 0.001) * K
    for eps, relax in [(1e-3, 0.0), (1e-2, 1.0)]:
        o.set_ic(eps, relax)
        for a, b in zip(r.ic(A, eps, relax), o.ic(A)):
            assert np.array_equal(a, b)
        rhs = np.random.default_rng(9).normal(size=r.dofs)
        assert np.array_equal(r.ic_apply(rhs), o.ic_apply(rhs))
