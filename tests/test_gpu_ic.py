"""Threshold incomplete Cholesky with fill (solver/inCholeskyPreconditioner.cpp)
on the GPU through the C ABI.

Tolerances:
* factor (host, od_ric.cpp): bit-identical to the reference's golden arrays
  and to the oracle on the same matrix values;
* apply (device sweeps, row sums by a fixed warp butterfly instead of the
  reference's sequential sums): within 1e-12 relative to the largest entry;
* PCG with it: iteration count within 1 of the reference's, solution within
  1e-9 relative; backward-Euler steps: displacements within 1e-8.
"""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, material, rel_err

pytestmark = pytest.mark.gpu

CASES = [(m, c) for m in ("corotational", "neohookean") for c in ("full", "partial")]


def golden_scene(golden, mat, case):
    d = golden(f"ic_{mat}_{case}")
    s = api.Scene(ctx(), d["X"], d["tets"], d["facets"], d["cdofs"], material(mat, *d["material"]))
    return s, d


@pytest.mark.parametrize("mat,case", CASES)
def test_factor_bit_identical_and_apply_matches_reference(golden, mat, case):
    s, d = golden_scene(golden, mat, case)
    for k, (eps, relax) in enumerate(d["eps"]):
        lv, lr, pc = s.ic_factor(d["A"], eps, relax)
        assert np.array_equal(lv, d[f"l_values_{k}"])
        assert np.array_equal(lr, d[f"l_rows_{k}"])
        assert np.array_equal(pc, d[f"l_pcol_{k}"])
        assert rel_err(s.ic_apply(d[f"apply_r_{k}"]), d[f"apply_z_{k}"]) <= 1e-12


@pytest.mark.parametrize("mat,case", CASES)
def test_pcg_with_ic_matches_reference(golden, mat, case):
    s, d = golden_scene(golden, mat, case)
    for k, (eps, relax) in enumerate(d["eps"]):
        solver = api.CGSolver(1e-10, 2000, api.InCholeskyPreconditioner(eps, relax))
        x, st = s.pcg(d["A"], d[f"cg_b_{k}"], solver=solver)
        assert st.status == 0
        assert abs(st.iterations - int(d[f"cg_iters_{k}"])) <= 1
        assert rel_err(x, d[f"cg_x_{k}"]) <= 1e-9


@pytest.mark.parametrize("mat,case", CASES)
def test_backward_euler_with_ic_matches_reference(golden, mat, case):
    s, d = golden_scene(golden, mat, case)
    eps, relax = d["eps"][0]
    dt, am, bk, tol = d["be_params"]
    s.setup_integrator(api.NonlinearImplicitBackwardEuler(am, bk, dt, api.CGSolver(tol, 2000,
                                                                                   api.InCholeskyPreconditioner(eps, relax))))
    s.set_external_forces(d["be_fext"])
    st = s.step(int(d["be_steps"]))
    assert st.status == 0
    assert abs(st.pcg_iterations - int(d["be_iters"])) <= int(d["be_steps"])
    assert rel_err(s.displacements(), d["be_u"]) <= 1e-8


def test_cantilever_factor_and_apply_match_oracle():
    from oracle import restated as O
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    rng = np.random.default_rng(31)
    s.set_displacements(rng.normal(scale=0.002, size=(g.n_nodes, 3)))
    vals, _ = s.evaluate()
    h = 1.0 / 60.0
    A = (1 + h * 0.01) * s.mass() + (h * h + h * 0.001) * vals
    for eps, relax in [(1e-3, 0.0), (1e-2, 1.0)]:
        o.set_ic(eps, relax)
        for a, b in zip(s.ic_factor(A, eps, relax), o.ic(A)):
            assert np.array_equal(a, b)
        r = rng.normal(size=s.dofs)
        assert rel_err(s.ic_apply(r), o.ic_apply(r)) <= 1e-12


def test_cantilever_newmark_with_ic_vs_oracle():
    from oracle import restated as O
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    o.set_ic(1e-3, 0.0)
    o.integrator_setup(1 / 60, 0.01, 0.001, newton=2, tol=1e-8, maxit=1000, precond="ic")
    o.set_fext(o.loads(body=[0, 0, -9800.0]))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                             api.CGSolver(1e-8, 1000, api.InCholeskyPreconditioner(1e-3, 0.0)), 2))
    s.set_loads(body=[0, 0, -9800.0])
    its_o = o.nm_step(10)
    st = s.step(10)
    assert st.status == 0
    assert abs(st.pcg_iterations - its_o) <= 0.02 * its_o + 2
    assert rel_err(s.displacements(), o.displacements()) <= 1e-8


def test_beam_98k_apply_matches_cpu_triangular_solve():
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve_triangular
    g = meshgen.beam_98k()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    lam, mu = 3.1e5, 3.4e4
    E = mu * (3 * lam + 2 * mu) / (lam + mu)
    nu = lam / (2 * (lam + mu))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.InvertibleNeoHookeanMaterial(1000, E, nu, 0.1))
    vals, _ = s.evaluate()
    h = 1.0 / 120.0
    A = (1 + h * 0.01) * s.mass() + (h * h + h * 0.001) * vals
    lv, lr, pc = s.ic_factor(A, 1e-2, 0.0)
    n = s.dofs
    cols = np.repeat(np.arange(n), np.diff(pc))
    L = sp.csr_matrix((lv, (lr, cols)), shape=(n, n))
    r = np.random.default_rng(37).normal(size=n)
    y = spsolve_triangular(L, r, lower=True)
    z = spsolve_triangular(L.T.tocsr(), y, lower=False)
    assert rel_err(s.ic_apply(r), z) <= 1e-12
    b = np.random.default_rng(41).normal(size=n)
    x, st = s.pcg(A, b, solver=api.CGSolver(1e-8, 1000, api.InCholeskyPreconditioner(1e-2, 0.0)))
    assert st.status == 0 and st.rel_residual <= 2e-8 and st.iterations < 40


def test_ic_rejected_with_mixed_precision_and_bad_parameters():
    g = meshgen.tet_grid(3, 2, 2, jitter=0.1, seed=1)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    with pytest.raises(api.ODError):
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                                 api.CGSolver(1e-8, 100, api.InCholeskyPreconditioner(),
                                                              precision="mixed"), 1))
    with pytest.raises(api.ODError):
        s.ic_factor(np.zeros(s.n_values), -1.0, 0.0)
    with pytest.raises(api.ODError):
        s.ic_apply(np.zeros(s.dofs))   # no factor yet
    s.ldlt_factor(s.mass(), 0.1, 0.01)
    with pytest.raises(api.ODError):
        s.ic_apply(np.zeros(s.dofs))   # the loaded factor is an LDL^T one
