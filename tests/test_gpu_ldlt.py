"""Incomplete LDL^T preconditioner (solver/inLDLTPreconditioner.cpp) on the
GPU through the C ABI.

Tolerances:
* factor (host, od_rif.cpp): bit-identical to the reference's golden arrays
  and to the oracle on the same matrix values;
* apply (device sweeps, row sums by a fixed warp butterfly instead of the
  reference's sequential sums): within 1e-12 relative to the largest entry;
* PCG with it: iteration count within 1 of the reference's (the GPU's dot
  products sum in another order), solution within 1e-9 relative;
* backward-Euler / Newmark steps: displacements within 1e-8 relative;
* full-size (98k-tet beam) apply: within 1e-12 of an independent CPU
  triangular solve with the same exported factor.
"""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, material, rel_err

pytestmark = pytest.mark.gpu

CASES = [(m, c) for m in ("corotational", "neohookean") for c in ("full", "partial")]


def golden_scene(golden, mat, case):
    d = golden(f"ldlt_{mat}_{case}")
    s = api.Scene(ctx(), d["X"], d["tets"], d["facets"], d["cdofs"], material(mat, *d["material"]))
    return s, d


@pytest.mark.parametrize("mat,case", CASES)
def test_factor_bit_identical_and_apply_matches_reference(golden, mat, case):
    s, d = golden_scene(golden, mat, case)
    for k, (se, le) in enumerate(d["eps"]):
        lv, lr, pc, dinv = s.ldlt_factor(d["A"], se, le)
        assert np.array_equal(lv, d[f"l_values_{k}"])
        assert np.array_equal(lr, d[f"l_rows_{k}"])
        assert np.array_equal(pc, d[f"l_pcol_{k}"])
        assert np.array_equal(dinv, d[f"inv_diag_{k}"])
        assert rel_err(s.ldlt_apply(d[f"apply_r_{k}"]), d[f"apply_z_{k}"]) <= 1e-12
        assert not np.any(s.ldlt_apply(np.zeros(s.dofs)))


@pytest.mark.parametrize("mat,case", CASES)
def test_pcg_with_ldlt_matches_reference(golden, mat, case):
    s, d = golden_scene(golden, mat, case)
    for k, (se, le) in enumerate(d["eps"]):
        solver = api.CGSolver(1e-10, 2000, api.InLDLTPreconditioner(se, le))
        x, st = s.pcg(d["A"], d[f"cg_b_{k}"], solver=solver)
        assert st.status == 0
        assert abs(st.iterations - int(d[f"cg_iters_{k}"])) <= 1
        assert rel_err(x, d[f"cg_x_{k}"]) <= 1e-9


@pytest.mark.parametrize("mat,case", CASES)
def test_backward_euler_with_ldlt_matches_reference(golden, mat, case):
    s, d = golden_scene(golden, mat, case)
    se, le = d["eps"][0]
    dt, am, bk, tol = d["be_params"]
    s.setup_integrator(api.NonlinearImplicitBackwardEuler(am, bk, dt, api.CGSolver(tol, 2000,
                                                                                   api.InLDLTPreconditioner(se, le))))
    s.set_external_forces(d["be_fext"])
    st = s.step(int(d["be_steps"]))
    assert st.status == 0
    assert abs(st.pcg_iterations - int(d["be_iters"])) <= int(d["be_steps"])
    assert rel_err(s.displacements(), d["be_u"]) <= 1e-8


def test_cantilever_factor_and_apply_match_oracle():
    """3000-tet cantilever, A from the GPU's own assembly: the product's factor
    equals the oracle's bit for bit, the apply within rounding."""
    from oracle import restated as O
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    rng = np.random.default_rng(17)
    s.set_displacements(rng.normal(scale=0.002, size=(g.n_nodes, 3)))
    vals, _ = s.evaluate()
    h = 1.0 / 60.0
    A = (1 + h * 0.01) * s.mass() + (h * h + h * 0.001) * vals
    for se, le in [(0.1, 0.01), (0.2, 0.05)]:
        o.set_ldlt(se, le)
        for a, b in zip(s.ldlt_factor(A, se, le), o.ldlt(A)):
            assert np.array_equal(a, b)
        r = rng.normal(size=s.dofs)
        assert rel_err(s.ldlt_apply(r), o.ldlt_apply(r)) <= 1e-12


def test_cantilever_newmark_with_ldlt_vs_oracle():
    from oracle import restated as O
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, "corotational", 1000, 1e5, 0.45, 0.1)
    o.set_ldlt(0.1, 0.01)
    o.integrator_setup(1 / 60, 0.01, 0.001, newton=2, tol=1e-8, maxit=1000, precond="ldlt")
    o.set_fext(o.loads(body=[0, 0, -9800.0]))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                             api.CGSolver(1e-8, 1000, api.InLDLTPreconditioner(0.1, 0.01)), 2))
    s.set_loads(body=[0, 0, -9800.0])
    its_o = o.nm_step(10)
    st = s.step(10)
    assert st.status == 0
    assert abs(st.pcg_iterations - its_o) <= 0.02 * its_o + 2
    assert rel_err(s.displacements(), o.displacements()) <= 1e-8


def test_beam_98k_apply_matches_cpu_triangular_solve():
    """Full-size sweeps (55k rows, dependency chains over a thousand rows
    deep): the device apply equals a CPU solve with the exported factor."""
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
    lv, lr, pc, dinv = s.ldlt_factor(A, 0.1, 0.01)
    n = s.dofs
    cols = np.repeat(np.arange(n - 1), np.diff(pc))   # pc: n entries, columns 0..n-2
    L = sp.csr_matrix((lv, (lr, cols)), shape=(n, n)) + sp.identity(n, format="csr")
    r = np.random.default_rng(23).normal(size=n)
    y = spsolve_triangular(L, r, lower=True, unit_diagonal=True)
    z = spsolve_triangular(L.T.tocsr(), y * dinv, lower=False, unit_diagonal=True)
    assert rel_err(s.ldlt_apply(r), z) <= 1e-12
    # one preconditioned solve on the full beam converges
    b = np.random.default_rng(29).normal(size=n)
    x, st = s.pcg(A, b, solver=api.CGSolver(1e-8, 1000, api.InLDLTPreconditioner(0.1, 0.01)))
    assert st.status == 0 and st.rel_residual <= 2e-8 and st.iterations < 60


def test_ldlt_rejected_with_mixed_precision_and_bad_bounds():
    g = meshgen.tet_grid(3, 2, 2, jitter=0.1, seed=1)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    with pytest.raises(api.ODError):
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                                 api.CGSolver(1e-8, 100, api.InLDLTPreconditioner(),
                                                              precision="mixed"), 1))
    with pytest.raises(api.ODError):
        s.ldlt_factor(np.zeros(s.n_values), -1.0, 0.01)
    with pytest.raises(api.ODError):
        s.ldlt_apply(np.zeros(s.dofs))   # no factor yet
