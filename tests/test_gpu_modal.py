"""The modal linear Newmark path on the GPU (od_modal_*) against the oracle.

* The Hooke stiffness assembled on the device equals the reference's
  (golden K from HookeMaterial, compared as products with seeded vectors
  through the reference's SpMDV layout) to 1e-12.
* The thick-restart Lanczos eigenpairs match ARPACK's (golden) to 1e-9 in
  lambda, the modes up to sign to 1e-7, M-orthonormal.
* After 25 LinearNewmark steps under gravity the displacements and
  velocities match the restated steps on ARPACK's modes within 1e-8.
* On a 5,184-tet grid the GPU eigenpairs match a live ARPACK solve (scipy
  eigsh in the reference's shift-invert mode on the compiled reference's
  K and M), and a 98,304-tet beam's 16 modes converge with residual below
  the tolerance.
"""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from oracle import modal as MO
from tests.gpu_util import ctx, rel_err

pytestmark = pytest.mark.gpu

CASES = ["full", "partial", "grid"]


def scene_of(z):
    rho, E, nu = z["material"]
    return api.Scene(ctx(), z["X"], z["tets"], z["facets"], z["cdofs"],
                     api.CorotationalHyperelasticMaterial(rho, E, nu, 0.1))


def modal_of(s, z, **kw):
    beta, gamma, am, bk, dt = z["step_params"]
    rho, E, nu = z["material"]
    return api.LinearNewmark(s, int(z["n_modes"]), beta, gamma, am, bk, dt, youngs=E, poisson=nu, **kw)


@pytest.mark.parametrize("case", CASES)
def test_hooke_stiffness_matches_reference(golden, case):
    z = golden(f"modal_{case}")
    s = scene_of(z)
    m = modal_of(s, z)
    K = MO.sym_from_lower_csc(z["K_pcol"], z["K_rows"], z["K_vals"], s.dofs)
    vals = m.stiffness()
    rng = np.random.default_rng(3)
    for _ in range(3):
        x = rng.normal(size=s.dofs)
        assert rel_err(s.spmdv(vals, x), K @ x) <= 1e-12
    m.close()
    s.close()


@pytest.mark.parametrize("case", CASES)
def test_modes_and_steps_match_oracle(golden, case):
    z = golden(f"modal_{case}")
    s = scene_of(z)
    s.set_loads(body=[0.0, 0.0, -9800.0])
    m = modal_of(s, z)
    lam, phi = m.modes()
    assert np.allclose(lam, z["lam"], rtol=1e-9, atol=0)
    M = MO.sym_from_lower_csc(z["M_pcol"], z["M_rows"], z["M_vals"], s.dofs)
    gram = phi @ (M @ phi.T)
    assert np.abs(gram - np.eye(lam.size)).max() < 1e-10
    overlap = np.abs(np.einsum("ij,ji->i", phi, M @ z["phi"]))
    assert np.allclose(overlap, 1.0, atol=1e-7)
    info = m.info
    assert info.max_residual <= 1e-10 and info.n_modes == lam.size
    # the scene's gravity load (the loads kernel) projected, then 25 steps
    m.setExternalVirtualWork()
    d0, v0, a0 = m.state()
    sign = np.sign(np.einsum("ij,ji->i", phi, M @ z["phi"]))
    assert np.allclose(a0 * sign, z["f_modal"], rtol=1e-9, atol=1e-12 * np.abs(z["f_modal"]).max())
    m.runOneTimeStep(int(z["steps"]))
    u = m.displacements()
    assert np.abs(u).max() > 1e-4
    assert rel_err(u, z["u"]) <= 1e-8
    assert rel_err(m.velocities(), z["vel"]) <= 1e-8
    d, v, a = m.state()
    assert rel_err(d * sign, z["d"]) <= 1e-8
    # a host force vector gives the same modal forces as the scene's loads
    m.setExternalVirtualWork(z["fext"])
    assert np.allclose(m.state()[2] * sign, z["f_modal"], rtol=1e-9, atol=1e-12 * np.abs(z["f_modal"]).max())
    m.close()
    s.close()


def test_modal_argument_checks(golden):
    z = golden("modal_full")
    s = scene_of(z)
    with pytest.raises(api.ODError):
        api.LinearNewmark(s, s.dofs, youngs=1e5, poisson=0.4)
    with pytest.raises(api.ODError):
        api.LinearNewmark(s, 4, ts=0.0, youngs=1e5, poisson=0.4)
    with pytest.raises(api.ODError):
        api.LinearNewmark(s, 4, youngs=1e5, poisson=0.5)
    with pytest.raises(api.ODError):
        api.LinearNewmark(s, 4, youngs=1e5, poisson=0.4, krylov=5)
    s.close()


def test_grid_modes_match_live_arpack():
    from oracle import reforacle as R
    if not R.available():
        pytest.skip("compiled reference not available (oracle/build_ref.py)")
    g = meshgen.tet_grid(24, 6, 6, h=0.05, jitter=0.15, seed=8)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    rho, E, nu = 1000.0, 2e5, 0.35
    rs = R.RefScene(g.X, g.tets, g.facets, cd, "corotational", rho, E, nu, 0.1)
    K, M = MO.reference_matrices(rs, E, nu)
    lam_ref, phi_ref = MO.modes(K, M, 10)
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(rho, E, nu, 0.1))
    m = api.LinearNewmark(s, 10, youngs=E, poisson=nu)
    lam, phi = m.modes()
    assert np.allclose(lam, lam_ref, rtol=1e-9, atol=0)
    gaps = np.diff(lam_ref) / lam_ref[1:]
    for i in range(10):
        # modes of well-separated eigenvalues agree up to sign
        if min(gaps[i - 1] if i > 0 else 1.0, gaps[i] if i < 9 else 1.0) > 1e-3:
            assert abs(abs(phi[i] @ (M @ phi_ref[:, i])) - 1.0) < 1e-6
    m.close()
    s.close()


def test_beam98k_modes_converge():
    g = meshgen.beam_98k()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000.0, 1e5, 0.4, 0.1))
    m = api.LinearNewmark(s, 16, youngs=1e5, poisson=0.4)
    lam, phi = m.modes()
    info = m.info
    assert info.max_residual <= 1e-10
    assert np.all(np.diff(lam) >= 0) and lam[0] > 0
    # K phi = lambda M phi through the reference-layout SpMDV
    vals = m.stiffness()
    mass = s.mass()
    for i in (0, 7, 15):
        kp = s.spmdv(vals, phi[i])
        mp = s.spmdv(mass, phi[i])
        # the residual is controlled in the shift-inverted operator's M norm
        # (relative 1e-10); in K phi - lambda M phi it grows with the
        # Krylov space's stiffness range
        assert np.abs(kp - lam[i] * mp).max() <= 1e-6 * np.abs(kp).max()
    m.close()
    s.close()
