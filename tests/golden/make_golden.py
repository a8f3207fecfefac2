"""Generate the golden fixtures from the compiled reference.

Run from the repository root after ``python oracle/build_ref.py``:

    python tests/golden/make_golden.py

Every array in ``tests/golden/*.npz`` is produced by the reference's own C++
code (``oracle/_ref/libodref.so``) on small seeded meshes from
``opendeformer_gb300.meshgen``; the tests compare the oracle restatement and
the GPU path against them.  Cases:

* ``pattern_*``: pattern arrays and element->value map, including a case with
  partial-axis constraints (DOF blocks straddling nodes, a degenerate last row
  block and scalar tail columns since the DOF count is not a multiple of 3);
* ``elements_<material>``: per-element 78 stiffness + 12 force values,
  assembled values, f_int and mass at a seeded displacement field;
* ``be_<material>``: displacements after backward-Euler steps (Jacobi CG);
* ``nm_<material>``: displacements after Newmark steps (restated integrator on
  reference components, Jacobi CG);
* ``kat_math``: polar decomposition, Givens QR and symmetric eigensolve on
  random and near-singular matrices;
* ``plastic``: the corotational plastic material: assembled values, f_int and
  plastic strain after three evaluations at growing displacements (each
  evaluation updates the plastic strain), and backward-Euler steps;
* ``ldlt_<material>_<constraints>``: InLDLTPreconditioner: the factor (L
  values, rows, pcol, inverted diagonal) of A = K/3600 + M at two drop-bound
  pairs, its apply on a seeded vector, CG with it, and backward-Euler steps
  preconditioned by it;
* ``ic_<material>_<constraints>``: InCholeskyPreconditioner (threshold IC
  with fill): the factor (values, rows, pcol) of A = K/3600 + M at two
  (epsilon, relaxedScale) pairs, its apply, CG with it, and backward-Euler
  steps preconditioned by it;
* ``damping``: MeshPlaneCollisionDampingForcer: damping values against two
  planes (a tilted one cutting elements with 0-3 vertices below it, a
  horizontal one with whole elements below it), with a repeated element,
  and backward-Euler steps with the forcer re-applied every step.

* ``modal_<case>``: the modal linear Newmark path: Hooke stiffness and
  consistent mass (scalar CSC from the reference's assembler), the lowest
  eigenpairs (ARPACK shift-invert at 0 through scipy's eigsh: the
  reference's ARPACK++/SuperLU binaries cannot run here), modal forces of a
  gravity load and the reduced state and displacements after restated
  LinearNewmark steps (oracle/modal.py).

``--only NAME`` writes one group (plastic, ldlt, ic, damping or modal; the
full run writes all).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from opendeformer_gb300 import meshgen  # noqa: E402
from oracle import reforacle as R  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

MATS = {"corotational": (1000.0, 1e5, 0.45, 0.1),
        "neohookean": (1000.0, 98640.0, 0.4506, 0.1),
        "stvk": (1000.0, 1e5, 0.40, 0.1)}


def small_mesh():
    return meshgen.tet_grid(4, 2, 2, h=0.05, jitter=0.1, seed=11, tets_per_cube=6)


def partial_constraints(g):
    """x=0 face fully fixed plus single-axis constraints on three more nodes."""
    cd = list(meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0)))
    top = g.face_nodes(2, 1)
    cd += [3 * int(top[3]) + 1, 3 * int(top[6]) + 2, 3 * int(top[7]) + 0, 3 * int(top[7]) + 2]
    return np.array(sorted(set(cd)), np.int32)


def save(name, **arrays):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrays)


PLASTIC = (1000.0, 1e5, 0.45, 0.1)              # rho, E, nu, compressing threshold
PLASTIC_PARAMS = (2e-3, 0.5, 0.02)              # yield criterion, creep ratio, max plastic strain
PLASTIC_SCALES = (0.1, 0.3, 1.0)                # displacement scales of the three evaluations


def plastic_case():
    g = small_mesh()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    rho, E, nu, thr = PLASTIC
    s = R.RefScene(g.X, g.tets, g.facets, cd, "corotational_plastic", rho, E, nu, thr, plastic=PLASTIC_PARAMS)
    rng = np.random.default_rng(99)
    u = rng.normal(scale=0.0015, size=(g.n_nodes, 3))
    u[g.face_nodes(0, 0)] = 0.0
    out = {}
    for k, scale in enumerate(PLASTIC_SCALES):
        s.set_displacements(u * scale)
        vals, fint = s.assemble()
        out[f"values_{k}"] = vals
        out[f"fint_{k}"] = fint
        out[f"plastic_{k}"] = s.plastic_state()
    s = R.RefScene(g.X, g.tets, g.facets, cd, "corotational_plastic", rho, E, nu, thr, plastic=PLASTIC_PARAMS)
    s.be_setup(1.0 / 60.0, 0.01, 0.001, tol=1e-10, maxit=2000, precond="jacobi")
    fext = s.loads(body=[0.0, 0.0, -9800.0 * 20])
    s.be_apply_loads()
    iters = s.be_step(20)
    save("plastic", X=g.X, tets=g.tets, facets=g.facets, cdofs=cd, u=u, scales=np.array(PLASTIC_SCALES),
         material=np.array(PLASTIC), plastic_params=np.array(PLASTIC_PARAMS), be_fext=fext,
         be_u=s.displacements(), be_v=s.be_velocity(), be_plastic=s.plastic_state(), be_steps=20, be_iters=iters,
         be_params=np.array([1.0 / 60.0, 0.01, 0.001, 1e-10]), **out)


LDLT_EPS = ((0.1, 0.01), (0.05, 0.005))         # (sainvEpsilon, ldltEpsilon) pairs


def ldlt_cases():
    g = small_mesh()
    cases = {"full": meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0)),
             "partial": partial_constraints(g)}
    rng = np.random.default_rng(321)
    u = rng.normal(scale=0.002, size=(g.n_nodes, 3))
    for mat in ("corotational", "neohookean"):
        rho, E, nu, thr = MATS[mat]
        for cname, cd in cases.items():
            s = R.RefScene(g.X, g.tets, g.facets, cd, mat, rho, E, nu, thr)
            s.set_displacements(u)
            vals, _ = s.assemble()
            A = vals * (1.0 / 3600.0) + s.mass()
            out = {}
            for k, (se, le) in enumerate(LDLT_EPS):
                lv, lr, pc, dinv = s.ldlt(A, se, le)
                r = rng.normal(size=s.dofs)
                out.update({f"l_values_{k}": lv, f"l_rows_{k}": lr, f"l_pcol_{k}": pc, f"inv_diag_{k}": dinv,
                            f"apply_r_{k}": r, f"apply_z_{k}": s.ldlt_apply(r)})
                b = rng.normal(size=s.dofs)
                x, its = s.cg(A, b, tol=1e-10, maxit=2000, precond="ldlt", eps=se, relax=le)
                out.update({f"cg_b_{k}": b, f"cg_x_{k}": x, f"cg_iters_{k}": its})
            se, le = LDLT_EPS[0]
            s = R.RefScene(g.X, g.tets, g.facets, cd, mat, rho, E, nu, thr)
            s.be_setup(1.0 / 60.0, 0.01, 0.001, tol=1e-10, maxit=2000, precond="ldlt", eps=se, relax=le)
            fext = s.loads(body=[0.0, 0.0, -9800.0])
            s.be_apply_loads()
            iters = s.be_step(10)
            save(f"ldlt_{mat}_{cname}", X=g.X, tets=g.tets, facets=g.facets, cdofs=cd, u=u, A=A,
                 eps=np.array(LDLT_EPS), material=np.array([rho, E, nu, thr]), be_fext=fext,
                 be_u=s.displacements(), be_v=s.be_velocity(), be_steps=10, be_iters=iters,
                 be_params=np.array([1.0 / 60.0, 0.01, 0.001, 1e-10]), **out)


IC_EPS = ((1e-3, 0.0), (1e-2, 0.5))              # (epsilon, relaxedScale) pairs


def ic_cases():
    g = small_mesh()
    cases = {"full": meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0)),
             "partial": partial_constraints(g)}
    rng = np.random.default_rng(654)
    u = rng.normal(scale=0.002, size=(g.n_nodes, 3))
    for mat in ("corotational", "neohookean"):
        rho, E, nu, thr = MATS[mat]
        for cname, cd in cases.items():
            s = R.RefScene(g.X, g.tets, g.facets, cd, mat, rho, E, nu, thr)
            s.set_displacements(u)
            vals, _ = s.assemble()
            A = vals * (1.0 / 3600.0) + s.mass()
            out = {}
            for k, (eps, relax) in enumerate(IC_EPS):
                lv, lr, pc = s.ic(A, eps, relax)
                r = rng.normal(size=s.dofs)
                out.update({f"l_values_{k}": lv, f"l_rows_{k}": lr, f"l_pcol_{k}": pc,
                            f"apply_r_{k}": r, f"apply_z_{k}": s.ic_apply(r)})
                b = rng.normal(size=s.dofs)
                x, its = s.cg(A, b, tol=1e-10, maxit=2000, precond="ic", eps=eps, relax=relax)
                out.update({f"cg_b_{k}": b, f"cg_x_{k}": x, f"cg_iters_{k}": its})
            eps, relax = IC_EPS[0]
            s = R.RefScene(g.X, g.tets, g.facets, cd, mat, rho, E, nu, thr)
            s.be_setup(1.0 / 60.0, 0.01, 0.001, tol=1e-10, maxit=2000, precond="ic", eps=eps, relax=relax)
            fext = s.loads(body=[0.0, 0.0, -9800.0])
            s.be_apply_loads()
            iters = s.be_step(10)
            save(f"ic_{mat}_{cname}", X=g.X, tets=g.tets, facets=g.facets, cdofs=cd, u=u, A=A,
                 eps=np.array(IC_EPS), material=np.array([rho, E, nu, thr]), be_fext=fext,
                 be_u=s.displacements(), be_v=s.be_velocity(), be_steps=10, be_iters=iters,
                 be_params=np.array([1.0 / 60.0, 0.01, 0.001, 1e-10]), **out)


DAMP_PLANES = ((0.1, 0.2, 1.0, -0.05), (0.0, 0.0, 1.0, -0.07))   # normal (normalised), constant
DAMP_COEFF = 50.0
DAMP_BE = (2000.0, 15)          # coefficient, steps (plane z = 0, all elements, 20 g)


def damping_case():
    g = small_mesh()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    rho, E, nu, thr = MATS["corotational"]
    s = R.RefScene(g.X, g.tets, g.facets, cd, "corotational", rho, E, nu, thr)
    rng = np.random.default_rng(77)
    u = rng.normal(scale=0.004, size=(g.n_nodes, 3))
    vel = rng.normal(size=(g.n_nodes, 3))
    s.set_displacements(u)
    elems = np.concatenate([np.arange(g.n_tets), [3, 3, 17]]).astype(np.int32)
    planes = []
    out = {}
    for k, (a, b, c, const) in enumerate(DAMP_PLANES):
        nrm = np.array([a, b, c]) / np.linalg.norm([a, b, c])
        planes.append(list(nrm) + [const])
        out[f"values_{k}"] = s.plane_damping(vel, nrm, const, DAMP_COEFF, elems)
    s = R.RefScene(g.X, g.tets, g.facets, cd, "corotational", rho, E, nu, thr)
    s.be_setup(1.0 / 60.0, 0.01, 0.001, tol=1e-10, maxit=2000, precond="jacobi")
    fext = s.loads(body=[0.0, 0.0, -9800.0 * 20])
    s.be_apply_loads()
    coeff, steps = DAMP_BE
    iters = 0
    for _ in range(steps):
        s.be_plane_damping([0.0, 0.0, 1.0], 0.0, coeff, np.arange(g.n_tets))
        iters += s.be_step(1)
    save("damping", X=g.X, tets=g.tets, facets=g.facets, cdofs=cd, u=u, vel=vel, elems=elems,
         planes=np.array(planes), coeff=DAMP_COEFF, material=np.array([rho, E, nu, thr]), be_fext=fext,
         be_u=s.displacements(), be_v=s.be_velocity(), be_steps=steps, be_iters=iters, be_coeff=coeff,
         be_params=np.array([1.0 / 60.0, 0.01, 0.001, 1e-10]), **out)


MODAL = (1000.0, 1e5, 0.4)                       # rho, E, nu of the Hooke material
MODAL_STEP = (0.25, 0.5, 0.01, 0.001, 1.0 / 60.0)  # beta, gamma, massDamp, stiffDamp, dt
MODAL_STEPS = 25


def modal_cases():
    """LinearNewmark: K (Hooke) and M from the reference's scalar assembler,
    the lowest eigenpairs by ARPACK in the reference's shift-invert mode
    (scipy's eigsh, the reference links ARPACK++/ARPACK/SuperLU binaries that
    cannot run here), modal forces of a gravity load through the reference's
    Forcer, and the restated per-mode Newmark steps (oracle/modal.py)."""
    from oracle import modal as MO
    rho, E, nu = MODAL
    beta, gamma, am, bk, dt = MODAL_STEP
    small = small_mesh()
    grid = meshgen.tet_grid(8, 3, 3, h=0.05, jitter=0.1, seed=5, tets_per_cube=6)
    cases = {"full": (small, meshgen.constrained_dofs_for_nodes(small.face_nodes(0, 0)), 6),
             "partial": (small, partial_constraints(small), 6),
             "grid": (grid, meshgen.constrained_dofs_for_nodes(grid.face_nodes(0, 0)), 12)}
    for cname, (g, cd, r) in cases.items():
        s = R.RefScene(g.X, g.tets, g.facets, cd, "corotational", rho, E, nu, 0.1)
        kp, kr, kv = s.linear_csc("K", E, nu)
        mp, mr, mv = s.linear_csc("M", E, nu)
        K = MO.sym_from_lower_csc(kp, kr, kv, s.dofs)
        M = MO.sym_from_lower_csc(mp, mr, mv, s.dofs)
        lam, phi = MO.modes(K, M, r)
        fext = s.loads(body=[0.0, 0.0, -9800.0])
        o = MO.LinearNewmarkOracle(lam, phi, beta, gamma, am, bk, dt)
        o.set_external(fext)
        f_modal = o.f.copy()
        o.step(MODAL_STEPS)
        u = MO.to_nodes(o.full_order(), g.n_nodes, cd)
        vel = MO.to_nodes(o.full_order(o.v), g.n_nodes, cd)
        save(f"modal_{cname}", X=g.X, tets=g.tets, facets=g.facets, cdofs=cd, material=np.array(MODAL),
             step_params=np.array(MODAL_STEP), steps=MODAL_STEPS, n_modes=r, K_pcol=kp, K_rows=kr, K_vals=kv,
             M_pcol=mp, M_rows=mr, M_vals=mv, lam=lam, phi=phi, fext=fext, f_modal=f_modal, d=o.d, v=o.v,
             a=o.a, u=u, vel=vel)


def main():
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only == "ic":
        ic_cases()
        print("golden fixtures ic_* written to", OUT)
        return
    if only == "damping":
        damping_case()
        print("golden fixture damping written to", OUT)
        return
    if only == "plastic":
        plastic_case()
        print("golden fixture plastic written to", OUT)
        return
    if only == "ldlt":
        ldlt_cases()
        print("golden fixtures ldlt_* written to", OUT)
        return
    if only == "modal":
        modal_cases()
        print("golden fixtures modal_* written to", OUT)
        return
    if only is not None:
        raise SystemExit(f"--only {only}: single groups are 'plastic', 'ldlt', 'ic', 'damping' and 'modal'")
    g = small_mesh()
    cases = {"full": meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0)),
             "partial": partial_constraints(g)}
    for cname, cd in cases.items():
        s = R.RefScene(g.X, g.tets, g.facets, cd, "corotational", *MATS["corotational"])
        pcol, rows, oris, emap = s.pattern()
        save(f"pattern_{cname}", X=g.X, tets=g.tets, facets=g.facets, cdofs=cd, dofs=s.dofs,
             sizes=s.sizes, pcol=pcol, rows=rows, oris=oris, emap=emap)

    rng = np.random.default_rng(123)
    u = rng.normal(scale=0.002, size=(g.n_nodes, 3))
    for mat, (rho, E, nu, thr) in MATS.items():
        for cname, cd in cases.items():
            s = R.RefScene(g.X, g.tets, g.facets, cd, mat, rho, E, nu, thr)
            s.set_displacements(u)
            K, f = s.element_values()
            vals, fint = s.assemble()
            mass = s.mass()
            x = rng.normal(size=s.dofs)
            y = s.spmdv(vals, x)
            A = vals * (1.0 / 3600.0) + mass
            b = rng.normal(size=s.dofs)
            xs, its = s.cg(A, b, tol=1e-10, maxit=2000, precond="jacobi")
            fext = s.loads(body=[0.0, 0.0, -9800.0],
                           tractions=[([0.0, -500.0, 0.0], g.face_facets(0, 1))])
            save(f"elements_{mat}_{cname}", u=u, K78=K, f12=f, values=vals, fint=fint,
                 mass=mass, spmv_x=x, spmv_y=y, cg_b=b, cg_x=xs, cg_iters=its, fext=fext,
                 material=np.array([rho, E, nu, thr]))

    for mat, (rho, E, nu, thr) in MATS.items():
        cd = cases["full"]
        s = R.RefScene(g.X, g.tets, g.facets, cd, mat, rho, E, nu, thr)
        s.be_setup(1.0 / 60.0, 0.01, 0.001, tol=1e-10, maxit=2000, precond="jacobi")
        fext = s.loads(body=[0.0, 0.0, -9800.0])
        s.be_apply_loads()
        iters = s.be_step(20)
        save(f"be_{mat}", fext=fext, u=s.displacements(), v=s.be_velocity(), steps=20, iters=iters,
             params=np.array([1.0 / 60.0, 0.01, 0.001, 1e-10]))
        s = R.RefScene(g.X, g.tets, g.facets, cd, mat, rho, E, nu, thr)
        s.nm_setup(1.0 / 60.0, 0.01, 0.001, beta=0.25, gamma=0.5, newton=2, tol=1e-10, maxit=2000,
                   precond="jacobi")
        fext = s.loads(body=[0.0, 0.0, -9800.0])
        s.nm_apply_loads()
        iters = s.nm_step(10)
        d, v, a = s.nm_state()
        save(f"nm_{mat}", fext=fext, u=s.displacements(), d=d, v=v, a=a, steps=10, iters=iters,
             params=np.array([1.0 / 60.0, 0.01, 0.001, 0.25, 0.5, 2, 1e-10]))

    # math known-answer vectors
    rng = np.random.default_rng(7)
    Fs = []
    for k in range(400):
        F = rng.normal(size=(3, 3)) * 10 ** rng.uniform(-2, 1)
        if k % 4 == 1:
            F = np.eye(3) + 1e-9 * rng.normal(size=(3, 3))
        if k % 4 == 2:
            F[:, 2] = 0.5 * F[:, 0] + 0.25 * F[:, 1] + 1e-12 * rng.normal(size=3)
        if k % 8 == 3:
            F = -F  # reflected
        Fs.append(F)
    Fs = np.array(Fs)
    polR = np.array([R.polar(F)[0] for F in Fs])
    polS = np.array([R.polar(F)[1] for F in Fs])
    qrQ = np.array([R.qr(F)[0] for F in Fs])
    qrR = np.array([R.qr(F)[1] for F in Fs])
    tri = []
    for F in Fs:
        S = F @ F.T
        tri.append([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]])
    tri = np.array(tri)
    ev = np.array([R.eigsym(t)[0] for t in tri])
    evec = np.array([R.eigsym(t)[1] for t in tri])
    save("kat_math", F=Fs, polar_R=polR, polar_S=polS, qr_Q=qrQ, qr_R=qrR, tri=tri, eig_vals=ev,
         eig_vecs=evec)
    plastic_case()
    ldlt_cases()
    ic_cases()
    damping_case()
    modal_cases()
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
