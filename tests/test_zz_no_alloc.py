"""The allocation-free PCG entry point (od_bsr_pcg_noalloc).

Callers that cannot allocate device memory (their host application's own
allocator owns the GPU's memory, or their host forbids allocation once it is
running) hand in a block-CSR matrix and vectors they already hold on the
device; the library keeps its work vectors in one fixed device array.  This
checks, through the C ABI, that two calls in a row agree with the allocating
entry point od_scene_pcg within the parity tolerance used by the other solver
tests, that systems above the fixed limit and malformed structures are
rejected, and the exits without convergence.  The file is named to be
collected last.
"""
import ctypes as C

import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx, rel_err

pytestmark = pytest.mark.gpu


def full_bsr(dofs, pcol, rows, oris, values):
    """Both-triangle block-CSR (row-major 3x3 blocks) of the reference's lower
    block-CSC values; needs a DOF count divisible by 3."""
    assert dofs % 3 == 0
    nb = dofs // 3
    blocks = {}
    for bc in range(nb):
        off = int(oris[bc])
        for k in range(int(pcol[bc]), int(pcol[bc + 1])):
            br = int(rows[k]) // 3
            if br == bc:
                v = values[off:off + 6]
                m = np.array([[v[0], v[1], v[2]], [v[1], v[3], v[4]], [v[2], v[4], v[5]]])
                blocks[(bc, bc)] = m
                off += 6
            else:
                m = values[off:off + 9].reshape(3, 3).T  # column-major storage
                blocks[(br, bc)] = m
                blocks[(bc, br)] = m.T
                off += 9
    keys = sorted(blocks)
    row_ptr = np.zeros(nb + 1, np.int32)
    for (r, _c) in keys:
        row_ptr[r + 1] += 1
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    col = np.array([c for (_r, c) in keys], np.int32)
    vals = np.concatenate([blocks[k].reshape(-1) for k in keys])
    return nb, row_ptr, col, vals


def solve_noalloc(nb, row_ptr, col, vals, b, solver, x0=None):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    t_rp = torch.from_numpy(row_ptr).to(dev)
    t_col = torch.from_numpy(col).to(dev)
    t_vals = torch.from_numpy(vals).to(dev)
    t_b = torch.from_numpy(np.ascontiguousarray(b)).to(dev)
    t_x = (torch.zeros(3 * nb, dtype=torch.float64, device=dev) if x0 is None else
           torch.from_numpy(np.ascontiguousarray(x0, dtype=np.float64)).to(dev))
    torch.cuda.synchronize()
    prm = solver.to_c()
    st = api.od_solve_stats()
    L = api.load_library()
    rc = L.od_bsr_pcg_noalloc(nb, t_rp.data_ptr(), t_col.data_ptr(), t_vals.data_ptr(), t_b.data_ptr(),
                              t_x.data_ptr(), C.byref(prm), None, C.byref(st))
    torch.cuda.synchronize()
    return rc, t_x.cpu().numpy(), st


def cantilever_system():
    g = meshgen.cantilever_3000()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, api.CorotationalHyperelasticMaterial(1000, 1e5, 0.45, 0.1))
    s.set_displacements(np.random.default_rng(4).normal(scale=0.002, size=(g.n_nodes, 3)))
    K, _ = s.evaluate()
    A = K * (1.0 / 3600.0) + s.mass()
    b = np.random.default_rng(5).normal(size=s.dofs)
    return s, A, b


@pytest.mark.parametrize("precond", ["none", "jacobi", "block_jacobi"])
def test_noalloc_pcg_matches_scene_pcg_twice(precond):
    s, A, b = cantilever_system()
    solver = api.CGSolver(1e-10, 6000, api.Preconditioner(precond))
    x_ref, st_ref = s.pcg(A, b, solver=solver)
    assert st_ref.status == 0
    pcol, rows, oris, _ = s.pattern()
    nb, row_ptr, col, vals = full_bsr(s.dofs, pcol, rows, oris, A)
    for call in range(2):  # the second call runs on the array the first left behind
        rc, x, st = solve_noalloc(nb, row_ptr, col, vals, b, solver)
        assert rc == 0 and st.status == 0, f"call {call}: rc {rc} status {st.status}"
        assert abs(st.iterations - st_ref.iterations) <= max(2, 0.02 * st_ref.iterations)
        assert st.rel_residual <= 1e-9
        assert rel_err(x, x_ref) <= 1e-8


def test_noalloc_rejects_systems_above_its_limit():
    limit = 32768  # OD_NOALLOC_MAX_BLOCK_ROWS
    rc, _, _ = solve_noalloc(1, np.array([0, 1], np.int32), np.array([0], np.int32), np.eye(3).reshape(-1),
                             np.ones(3), api.CGSolver(1e-8, 10, api.JacobiPreconditioner()))
    assert rc == 0
    torch = pytest.importorskip("torch")
    small = torch.zeros(16, dtype=torch.float64, device="cuda")  # valid memory; never read past the size check
    L = api.load_library()
    prm = api.CGSolver(1e-8, 10, api.JacobiPreconditioner()).to_c()
    st = api.od_solve_stats()
    ptr = small.data_ptr()
    rc = L.od_bsr_pcg_noalloc(limit + 1, ptr, ptr, ptr, ptr, ptr, C.byref(prm), None, C.byref(st))
    assert rc == 1  # OD_ERR_INVALID_ARG
    assert b"OD_NOALLOC_MAX_BLOCK_ROWS" in L.od_last_error()


def test_noalloc_exits_without_convergence_and_keeps_the_warm_start():
    s, A, b = cantilever_system()
    pcol, rows, oris, _ = s.pattern()
    nb, row_ptr, col, vals = full_bsr(s.dofs, pcol, rows, oris, A)
    # too few iterations: the call succeeds, the solve reports NOT_CONVERGED
    rc, x, st = solve_noalloc(nb, row_ptr, col, vals, b, api.CGSolver(1e-10, 5, api.JacobiPreconditioner()))
    assert rc == 0 and st.status == 3 and st.iterations == 5
    assert np.all(np.isfinite(x)) and st.rel_residual > 1e-10
    # no iteration at all: the warm start comes back unchanged
    x0 = np.random.default_rng(6).normal(size=s.dofs)
    rc, x, st = solve_noalloc(nb, row_ptr, col, vals, b, api.CGSolver(1e-10, 0, api.JacobiPreconditioner()), x0=x0)
    assert rc == 0 and st.iterations == 0
    assert np.array_equal(x, x0)


def test_noalloc_rejects_malformed_structures_and_other_preconditioners():
    s, A, b = cantilever_system()
    pcol, rows, oris, _ = s.pattern()
    nb, row_ptr, col, vals = full_bsr(s.dofs, pcol, rows, oris, A)
    L = api.load_library()
    solver = api.CGSolver(1e-10, 100, api.JacobiPreconditioner())
    bad = col.copy()
    bad[len(bad) // 2] = nb  # one block column past the last block row
    rc, x, st = solve_noalloc(nb, row_ptr, bad, vals, b, solver)
    assert rc == 1 and st.status == 1  # OD_ERR_INVALID_ARG, found on the device
    assert b"block column" in L.od_last_error()
    assert np.array_equal(x, np.zeros_like(x))
    bad_rp = row_ptr.copy()
    bad_rp[nb // 2] = bad_rp[nb // 2 + 1] + 1  # a decreasing row pointer
    rc, _, st = solve_noalloc(nb, bad_rp, col, vals, b, solver)
    assert rc == 1 and st.status == 1
    # a later valid call on the same array is unaffected
    rc, _, st = solve_noalloc(nb, row_ptr, col, vals, b, api.CGSolver(1e-10, 6000, api.JacobiPreconditioner()))
    assert rc == 0 and st.status == 0
    rc, _, _ = solve_noalloc(nb, row_ptr, col, vals, b, api.CGSolver(1e-10, 100, api.IC0Preconditioner()))
    assert rc == 7  # OD_ERR_UNSUPPORTED: IC(0) needs factor storage
