"""Seeded synthetic tetrahedral grid meshes (the workload generator).

The reference ships no meshes or datasets; every workload here is a jittered
structured grid of cubes split into tetrahedra, generated from a seed so the
GPU path, the CPU oracle and the compiled reference all see bit-identical
inputs.

Conventions (written down once, used everywhere):

* Node (i, j, k) of an ``nx x ny x nz`` cube grid sits at ``(i*h, j*h, k*h)``;
  node index = ``i + (nx+1)*(j + (ny+1)*k)``.
* Interior nodes get a uniform jitter in ``[-c*h, +c*h]^3`` drawn from
  ``numpy.random.default_rng(seed)`` in node-index order; boundary nodes are
  not jittered so the faces stay planar for constraints and tractions.
* ``tets_per_cube=6``: Kuhn split around the main diagonal (same orientation
  in every cube, conforming).  ``tets_per_cube=5``: one central tet plus four
  corner tets, mirrored on odd ``i+j+k`` so face diagonals match.
* Facets are the boundary triangles of the tet mesh (faces used by exactly
  one tet), ordered by (min node, mid node, max node).

The mesh container mirrors the reference's ``TetMesh`` inputs
(``mesh/tetmesh.h:12``: node count, element count, facet count, then
``setVertex``/``setElement``/``setFacet`` in ``core/mesh.cpp:7-40``).
"""
from __future__ import annotations

import dataclasses

import numpy as np

# Kuhn split: the six monotone lattice paths from corner 0 to corner 7
# (corner bit 0 = +x, bit 1 = +y, bit 2 = +z).
_KUHN6 = np.array([[0, 1, 3, 7], [0, 1, 5, 7], [0, 2, 3, 7],
                   [0, 2, 6, 7], [0, 4, 5, 7], [0, 4, 6, 7]], dtype=np.int64)
# Five-tet split (central tet 0,3,5,6) and its mirror (central tet 1,2,4,7).
_FIVE_EVEN = np.array([[0, 3, 5, 6], [1, 0, 3, 5], [2, 0, 3, 6],
                       [4, 0, 5, 6], [7, 3, 5, 6]], dtype=np.int64)
_FIVE_ODD = np.array([[1, 2, 4, 7], [0, 1, 2, 4], [3, 1, 2, 7],
                      [5, 1, 4, 7], [6, 2, 4, 7]], dtype=np.int64)


@dataclasses.dataclass
class TetGrid:
    """A tetrahedral mesh plus the grid metadata used to pick faces."""

    X: np.ndarray          # (n_nodes, 3) float64 rest positions
    tets: np.ndarray       # (n_tets, 4) int32 node indices
    facets: np.ndarray     # (n_facets, 3) int32 boundary triangles
    dims: tuple            # (nx, ny, nz) cube counts
    h: float               # cube edge length

    @property
    def n_nodes(self) -> int:
        return int(self.X.shape[0])

    @property
    def n_tets(self) -> int:
        return int(self.tets.shape[0])

    @property
    def n_facets(self) -> int:
        return int(self.facets.shape[0])

    def node_ijk(self) -> np.ndarray:
        nx, ny, _ = self.dims
        idx = np.arange(self.n_nodes, dtype=np.int64)
        i = idx % (nx + 1)
        j = (idx // (nx + 1)) % (ny + 1)
        k = idx // ((nx + 1) * (ny + 1))
        return np.stack([i, j, k], axis=1)

    def face_nodes(self, axis: int, side: int) -> np.ndarray:
        """Sorted node indices on the grid face ``axis`` = 0 (side 0) or max."""
        ijk = self.node_ijk()
        target = 0 if side == 0 else self.dims[axis]
        return np.nonzero(ijk[:, axis] == target)[0].astype(np.int32)

    def face_facets(self, axis: int, side: int) -> np.ndarray:
        """Indices of boundary facets lying on a grid face."""
        ijk = self.node_ijk()
        target = 0 if side == 0 else self.dims[axis]
        on = ijk[:, axis] == target
        return np.nonzero(on[self.facets].all(axis=1))[0].astype(np.int32)


def constrained_dofs_for_nodes(nodes: np.ndarray) -> np.ndarray:
    """Sorted DOF list ``3*node + axis`` fixing every axis of ``nodes``.

    Mirrors ``Constrainer::setConstrains(nodeCounts, nodeIndices)`` with no
    constraint types (``core/constrainer.cpp:43-50``), whose std::set output is
    sorted (``core/constrainer.cpp:74-79``).
    """
    nodes = np.unique(np.asarray(nodes, dtype=np.int64))
    d = (3 * nodes[:, None] + np.arange(3)[None, :]).reshape(-1)
    return d.astype(np.int32)


def _boundary_facets(tets: np.ndarray) -> np.ndarray:
    faces = np.concatenate([tets[:, [0, 1, 2]], tets[:, [0, 1, 3]],
                            tets[:, [0, 2, 3]], tets[:, [1, 2, 3]]], axis=0)
    faces = np.sort(faces, axis=1)
    order = np.lexsort((faces[:, 2], faces[:, 1], faces[:, 0]))
    faces = faces[order]
    same_next = np.all(faces[1:] == faces[:-1], axis=1)
    dup = np.zeros(faces.shape[0], dtype=bool)
    dup[1:] |= same_next
    dup[:-1] |= same_next
    return faces[~dup].astype(np.int32)


def tet_grid(nx: int, ny: int, nz: int, h: float = 0.05, jitter: float = 0.0,
             seed: int = 0, tets_per_cube: int = 6) -> TetGrid:
    """Build a jittered cube grid split into 5 or 6 tets per cube."""
    if tets_per_cube not in (5, 6):
        raise ValueError("tets_per_cube must be 5 or 6")
    if min(nx, ny, nz) < 1:
        raise ValueError("grid needs at least one cube per axis")
    px, py, pz = nx + 1, ny + 1, nz + 1
    n_nodes = px * py * pz
    idx = np.arange(n_nodes, dtype=np.int64)
    i = idx % px
    j = (idx // px) % py
    k = idx // (px * py)
    X = np.stack([i * h, j * h, k * h], axis=1).astype(np.float64)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        jit = rng.uniform(-jitter * h, jitter * h, size=(n_nodes, 3))
        interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
        X[interior] += jit[interior]

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci = ci.transpose(2, 1, 0).reshape(-1)   # cube order: i fastest, then j, then k
    cj = cj.transpose(2, 1, 0).reshape(-1)
    ck = ck.transpose(2, 1, 0).reshape(-1)
    base = ci + px * (cj + py * ck)
    corner = np.array([0, 1, px, px + 1, px * py, px * py + 1, px * py + px,
                       px * py + px + 1], dtype=np.int64)
    cube_nodes = base[:, None] + corner[None, :]            # (n_cubes, 8)
    if tets_per_cube == 6:
        tets = cube_nodes[:, _KUHN6].reshape(-1, 4)
    else:
        parity = ((ci + cj + ck) & 1).astype(bool)
        t_even = cube_nodes[:, _FIVE_EVEN]
        t_odd = cube_nodes[:, _FIVE_ODD]
        tets = np.where(parity[:, None, None], t_odd, t_even).reshape(-1, 4)
    tets = tets.astype(np.int32)
    facets = _boundary_facets(tets.astype(np.int64))
    return TetGrid(X=X, tets=tets, facets=facets, dims=(nx, ny, nz), h=float(h))


def cantilever_3000(seed: int = 1) -> TetGrid:
    """20x5x5 cubes of 0.05 m, 6 tets each (3000 tets, 756 nodes), jitter 0.1h."""
    return tet_grid(20, 5, 5, h=0.05, jitter=0.10, seed=seed, tets_per_cube=6)


def beam_98k(seed: int = 2) -> TetGrid:
    """64x16x16 cubes of 0.05 m, 6 tets each (98,304 tets, 18,785 nodes), jitter 0.15h."""
    return tet_grid(64, 16, 16, h=0.05, jitter=0.15, seed=seed, tets_per_cube=6)


def block_2m6(seed: int = 4) -> TetGrid:
    """128x64x64 cubes, 5 tets each (2,621,440 tets), longest side 1 m, jitter 0.2h."""
    return tet_grid(128, 64, 64, h=1.0 / 128, jitter=0.20, seed=seed, tets_per_cube=5)


def batch_instances(n: int = 512, seed: int = 3):
    """Uneven batch: n independent jittered grids (0.05 m cubes, 6 tets each,
    interior jitter 0.1 h) whose cube counts are drawn per axis log-uniformly
    in [4, 40]; per instance a corotational or invertible Neo-Hookean
    material (probability 1/2), E log-uniform in [1e4, 1e6] Pa and nu uniform
    in [0.3, 0.48].  Returns dicts (dims, kind, E, nu, seed); build a mesh
    with instance_grid."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(v) for v in np.rint(np.exp(rng.uniform(np.log(4.0), np.log(40.0), size=3))))
        kind = "corotational" if rng.random() < 0.5 else "neohookean"
        E = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
        nu = float(rng.uniform(0.3, 0.48))
        out.append(dict(dims=dims, kind=kind, E=E, nu=nu, seed=seed * 100000 + i))
    return out


def instance_grid(inst) -> TetGrid:
    nx, ny, nz = inst["dims"]
    return tet_grid(nx, ny, nz, h=0.05, jitter=0.10, seed=inst["seed"], tets_per_cube=6)



def serving_pool(n: int = 4096, seed: int = 5):
    """Scene pool for serving: tet counts log-uniform in [1e3, 2e5], box
    aspect ratios (x and y against z) uniform in [1, 8], 6 tets per cube,
    longest side 1 m, interior jitter 0.1 h; corotational or invertible
    Neo-Hookean (probability 1/2), E log-uniform in [1e4, 1e6] Pa, nu uniform
    in [0.3, 0.48].  Returns dicts (dims, h, kind, E, nu, seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        tets = float(np.exp(rng.uniform(np.log(1e3), np.log(2e5))))
        ax, ay = rng.uniform(1.0, 8.0, size=2)
        s = (tets / 6.0 / (ax * ay)) ** (1.0 / 3.0)
        dims = tuple(max(1, int(round(v))) for v in (ax * s, ay * s, s))
        kind = "corotational" if rng.random() < 0.5 else "neohookean"
        E = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
        nu = float(rng.uniform(0.3, 0.48))
        out.append(dict(dims=dims, h=1.0 / max(dims), kind=kind, E=E, nu=nu, seed=seed * 100000 + i))
    return out


def pool_grid(inst) -> TetGrid:
    nx, ny, nz = inst["dims"]
    return tet_grid(nx, ny, nz, h=inst["h"], jitter=0.10, seed=inst["seed"], tets_per_cube=6)
