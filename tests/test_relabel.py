"""Node relabeling (core/meshRelabler.cpp, Gibbs-Poole-Stockmeyer).  A host
function of the library (no GPU): a valid permutation, the same elements,
elements ordered by label sum, deterministic, every connected component
labelled, and bandwidth / profile as small as the reference's own
relabeling of the same shuffled meshes (the labels themselves cannot match:
the reference's ties follow its standard library's hash and heap orders)."""
import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from oracle import reforacle as R


def bandwidth(t):
    s = np.sort(t, axis=1)
    return int((s[:, -1] - s[:, 0]).max())


def profile(t, n):
    lo = np.full(n, n)
    for k in range(t.shape[1]):
        np.minimum.at(lo, t[:, k], t.min(axis=1))
    return int((np.arange(n) - np.minimum(lo, np.arange(n))).sum())


def shuffled(g, seed=0):
    perm = np.random.default_rng(seed).permutation(g.n_nodes)
    return perm[g.tets].astype(np.int32)


@pytest.mark.parametrize("mesh", ["cantilever", "small"])
def test_permutation_and_same_elements(mesh):
    g = meshgen.cantilever_3000() if mesh == "cantilever" else meshgen.tet_grid(4, 3, 2, jitter=0.1, seed=2)
    t = shuffled(g)
    labels, t2 = api.mesh_relabel(g.n_nodes, t)
    assert np.array_equal(np.sort(labels), np.arange(g.n_nodes))
    def canon(e):   # the elements as a set of sorted node tuples
        r = np.sort(e, axis=1)
        return r[np.lexsort(r.T[::-1])]
    assert np.array_equal(canon(labels[t]), canon(t2))
    # element order: by the sum of the new labels; node order inside an element kept
    assert np.all(np.diff(t2.sum(axis=1)) >= 0)
    assert bandwidth(t2) < bandwidth(t)


def test_deterministic_and_components():
    g = meshgen.tet_grid(5, 2, 2, jitter=0.1, seed=4)
    t = shuffled(g, 3)
    a = api.mesh_relabel(g.n_nodes, t)
    b = api.mesh_relabel(g.n_nodes, t)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    # two disjoint copies plus one node in no element: every node labelled
    n = g.n_nodes
    t2 = np.concatenate([t, t + n]).astype(np.int32)
    labels, e = api.mesh_relabel(2 * n + 1, t2)
    assert np.array_equal(np.sort(labels), np.arange(2 * n + 1))
    assert labels[2 * n] == 2 * n                      # the unused node goes last
    first = set(labels[:n].tolist())
    assert first == set(range(n)) or first == set(range(n, 2 * n))   # components keep contiguous labels


def test_bad_arguments():
    with pytest.raises(api.ODError):
        api.mesh_relabel(3, np.array([[0, 1, 2, 3]]))     # node id out of range
    with pytest.raises(api.ODError):
        api.mesh_relabel(4, np.array([[0, 1, 2, -1]]))


@pytest.mark.skipif(not R.available(), reason="compiled reference not built")
@pytest.mark.parametrize("mesh", ["cantilever", "beam"])
def test_as_good_as_the_reference(mesh):
    g = meshgen.cantilever_3000() if mesh == "cantilever" else meshgen.beam_98k()
    t = shuffled(g)
    _, er = R.relabel(g.n_nodes, t)
    _, ep = api.mesh_relabel(g.n_nodes, t)
    assert bandwidth(ep) <= 1.05 * bandwidth(er) + 2
    assert profile(ep, g.n_nodes) <= 1.15 * profile(er, g.n_nodes)
