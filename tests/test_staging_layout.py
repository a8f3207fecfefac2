"""CPU checks of the element staging layout shared by the element kernels
(writers) and the gather lists (readers), both in
opendeformer_gb300/csrc/od_elements.cu: c_kslot maps the packed entry k of
the 12x12 element matrix's upper triangle (row-major, the order of
Element::getLocalMatrixIndex, core/element.h:109-118) to its slot in the
element's 78 staged values, with every local 3x3 node block contiguous --
blocks (0,0), (0,1), (0,2), (0,3), (1,1), ..., (3,3); a diagonal block's 6
upper entries, an off-diagonal block's 9 row-major.  The assembly reads one
contiguous run per contributing element only if this holds."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "opendeformer_gb300", "csrc", "od_elements.cu")


def kslot_table():
    src = open(SRC).read()
    m = re.search(r"__constant__ int c_kslot\[78\]\s*=\s*\{([^}]*)\}", src)
    assert m, "c_kslot initializer not found"
    return [int(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]


def packed_entries():
    """(row, col) of packed entry k, row <= col, row-major upper triangle."""
    return [(r, c) for r in range(12) for c in range(r, 12)]


def test_kslot_is_a_permutation():
    t = kslot_table()
    assert len(t) == 78 and sorted(t) == list(range(78))


def test_kslot_groups_node_blocks_contiguously():
    t = kslot_table()
    blocks = [(a, b) for a in range(4) for b in range(a, 4)]
    start, off = {}, 0
    for a, b in blocks:
        start[(a, b)] = off
        off += 6 if a == b else 9
    assert off == 78
    upper3 = {(0, 0): 0, (0, 1): 1, (0, 2): 2, (1, 1): 3, (1, 2): 4, (2, 2): 5}
    for k, (r, c) in enumerate(packed_entries()):
        a, i = divmod(r, 3)
        b, j = divmod(c, 3)
        expect = start[(a, b)] + (upper3[(i, j)] if a == b else 3 * i + j)
        assert t[k] == expect, (k, r, c)


def test_packed_index_of_the_diagonal_matches_its_table():
    # c_diag12 (the packed position of (i, i)) and c_kslot agree on the
    # diagonal entries, which sit first in each diagonal node block's run
    src = open(SRC).read()
    m = re.search(r"__constant__ int c_diag12\[12\]\s*=\s*\{([^}]*)\}", src)
    diag = [int(v) for v in m.group(1).split(",")]
    pk = packed_entries()
    for i, k in enumerate(diag):
        assert pk[k] == (i, i)
    t = kslot_table()
    for a in range(4):
        assert t[diag[3 * a]] == [0, 33, 57, 72][a]
