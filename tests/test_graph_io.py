"""Graph parsing: the product's four parsers against hl::Graph::read itself.

The .dump fixtures were printed by oracle/_ref/graphdump, a harness compiled
against the reference's shared_memory/graph.hpp (see tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

GDIR = os.path.join(GOLDEN, "graphs")
FILES = sorted(f for f in os.listdir(GDIR) if not f.endswith(".dump"))


def product_dump(P, path, undirected):
    try:
        g = P.Graph.read(path, undirected)
    except P.CHLError as e:
        assert e.status == P.CHL_ERR_FORMAT
        return "FAIL\n"
    lines = [f"{g.get_n()} {g.get_m()}"]
    for v in range(g.get_n()):
        for side in (0, 1):
            h, w = g.arcs(v, bool(side))
            parts = [str(v), str(side), str(len(h))]
            for a, b in zip(h, w):
                parts += [str(a), str(b)]
            lines.append(" ".join(parts))
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("fname", FILES)
@pytest.mark.parametrize("undirected", [0, 1])
def test_parser_matches_reference(P, fname, undirected):
    exp = open(os.path.join(GDIR, f"{fname}.u{undirected}.dump")).read()
    got = product_dump(P, os.path.join(GDIR, fname), undirected)
    assert got == exp


def test_missing_file_is_io_error(P, tmp_path):
    with pytest.raises(P.CHLError) as e:
        P.Graph.read(str(tmp_path / "nope.gr"))
    assert e.value.status == P.CHL_ERR_IO


def test_dimacs_roundtrip(P, tmp_path):
    g = P.Graph.grid(9, 7, seed=4)
    p = str(tmp_path / "g.gr")
    g.write(p)
    g2 = P.Graph.read(p)
    assert g2.get_n() == g.get_n() and g2.out_arcs() == g.out_arcs() and g2.symmetric()
    for v in range(g.get_n()):
        for f in (True, False):
            a, b = g.arcs(v, f), g2.arcs(v, f)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_oracle_reads_same_adjacency(P, O, tmp_path):
    g = P.Graph.grid(15, 11, highways=5, hw_steps=6, seed=8)
    p = str(tmp_path / "g.gr")
    g.write(p)
    og = O.OGraph.read_dimacs(p)
    for side in (0, 1):
        off, head, ln = og.csr(side)
        off2, head2, ln2 = g.csr(bool(side))
        assert np.array_equal(off, off2) and np.array_equal(head, head2) and np.array_equal(ln, ln2)


def test_graph_from_csr_matches_from_arcs(P):
    """chl_graph_from_csr gives the arc lists chl_graph_from_arcs builds from
    the same arcs (duplicates, loops and both directions merged alike)."""
    import numpy as np
    rng = np.random.default_rng(4)
    for t in range(4):
        n = int(rng.integers(1, 200))
        deg = rng.integers(0, 6, n)
        off = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
        k = int(off[-1])
        head = rng.integers(0, n, k).astype(np.uint32)
        length = rng.integers(1, 9, k).astype(np.int32)
        src = np.repeat(np.arange(n, dtype=np.uint32), deg)
        for und in (False, True):
            a = P.Graph.from_csr(n, off, head, length, und)
            b = P.Graph.from_arcs(n, src, head, length, und)
            assert a.get_n() == b.get_n() and a.get_m() == b.get_m()
            for fwd in (True, False):
                for x, y in zip(a.csr(fwd), b.csr(fwd)):
                    assert np.array_equal(x, y)


def test_graph_from_csr_rejects_bad_input(P):
    import numpy as np
    import pytest
    with pytest.raises(P.CHLError):
        P.Graph.from_csr(2, np.array([0, 2, 1], np.uint64), [1, 0], [1, 1])   # decreasing offsets
    with pytest.raises(P.CHLError):
        P.Graph.from_csr(2, np.array([0, 1, 2], np.uint64), [1, 5], [1, 1])   # head out of range
    with pytest.raises(P.CHLError):
        P.Graph.from_csr(2, np.array([0, 1], np.uint64), [1], [1])           # off too short
