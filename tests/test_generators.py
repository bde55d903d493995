"""Seeded generators: shapes of the benchmark graphs, determinism."""
import numpy as np


def test_grid_config1_shape(P):
    g = P.Graph.grid(100, 100, seed=1)
    n = g.get_n()
    assert 9000 < n <= 10000
    assert g.symmetric()
    # 4-neighbour grid minus 5% plus 1% diagonals: about 2*(2*100*99)*0.95 arcs
    assert 35000 < g.out_arcs() < 40000
    assert min(g.get_degree(v) for v in range(0, n, 97)) >= 2


def test_grid_is_deterministic(P):
    a = P.Graph.grid(30, 30, highways=20, hw_steps=10, seed=5)
    b = P.Graph.grid(30, 30, highways=20, hw_steps=10, seed=5)
    c = P.Graph.grid(30, 30, highways=20, hw_steps=10, seed=6)
    assert a.get_n() == b.get_n()
    oa, ha, la = a.csr()
    ob, hb, lb = b.csr()
    assert np.array_equal(oa, ob) and np.array_equal(ha, hb) and np.array_equal(la, lb)
    oc, hc, lc = c.csr()
    assert not (len(hc) == len(ha) and np.array_equal(hc, ha) and np.array_equal(lc, la))


def test_grid_weights_and_highways(P):
    g = P.Graph.grid(40, 40, highways=30, hw_steps=12, hw_factor=150.0, seed=2)
    _, _, ln = g.csr()
    assert ln.min() >= 1
    assert (ln <= 1000).sum() > 0.98 * len(ln)
    big = ln[ln > 1000]
    assert len(big) > 0 and all(w % 150 == 0 for w in big)


def test_rmat_shape(P):
    g = P.Graph.rmat(12, 16, seed=3)
    assert g.get_n() == 4096 and g.symmetric()
    off, head, ln = g.csr()
    assert (ln == 1).all()
    src = np.repeat(np.arange(g.get_n()), np.diff(off).astype(np.int64))
    assert (src != head).all()                      # no self loops
    key = src.astype(np.int64) * 4096 + head
    assert len(np.unique(key)) == len(key)          # no duplicates
    deg = np.diff(off)
    assert deg.max() > 20 * max(1, np.median(deg))  # skewed degrees
