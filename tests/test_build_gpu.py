"""Label construction on the GPU: bit-exact against the reference's labels.

Parity targets: the golden label files printed by the reference GLL binary,
and the CPU oracle (whose GLL restatement reproduces those files byte for
byte) on larger seeded graphs.  Every build mode must give the same labels:
canonical labels are unique for a given order.
"""
import filecmp

import numpy as np
import pytest

from conftest import label_case

pytestmark = pytest.mark.gpu

MODES = {"hybrid": 0, "gll": 1, "plant": 2}
CASES = ["grid12", "grid20hw", "rmat8", "directed60", "unit_path"]


def same_labels(L, ref, n):
    a = L.export()
    b = ref.export(n)
    for x, y in zip(a, b):
        if not np.array_equal(np.asarray(x), np.asarray(y)):
            return False
    return True


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("sched", ["default", "small", "rounds", "win1", "win8"])
def test_golden_label_files(P, case, mode, sched, tmp_path):
    c = label_case(case)
    g = P.Graph.read(c["gr"])
    order = P.Order.read(c["order"])
    kw = {"small": {"first_superstep": 7, "growth": 0.3},
          # first superstep by settle rounds instead of label-correcting windows
          "rounds": {"window_target": 1},
          # windows of about 2 vertices, one warp per tree; 8 warps per tree
          "win1": {"window_target": 2, "window_warps": 1, "first_superstep": 40},
          "win8": {"window_warps": 8, "window_target": 8}}.get(sched, {})
    L = P.build(g, order, mode=MODES[mode], **kw)
    out = str(tmp_path / "gpu.labels")
    L.write(out)
    assert filecmp.cmp(out, c["labels"], shallow=False)


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("sf", [32.0, 0.05])
def test_config1_grid_matches_oracle(P, O, mode, sf):
    g = P.Graph.grid(100, 100, seed=1)
    order = P.Order.degree(g, seed=1)
    off, head, ln = g.csr(True)
    og = O.OGraph.from_csr(g.get_n(), off, head, ln)
    ref, _ = O.gll(og, order)
    L = P.build(g, order, mode=MODES[mode], sf=sf)
    assert same_labels(L, ref, g.get_n())
    st = L.stats()
    assert st["supersteps"] >= 1 and st["labels"] == ref.total()


@pytest.mark.parametrize("split", [2, 16, 300])
@pytest.mark.parametrize("kind", ["grid", "rmat"])
def test_queue_split_matches_oracle(P, O, split, kind):
    # trees whose queues are split into near and far piles give the oracle's labels
    if kind == "grid":
        g = P.Graph.grid(120, 120, highways=30, seed=6)
        order = P.Order.degree(g, seed=3)
    else:
        g = P.Graph.rmat(12, 8, seed=8)
        order = P.Order.degree(g, seed=3)
    off, head, ln = g.csr(True)
    og = O.OGraph.from_csr(g.get_n(), off, head, ln)
    ref, _ = O.gll(og, order)
    for mode in (MODES["hybrid"], MODES["gll"]):
        L = P.build(g, order, mode=mode, queue_split=split)
        assert same_labels(L, ref, g.get_n()), (split, mode)
        # the first superstep's windows sized like the split
        L = P.build(g, order, mode=mode, window_target=split, first_superstep=split * 4)
        assert same_labels(L, ref, g.get_n()), ("window", split, mode)


@pytest.mark.parametrize("mode", list(MODES))
def test_rmat_unit_lengths_matches_oracle(P, O, mode):
    g = P.Graph.rmat(12, 16, seed=5)
    order = P.Order.degree(g, seed=2)
    off, head, ln = g.csr(True)
    og = O.OGraph.from_csr(g.get_n(), off, head, ln)
    ref, _ = O.gll(og, order)
    L = P.build(g, order, mode=MODES[mode], sf=1.0)
    assert same_labels(L, ref, g.get_n())
    L = P.build(g, order, mode=MODES[mode], sf=1.0, first_superstep=1, growth=0.05)
    assert same_labels(L, ref, g.get_n())


@pytest.mark.parametrize("mode", list(MODES))
def test_directed_weighted_matches_oracle(P, O, mode, tmp_path):
    rng = np.random.default_rng(7)
    n, m = 700, 4000
    src = rng.integers(0, n, m).astype(np.uint32)
    dst = rng.integers(0, n, m).astype(np.uint32)
    keep = src != dst
    w = rng.integers(1, 50, m).astype(np.int32)
    g = P.Graph.from_arcs(n, src[keep], dst[keep], w[keep])
    assert not g.symmetric()
    p = str(tmp_path / "d.gr")
    g.write(p)
    og = O.OGraph.read_dimacs(p)
    order = og.degree_order(3)
    ref, _ = O.gll(og, order)
    L = P.build(g, order, mode=MODES[mode], sf=0.5)
    assert same_labels(L, ref, n)


def test_directed_power_law_matches_oracle(P, O, tmp_path):
    """Directed, weighted, skewed degrees (2^15 vertices, ~2^18 arcs): two
    distinct label sides at a size where supersteps, the hash probe and the
    extension all engage."""
    rng = np.random.default_rng(11)
    n, m = 1 << 15, 1 << 18
    # endpoints: half uniform, half from a Pareto tail over a permutation
    perm = rng.permutation(n).astype(np.uint32)

    def pick(k):
        z = perm[np.minimum((rng.pareto(1.2, k) * 40).astype(np.int64), n - 1)]
        u = rng.integers(0, n, k).astype(np.uint32)
        return np.where(rng.random(k) < 0.5, z, u).astype(np.uint32)

    src, dst = pick(m), pick(m)
    keep = src != dst
    w = rng.integers(1, 100, m).astype(np.int32)
    g = P.Graph.from_arcs(n, src[keep], dst[keep], w[keep])
    assert not g.symmetric()
    p = str(tmp_path / "pl.gr")
    g.write(p)
    og = O.OGraph.read_dimacs(p)
    order = og.degree_order(5)
    ref, _ = O.gll(og, order)
    for kw in ({"queue_split": 64}, {"mode": MODES["gll"], "queue_split": 16}, {"label_cap": 5000},
               {}, {"mode": MODES["gll"]}, {"first_superstep": 100, "growth": 0.5}):
        L = P.build(g, order, **kw)
        assert same_labels(L, ref, n), kw
    pairs = P.generate_query(20000, n, seed=3)
    assert np.array_equal(P.query(L, pairs), ref.query(pairs))


def test_tiny_and_disconnected(P, O):
    # isolated vertices, a 2-cycle and a single arc
    g = P.Graph.from_arcs(5, [0, 1, 3], [1, 0, 4], [2, 2, 7])
    order = np.array([4, 2, 0, 3, 1], np.uint32)
    off, head, ln = g.csr(True)
    og = O.OGraph.from_csr(5, off, head, ln)
    ref, _ = O.gll(og, order)
    for mode in MODES.values():
        L = P.build(g, order, mode=mode)
        assert same_labels(L, ref, 5)
    L = P.build(g, order)
    q = P.query(L, [[0, 1], [3, 4], [4, 3], [2, 0], [2, 2]])
    assert q.tolist() == [2, 7, P.INFTY, P.INFTY, 0]


def test_single_vertex(P):
    g = P.Graph.from_arcs(1, [], [], [])
    L = P.build(g, np.array([0], np.uint32))
    assert L.label(0, 0)[0].tolist() == [0] and L.label(0, 1)[1].tolist() == [0]


def test_bad_order_rejected(P):
    g = P.Graph.grid(5, 5, seed=1)
    n = g.get_n()
    with pytest.raises(P.CHLError) as e:
        P.build(g, np.zeros(n, np.uint32))
    assert e.value.status == P.CHL_ERR_INVALID
    with pytest.raises(P.CHLError):
        P.build(g, np.arange(n - 1, dtype=np.uint32))


def test_build_is_deterministic(P):
    g = P.Graph.grid(60, 60, highways=40, hw_steps=16, seed=9)
    order = P.Order.degree(g, seed=4)
    a = P.build(g, order, sf=0.2).export()
    for kw in ({"max_warps": 64}, {"max_warps": 8}, {"first_superstep": 1, "growth": 0.05},
               {"first_superstep": 5000, "growth": 4.0}, {"first_superstep": 3},
               {"use_graphs": 0}, {"use_graphs": 0, "mode": 1}, {"use_graphs": 1, "mode": 1},
               {"superstep_extend": 1}, {"superstep_extend": 16, "first_superstep": 9, "growth": 0.2},
               {"superstep_extend": 16, "mode": 1, "first_superstep": 9},
               {"first_superstep": 1, "growth": 0.01, "superstep_extend": 1},
               # new-label buffers far below a superstep's labels: every
               # overflowed superstep re-runs its root range
               {"label_cap": 1000}, {"label_cap": 1000, "mode": 1}, {"label_cap": 4000, "max_warps": 8},
               {"label_cap": 3000, "first_superstep": 3}, {"label_cap": 2000, "mode": 2},
               # near/far queue split at tiny queue sizes (refills, stale
               # far entries, threshold doubling and halving), and off
               {"queue_split": 1}, {"queue_split": 2}, {"queue_split": 8}, {"queue_split": 8, "mode": 1},
               {"queue_split": 33, "first_superstep": 1, "growth": 0.05}, {"queue_split": 200},
               {"queue_split": 8, "mode": 2}, {"queue_split": 8, "max_warps": 4},
               # first-superstep windows: off, tiny, large; 1, 2 and 8 warps per tree
               {"window_target": 1}, {"window_target": 2}, {"window_target": 3, "mode": 1},
               {"window_target": 100000}, {"window_warps": 1}, {"window_warps": 2, "window_target": 16},
               {"window_warps": 8, "mode": 1}, {"window_warps": 8, "first_superstep": 5000, "window_target": 5}):
        b = P.build(g, order, sf=0.2, **kw).export()
        for x, y in zip(a, b):
            assert np.array_equal(x, y), kw


def test_sampled_queries_equal_dijkstra(P, O):
    g = P.Graph.grid(80, 80, highways=30, hw_steps=20, seed=2)
    order = P.Order.degree(g, seed=6)
    L = P.build(g, order)
    off, head, ln = g.csr(True)
    og = O.OGraph.from_csr(g.get_n(), off, head, ln)
    rng = np.random.default_rng(1)
    n = g.get_n()
    for s in rng.integers(0, n, 8):
        d = og.dijkstra(int(s))
        pairs = np.stack([np.full(n, s), np.arange(n)], 1).astype(np.uint32)
        assert np.array_equal(P.query(L, pairs), d)


def test_config1_100k_queries_equal_dijkstra(P, O):
    """Config 1: 100x100 grid, degree order, 100,000 uniform (s, t) pairs
    answered by the GPU labels and by plain Dijkstra on the CPU."""
    g = P.Graph.grid(100, 100, seed=1)
    order = P.Order.degree(g, seed=1)
    L = P.build(g, order)
    n = g.get_n()
    off, head, ln = g.csr(True)
    og = O.OGraph.from_csr(n, off, head, ln)
    pairs = P.generate_query(100000, n, seed=3)
    got = P.query(L, pairs)
    exp = np.empty(len(pairs), np.int32)
    by_src = np.argsort(pairs[:, 0], kind="stable")
    srcs, first, cnt = np.unique(pairs[by_src, 0], return_index=True, return_counts=True)
    for s, a, c in zip(srcs, first, cnt):
        sel = by_src[a:a + c]
        exp[sel] = og.dijkstra(int(s))[pairs[sel, 1]]
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("mode", list(MODES))
def test_root_limit_gives_the_label_prefix(P, mode):
    """A build of the roots of rank < R holds exactly the full labeling's
    entries whose hub rank is below R (labels of committed hubs are final)."""
    g = P.Graph.grid(50, 50, highways=12, hw_steps=10, seed=13)
    order = P.Order.betweenness(g, 64, seed=2)
    full_off, full_hub, full_dist = P.build(g, order, mode=MODES[mode], sf=0.5).export()
    for limit in (1, 37, 400):
        off, hub, dist = P.build(g, order, mode=MODES[mode], sf=0.5, first_superstep=16, growth=0.5,
                                 root_limit=limit).export()
        top = int(hub.max())
        assert top == limit - 1
        for i in range(off.size - 1):
            a, b = int(full_off[i]), int(full_off[i + 1])
            keep = full_hub[a:b] <= top
            assert np.array_equal(hub[off[i]:off[i + 1]], full_hub[a:b][keep])
            assert np.array_equal(dist[off[i]:off[i + 1]], full_dist[a:b][keep])
