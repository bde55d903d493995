"""Schedule autotuner: search and cache logic on the host, exactness on the GPU."""
import json

import numpy as np
import pytest


class FakeLabels:
    def __init__(self, ms):
        self.ms = ms

    def stats(self):
        return {"build_ms": self.ms}


def test_search_and_cache(P, tmp_path, monkeypatch):
    from plant_gb300 import autotune as A
    calls = []

    def fake_build(g, order, root_limit=0, first_superstep=0, growth=0.0, sf=0.0, queue_split=0, window_target=0,
                   window_warps=0, ps=0.0, **kw):
        calls.append((root_limit, first_superstep, growth, sf, queue_split))
        # minimum at first=1024, growth=2.0, sf=128, queue_split=512
        ms = (100 + abs(first_superstep - 1024) / 10 + abs(growth - 2.0) * 7 + abs(sf - 128) / 50
              + (0 if queue_split == 512 else 3))
        return FakeLabels(ms)

    monkeypatch.setattr(A, "build", fake_build)
    g = P.Graph.grid(30, 30, seed=3)
    order = np.arange(g.get_n(), dtype=np.uint32)
    cache = str(tmp_path / "tune.json")
    cfg = A.tune(g, order, fraction=0.1, min_roots=10, cache=cache)
    assert cfg == {"first_superstep": 1024, "growth": 2.0, "sf": 128.0, "queue_split": 512, "window_target": 0,
                   "window_warps": 0, "ps": 0.0}
    assert all(c[0] == max(10, int(0.1 * g.get_n())) for c in calls)
    n_calls = len(calls)
    assert n_calls <= sum(len(v) for _, v in A.KNOBS)
    data = json.load(open(cache))
    assert A.graph_key(g) in data and data[A.graph_key(g)]["config"] == cfg
    # cached: no further builds
    assert A.tune(g, order, cache=cache) == cfg
    assert len(calls) == n_calls
    # force: searched again
    A.tune(g, order, fraction=0.1, min_roots=10, cache=cache, force=True)
    assert len(calls) > n_calls


def test_graph_key_separates_families(P):
    from plant_gb300 import autotune as A
    a = A.graph_key(P.Graph.grid(64, 64, seed=1))
    b = A.graph_key(P.Graph.rmat(12, 16, seed=1))
    assert a != b and "flat" in a and "heavy" in b


@pytest.mark.gpu
def test_tuned_build_is_exact(P, tmp_path):
    from plant_gb300 import autotune as A
    g = P.Graph.rmat(12, 16, seed=5)
    order = P.Order.degree(g, seed=1)
    ref = P.build(g, order).export()
    L = A.tuned_build(g, order, cache=str(tmp_path / "t.json"))
    for x, y in zip(L.export(), ref):
        assert np.array_equal(x, y)


def test_table_round_trip(P, tmp_path):
    """write_table writes the text table the library reads; a class's line
    is replaced, other lines are kept."""
    from plant_gb300 import autotune as A
    path = str(tmp_path / "sched.txt")
    g = P.Graph.grid(40, 40, seed=2)
    key = g.graph_class()
    assert key == A.graph_key(g) and key.startswith("sym-n2^11-deg")
    A.write_table(path, entries={key: {"first_superstep": 7, "growth": 0.5, "sf": 2.0, "queue_split": 1,
                                       "window_target": 1, "window_warps": 4}, "dir-n2^3-deg1-skewflat": {
        "first_superstep": 1, "growth": 1.0, "sf": 1.0, "queue_split": 0, "window_target": 256, "window_warps": 8}})
    A.write_table(path, entries={key: {"first_superstep": 9, "growth": 0.25, "sf": 4.0, "queue_split": 0,
                                       "window_target": 1, "window_warps": 4}})
    lines = [x.split() for x in open(path) if x.strip() and not x.startswith("#")]
    assert sorted(x[0] for x in lines) == sorted([key, "dir-n2^3-deg1-skewflat"])
    assert [x for x in lines if x[0] == key][0][1:] == ["9", "0.25", "4.0", "0", "1", "4", "0.0"]


@pytest.mark.gpu
def test_build_reads_the_table(P, tmp_path, monkeypatch):
    """With autotune set, options left at 0 come from the table for the
    graph's class (CHL_SCHEDULES), and the labels stay exact."""
    from plant_gb300 import autotune as A
    g = P.Graph.grid(50, 50, seed=6)
    order = P.Order.degree(g, seed=2)
    ref = P.build(g, order, autotune=0)
    path = str(tmp_path / "sched.txt")
    A.write_table(path, entries={g.graph_class(): {"first_superstep": 1, "growth": 0.01, "sf": 0.5,
                                                   "queue_split": 1, "window_target": 1, "window_warps": 4}})
    monkeypatch.setenv("CHL_SCHEDULES", path)
    L = P.build(g, order)
    assert L.stats()["supersteps"] > 3 * ref.stats()["supersteps"]
    for x, y in zip(L.export(), ref.export()):
        assert np.array_equal(x, y)
    # explicit options win over the table
    L2 = P.build(g, order, first_superstep=100000, sf=1e6)
    assert L2.stats()["supersteps"] == 1


def test_shipped_table_is_well_formed():
    """The table shipped beside the library: one line per graph class with
    the seven schedule values chl_build reads."""
    import os
    import re
    from plant_gb300 import autotune as A
    rows = [x.split() for x in open(A.SHIPPED) if x.strip() and not x.startswith("#")]
    assert rows
    for r in rows:
        assert re.fullmatch(r"(sym|dir)-n2\^\d+-deg\d+-skew(heavy|flat)", r[0]) and len(r) == 8
        float(r[2]), float(r[3]), float(r[7])
        assert all(x.isdigit() for x in (r[1], r[4], r[5], r[6]))
