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

    def fake_build(g, order, root_limit=0, first_superstep=0, growth=0.0, sf=0.0, queue_split=0, **kw):
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
    assert cfg == {"first_superstep": 1024, "growth": 2.0, "sf": 128.0, "queue_split": 512}
    assert all(c[0] == max(10, int(0.1 * g.get_n())) for c in calls)
    n_calls = len(calls)
    assert n_calls <= len(A.FIRST) + len(A.GROWTH) + len(A.SF) + len(A.QSPLIT)
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
