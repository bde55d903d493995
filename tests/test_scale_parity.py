"""GPU builds at benchmark scale against the reference's own labels.

tests/golden/scale_digests.json holds, per workload, digests of the graph,
of the CPU oracle's plain order and of the labels built by the reference's
run_paraPLL (shared_memory/akiba.hpp:132-217, as shared_memory/hhl.cpp:65
calls it), made by tests/golden/make_scale_digests.py.  Here the same
graph is generated, the order is computed on the GPU, the labels are built
on the GPU, and their digest is computed on the device (chl_labels_digest):
equal digests mean the label files would be byte-identical.

Workloads: the 100 x 100 grid (degree order), the 1024 x 1024 grid with
2,000 highways (256-source betweenness order), and RMAT scale 20 (degree
order) -- the benchmark's two 1M-vertex graphs.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from tests.golden import digests as D

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "scale_digests.json")) as _f:
    REF = json.load(_f)


def make_graph(P, gen):
    if gen["kind"] == "grid":
        return P.Graph.grid(gen["rows"], gen["cols"], del_frac=0.05, diag_frac=0.01, wmin=1, wmax=1000,
                            highways=gen.get("highways", 0), hw_steps=gen.get("hw_steps", 64),
                            hw_factor=gen.get("hw_factor", 150.0), seed=gen["seed"])
    return P.Graph.rmat(gen["scale"], gen["ef"], gen["a"], gen["b"], gen["c"], seed=gen["seed"])


def gpu_order(P, g, spec):
    if spec["kind"] == "degree":
        return P.Order.degree(g, seed=spec["seed"])
    assert spec["kind"] == "betweenness256"
    return P.Order.betweenness(g, 256, seed=spec["seed"])


_cache = {}


def workload(P, name):
    if name not in _cache:
        _cache.clear()
        ref = REF[name]
        g = make_graph(P, ref["generator"])
        off, head, ln = g.csr(True)
        assert g.get_n() == ref["n"]
        assert f"{D.graph_digest(g.get_n(), off, head, ln):016x}" == ref["graph_digest"], "generator differs"
        order = gpu_order(P, g, ref["order"])
        assert f"{D.order_digest(order):016x}" == ref["order_digest"], "GPU order differs from the oracle's"
        g.to_device()
        _cache[name] = (g, order)
    return _cache[name]


CASES = [("grid100", "hybrid"), ("grid100", "gll"), ("grid100", "plant"),
         ("grid1024_hw2000_bc256", "hybrid"), ("rmat20", "hybrid"), ("rmat20", "gll")]


@pytest.mark.parametrize("name,mode", CASES)
def test_labels_digest_equals_reference(P, name, mode):
    if name not in REF:
        pytest.skip(f"{name}: no reference digest committed")
    ref = REF[name]
    g, order = workload(P, name)
    L = P.build(g, order, mode={"hybrid": P.MODE_HYBRID, "gll": P.MODE_GLL, "plant": P.MODE_PLANT}[mode])
    st = L.stats()
    assert st["labels"] == ref["labels_total"]
    assert f"{L.digest():016x}" == ref["labels_digest"]


@pytest.mark.parametrize("kind", ["grid", "directed"])
def test_device_digest_equals_host_digest(P, kind):
    if kind == "grid":
        g = P.Graph.grid(40, 40, highways=20, hw_steps=10, seed=9)
    else:
        rng = np.random.default_rng(3)
        src = rng.integers(0, 500, 3000, dtype=np.uint32)
        dst = rng.integers(0, 500, 3000, dtype=np.uint32)
        keep = src != dst
        g = P.Graph.from_arcs(500, src[keep], dst[keep], rng.integers(1, 9, 3000, dtype=np.int32)[keep])
    order = P.Order.degree(g, seed=4)
    L = P.build(g, order)
    off, hub, dist = L.export()
    assert L.digest() == D.label_digest(g.get_n(), off, hub, dist)
