"""Pin the CPU oracle to the reference.

* golden fixtures: label files printed by the reference GLL binary
  (shared_memory/hhl) and answers of the reference Labeling::query, made by
  tests/golden/make_golden.py -- the oracle must reproduce them exactly;
* live reference (only where oracle/_ref was built from the reference
  sources): labels of a fresh config-1-style graph, byte for byte;
* canonical definition by brute force, and plain Dijkstra on sampled pairs.
"""
import filecmp
import os
import subprocess

import numpy as np
import pytest

from conftest import label_case

CASES = ["grid12", "grid20hw", "rmat8", "directed60", "unit_path"]


@pytest.mark.parametrize("case", CASES)
def test_oracle_gll_reproduces_reference_labels(O, case, tmp_path):
    c = label_case(case)
    og = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    L, _ = O.gll(og, order, threads=4)
    out = str(tmp_path / "o.labels")
    L.write(out)
    assert filecmp.cmp(out, c["labels"], shallow=False)


@pytest.mark.parametrize("case", CASES)
def test_oracle_plant_equals_gll(O, case):
    c = label_case(case)
    og = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    a, _ = O.gll(og, order, threads=2)
    b, ts, lc = O.plant_all(og, order)
    n = len(order)
    for x, y in zip(a.export(n), b.export(n)):
        assert np.array_equal(x, y)
    assert (ts >= lc).all() and (lc >= 2).all()   # root labels itself on both sides


@pytest.mark.parametrize("case", CASES)
def test_oracle_query_matches_reference_query(O, case):
    c = label_case(case)
    og = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    L, _ = O.gll(og, order, threads=2)
    pairs = np.loadtxt(c["pairs"], dtype=np.uint32).reshape(-1, 2)
    exp = np.loadtxt(c["dist"], dtype=np.int64)
    assert np.array_equal(L.query(pairs).astype(np.int64), exp)


@pytest.mark.parametrize("case", ["grid12", "rmat8", "directed60", "unit_path"])
def test_oracle_labels_are_canonical(O, case):
    c = label_case(case)
    og = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    L, _ = O.gll(og, order, threads=2)
    assert O.canonical_check(og, order, L) == 0


def test_planted_mistake_is_caught(O):
    """A label removed from the oracle's output must fail the canonical check."""
    c = label_case("grid12")
    og = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    L, _ = O.gll(og, order, threads=2)
    n = len(order)
    off, hub, dist = L.export(n)
    dist = dist.copy()
    dist[len(dist) // 2] += 1
    bad = O.OLabels.from_csr(n, off, hub, dist)
    assert O.canonical_check(og, order, bad) > 0


def test_oracle_queries_equal_dijkstra(O):
    c = label_case("grid20hw")
    og = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    L, _ = O.gll(og, order, threads=2)
    rng = np.random.default_rng(0)
    for s in rng.integers(0, og.n, 10):
        d = og.dijkstra(int(s))
        pairs = np.stack([np.full(og.n, s), np.arange(og.n)], 1)
        assert np.array_equal(L.query(pairs), d)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "hhl")),
                    reason="reference binary not built here (needs the reference sources)")
def test_oracle_matches_live_reference_config1(P, O, tmp_path):
    g = P.Graph.grid(100, 100, seed=1)
    gp = str(tmp_path / "g.gr")
    g.write(gp)
    og = O.OGraph.read_dimacs(gp)
    order = og.degree_order(1)
    op = str(tmp_path / "g.order")
    P.Order.write(op, order)
    ref = str(tmp_path / "ref.labels")
    subprocess.run([O.ref_bin("hhl"), "-g", gp, "-o", op, "-p", "4", "-l", ref], check=True,
                   capture_output=True)
    L, _ = O.gll(og, order, threads=4)
    out = str(tmp_path / "orc.labels")
    L.write(out)
    assert filecmp.cmp(out, ref, shallow=False)


@pytest.mark.parametrize("case", CASES)
def test_pll_trace_builds_the_canonical_labels(O, case):
    """The sequential PLL behind the build roofline's work counts produces
    the reference's labels (the same count as the GLL restatement), and its
    counters are consistent."""
    c = label_case(case)
    g = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    ref, _ = O.gll(g, order, threads=2)
    tr = O.pll_trace(g, order)
    assert tr["labels"] == ref.total()
    assert tr["label_reads"] <= tr["list_entries"] and tr["arcs"] <= tr["settled_out_arcs"]
    assert tr["settled"] >= tr["labels"]
    assert tr["algorithmic_bytes"] == 8 * (tr["list_entries"] + tr["settled_out_arcs"] + tr["labels"])
    assert tr["scanned_bytes"] == 8 * (tr["label_reads"] + tr["arcs"] + tr["labels"])
