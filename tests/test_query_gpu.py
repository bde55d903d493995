"""Batched distance queries on the GPU vs the reference Labeling::query."""
import numpy as np
import pytest

from conftest import label_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["grid12", "grid20hw", "rmat8", "directed60", "unit_path"])
def test_query_matches_reference_answers(P, case):
    c = label_case(case)
    L = P.Labeling.read(c["labels"])
    pairs = np.loadtxt(c["pairs"], dtype=np.uint32).reshape(-1, 2)
    exp = np.loadtxt(c["dist"], dtype=np.int64)
    got = P.query(L, pairs).astype(np.int64)
    assert np.array_equal(got, exp)


def test_query_large_batch_vs_oracle(P, O):
    g = P.Graph.rmat(13, 16, seed=21)
    order = P.Order.degree(g, seed=1)
    L = P.build(g, order)
    off, hub, dist = L.export()
    ref = O.OLabels.from_csr(g.get_n(), off, hub, dist)
    pairs = P.generate_query(200_000, g.get_n(), seed=3)
    assert np.array_equal(P.query(L, pairs), ref.query(pairs))


def test_query_long_labels(P, O):
    # hand-made labels with long lists to exercise multi-chunk merges
    rng = np.random.default_rng(0)
    n = 50
    lists = []
    for x in range(2 * n):
        k = int(rng.integers(0, 300))
        hubs = np.sort(rng.choice(2000, k, replace=False)).astype(np.uint32)
        d = rng.integers(0, 10**6, k).astype(np.int32)
        lists.append((hubs, d))
    off = np.zeros(2 * n + 1, np.uint64)
    off[1:] = np.cumsum([len(h) for h, _ in lists])
    hub = np.concatenate([h for h, _ in lists])
    dist = np.concatenate([d for _, d in lists])
    L = P.Labeling.from_csr(n, off, hub, dist)
    ref = O.OLabels.from_csr(n, off, hub, dist)
    pairs = np.stack(np.meshgrid(np.arange(n), np.arange(n)), -1).reshape(-1, 2).astype(np.uint32)
    assert np.array_equal(P.query(L, pairs), ref.query(pairs))


def test_query_out_of_range_rejected(P):
    c = label_case("grid12")
    L = P.Labeling.read(c["labels"])
    with pytest.raises(P.CHLError) as e:
        P.query(L, [[0, 10**6]])
    assert e.value.status == P.CHL_ERR_INVALID


def test_empty_batch(P):
    c = label_case("grid12")
    L = P.Labeling.read(c["labels"])
    assert len(P.query(L, np.zeros((0, 2), np.uint32))) == 0
