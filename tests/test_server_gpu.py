"""Continuous-batching server: each answer is the same alone and in the mix."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def labels(P):
    g = P.Graph.rmat(12, 16, seed=8)
    order = P.Order.degree(g, seed=8)
    return P.build(g, order), g.get_n()


def test_alone_equals_mixed(P, labels):
    L, n = labels
    rng = np.random.default_rng(5)
    reqs = [P.generate_query(int(k), n, seed=int(s)) for k, s in
            zip(rng.integers(1, 5000, 40), rng.integers(0, 10**9, 40))]
    # alone: one request in the server at a time
    srv = P.Server(L, max_inflight_pairs=1 << 16, max_batch_pairs=1 << 12)
    alone = []
    for r in reqs:
        rid = srv.submit(r)
        alone.append(srv.wait(rid, len(r))[0])
    # mixed: many client threads submitting at once
    mixed = [None] * len(reqs)

    def client(i):
        rid = srv.submit(reqs[i])
        mixed[i] = srv.wait(rid, len(reqs[i]))[0]

    th = [threading.Thread(target=client, args=(i,)) for i in range(len(reqs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for a, m, r in zip(alone, mixed, reqs):
        assert np.array_equal(a, m)
        assert np.array_equal(a, P.query(L, r))
    st = srv.stats()
    assert st["requests"] == 2 * len(reqs)
    srv.close()


def test_admission_limits(P, labels):
    L, n = labels
    srv = P.Server(L, max_inflight_pairs=1000, max_batch_pairs=256)
    with pytest.raises(P.CHLError) as e:
        srv.submit(P.generate_query(1001, n))
    assert e.value.status == P.CHL_ERR_OOM
    # a request larger than one batch is split across launches
    q = P.generate_query(1000, n, seed=2)
    rid = srv.submit(q)
    out, lat = srv.wait(rid, 1000)
    assert np.array_equal(out, P.query(L, q)) and lat >= 0
    assert srv.stats()["launches"] >= 4
    srv.close()


def test_wait_timeout_and_unknown_id(P, labels):
    L, n = labels
    srv = P.Server(L)
    with pytest.raises(P.CHLError) as e:
        srv.wait(12345, 1)
    assert e.value.status == P.CHL_ERR_INVALID
    srv.close()
