"""Continuous-batching server: each answer is the same alone and in the mix."""
import ctypes as C
import threading
import time

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


def test_unclaimed_requests_do_not_starve_admission(P, labels):
    """A request's pairs leave the admission budget once answered, even if
    its client never waits for it, so later submits are admitted."""
    L, n = labels
    srv = P.Server(L, max_inflight_pairs=1000, max_requests=64, max_batch_pairs=256)
    ids = []
    for i in range(5):
        got = []
        t = threading.Thread(target=lambda: got.append(srv.submit(P.generate_query(800, n, seed=i))), daemon=True)
        t.start()
        t.join(timeout=60)
        assert got, "submit starved by requests nobody waited for"
        ids.append(got[0])
    # the answers are kept for a late wait
    for i, rid in enumerate(ids):
        out, _ = srv.wait(rid, 800)
        assert np.array_equal(out, P.query(L, P.generate_query(800, n, seed=i)))
    srv.close()


def test_free_fails_a_blocked_submit(P, labels):
    """A submit blocked on admission returns CHL_ERR_INVALID when the server
    is freed (the caller is seen blocked before the free)."""
    L, n = labels
    srv = P.Server(L, max_inflight_pairs=1 << 16, max_requests=1, max_batch_pairs=256)
    h = srv._h
    srv.submit(P.generate_query(10, n, seed=1))   # holds the only request entry
    res = []
    q = P.generate_query(10, n, seed=2)

    def blocked():
        rid = C.c_uint64()
        res.append(P.lib().chl_server_submit(h, q.ctypes.data_as(C.POINTER(C.c_uint32)), len(q), C.byref(rid)))

    t = threading.Thread(target=blocked, daemon=True)
    t.start()
    deadline = time.time() + 30
    while srv.blocked() < 1 and time.time() < deadline:
        time.sleep(0.01)
    assert srv.blocked() == 1 and not res, "the second submit should wait for a free entry"
    srv.close()
    t.join(timeout=60)
    assert res == [P.CHL_ERR_INVALID]
