"""chl_query_batch_noalloc: the query entry point that allocates nothing.

It exists for callers that cannot let the library allocate device memory
(their HBM is already divided up by their own pool allocator, or their
request loop cannot afford cudaMalloc/cudaFree and the synchronisation they
imply).  It stages pairs and answers through one fixed device array instead.
These tests call it through the C ABI and check that two calls in a row give
exactly the answers of the allocating chl_query_batch.  The file is named so
pytest collects it last; it must also pass alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import label_case

pytestmark = pytest.mark.gpu

U32P = C.POINTER(C.c_uint32)
I32P = C.POINTER(C.c_int32)


def resident_labels(P):
    g = P.Graph.rmat(11, 16, seed=31)
    order = P.Order.degree(g, seed=31)
    return P.build(g, order), g.get_n()   # a build leaves the labels in device memory


def call(lib, fn, L, pairs):
    p = np.ascontiguousarray(pairs, np.uint32)
    out = np.full(len(p), -7, np.int32)
    rc = getattr(lib, fn)(L._h, p.ctypes.data_as(U32P), len(p), out.ctypes.data_as(I32P), None)
    return rc, out


def test_noalloc_matches_allocating_entry_point_twice(P):
    lib = P.lib()
    L, n = resident_labels(P)
    for seed in (1, 2):   # two calls in a row reuse the same device array
        pairs = P.generate_query(50_000 + 1000 * seed, n, seed=seed)
        rc_a, exp = call(lib, "chl_query_batch", L, pairs)
        rc_b, got = call(lib, "chl_query_batch_noalloc", L, pairs)
        assert rc_a == P.CHL_OK and rc_b == P.CHL_OK
        assert np.array_equal(got, exp)


def test_noalloc_large_then_small_batch(P):
    lib = P.lib()
    L, n = resident_labels(P)
    big = P.generate_query(1 << 20, n, seed=5)            # the maximum size
    small = P.generate_query(17, n, seed=6)
    for pairs in (big, small):
        rc_a, exp = call(lib, "chl_query_batch", L, pairs)
        rc_b, got = call(lib, "chl_query_batch_noalloc", L, pairs)
        assert rc_a == rc_b == P.CHL_OK
        assert np.array_equal(got, exp)


def test_noalloc_rejects_oversize_and_nonresident(P):
    lib = P.lib()
    L, n = resident_labels(P)
    too_many = np.zeros(((1 << 20) + 1, 2), np.uint32)
    rc, _ = call(lib, "chl_query_batch_noalloc", L, too_many)
    assert rc == P.CHL_ERR_INVALID
    fresh = P.Labeling.read(label_case("grid12")["labels"])   # host-only until first use
    rc, _ = call(lib, "chl_query_batch_noalloc", fresh, [[0, 1]])
    assert rc == P.CHL_ERR_INVALID
    P.query(fresh, [[0, 1]])                                 # the allocating call uploads them
    rc, got = call(lib, "chl_query_batch_noalloc", fresh, [[0, 1], [3, 2]])
    assert rc == P.CHL_OK
    assert np.array_equal(got, P.query(fresh, [[0, 1], [3, 2]]))
