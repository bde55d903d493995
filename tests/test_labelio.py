"""Label files at scale: GPU-formatted text and the binary CSR twin.

The text written from HBM must be byte-identical to the host writer's (which
the golden tests pin to the reference's own files); the binary file must
round-trip exactly and reject malformed input.
"""
import filecmp
import struct

import numpy as np
import pytest

from conftest import label_case


def host_copy(P, L):
    off, hub, dist = L.export()
    return P.Labeling.from_csr(L.n(), off, hub, dist)


def parse_binary(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"CHLLBL01"
    n, sym, total, nl = struct.unpack_from("<IIQQ", raw, 8)
    off = np.frombuffer(raw, np.uint64, nl + 1, 32)
    ent = np.frombuffer(raw, np.uint32, 2 * total, 32 + 8 * (nl + 1)).reshape(-1, 2)
    assert len(raw) == 32 + 8 * (nl + 1) + 8 * total
    return n, sym, off, ent


@pytest.mark.parametrize("case", ["grid20hw", "directed60"])
def test_binary_layout_from_host_labels(P, case, tmp_path):
    """No GPU needed: labels read from a text file live in host memory."""
    L = P.Labeling.read(label_case(case)["labels"])
    p = str(tmp_path / "l.bin")
    L.save(p)
    n, sym, off, ent = parse_binary(p)
    o2, hub, dist = L.export()
    assert n == L.n()
    if sym:
        # one stored side: lists v
        for v in range(n):
            a, b = int(o2[2 * v]), int(o2[2 * v + 1])
            assert np.array_equal(ent[off[v]:off[v + 1], 0], hub[a:b])
            assert np.array_equal(ent[off[v]:off[v + 1], 1].astype(np.int32), dist[a:b])
    else:
        assert np.array_equal(off, o2)
        assert np.array_equal(ent[:, 0], hub) and np.array_equal(ent[:, 1].astype(np.int32), dist)


GRAPHS = {
    "grid": lambda P: P.Graph.grid(60, 60, highways=30, hw_steps=16, seed=4),
    "rmat": lambda P: P.Graph.rmat(11, 16, seed=8),
    "directed": lambda P: P.Graph.read(label_case("directed60")["gr"]),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GRAPHS))
def test_gpu_text_equals_host_text(P, name, tmp_path):
    g = GRAPHS[name](P)
    order = P.Order.degree(g, seed=3)
    L = P.build(g, order)
    a, b = str(tmp_path / "gpu.txt"), str(tmp_path / "host.txt")
    L.write(a)                      # device-resident: formatted on the GPU
    host_copy(P, L).write(b)        # host-resident: the host writer
    assert filecmp.cmp(a, b, shallow=False)
    back = P.Labeling.read(a).export()
    for x, y in zip(back, L.export()):
        assert np.array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GRAPHS))
def test_binary_round_trip(P, name, tmp_path):
    g = GRAPHS[name](P)
    order = P.Order.degree(g, seed=3)
    L = P.build(g, order)
    p = str(tmp_path / "l.bin")
    L.save(p)
    M = P.Labeling.load(p)
    for x, y in zip(M.export(), L.export()):
        assert np.array_equal(x, y)
    assert M.get_avg() == pytest.approx(L.get_avg())
    pairs = P.generate_query(20000, g.get_n(), seed=2)
    assert np.array_equal(P.query(M, pairs), P.query(L, pairs))
    # host-resident labels save the same bytes
    q = str(tmp_path / "h.bin")
    host_copy(P, L).save(q)
    assert filecmp.cmp(p, q, shallow=False)


@pytest.mark.gpu
def test_binary_load_rejects_malformed(P, tmp_path):
    g = P.Graph.grid(20, 20, seed=2)
    L = P.build(g, P.Order.degree(g, seed=1))
    p = tmp_path / "l.bin"
    L.save(str(p))
    raw = bytearray(p.read_bytes())
    n, sym, total, nl = struct.unpack_from("<IIQQ", raw, 8)
    cases = {
        "magic": b"XHLLBL01" + raw[8:],
        "truncated": raw[:-8],
        "short offsets": raw[:40],
    }
    # a list out of hub order
    ent0 = 32 + 8 * (nl + 1)
    off = np.frombuffer(bytes(raw), np.uint64, nl + 1, 32)
    x = int(np.argmax(np.diff(off) >= 2))
    k = ent0 + 8 * int(off[x])
    swapped = bytearray(raw)
    swapped[k:k + 8], swapped[k + 8:k + 16] = raw[k + 8:k + 16], raw[k:k + 8]
    cases["unsorted"] = swapped
    # a negative distance
    neg = bytearray(raw)
    struct.pack_into("<i", neg, k + 4, -5)
    cases["negative"] = neg
    # offsets that overrun the entries
    over = bytearray(raw)
    struct.pack_into("<Q", over, 32 + 8 * nl, total + 1)
    cases["overrun"] = over
    for what, data in cases.items():
        q = tmp_path / f"bad_{what.replace(' ', '_')}.bin"
        q.write_bytes(bytes(data))
        with pytest.raises(P.CHLError) as e:
            P.Labeling.load(str(q))
        assert e.value.status in (P.CHL_ERR_FORMAT,), what


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GRAPHS))
def test_export_paths_agree(P, name):
    """chl_labels_export of labels in HBM (fetched to host memory by the
    call) equals a second export of the same, now host-resident, labels."""
    g = GRAPHS[name](P)
    order = P.Order.degree(g, seed=3)
    L = P.build(g, order)
    first = L.export()
    L.label(0, 0)                   # fetches the labels to host memory
    second = L.export()             # expanded on the host
    for x, y in zip(first, second):
        assert np.array_equal(x, y)
    assert int(first[0][-1]) == len(first[1]) == L.total()
