"""Label / order / query file formats against the reference's layouts."""
import filecmp

import numpy as np
import pytest

from conftest import label_case


@pytest.mark.parametrize("case", ["grid12", "directed60", "rmat8"])
def test_label_file_roundtrip_is_byte_identical(P, case, tmp_path):
    c = label_case(case)
    L = P.Labeling.read(c["labels"])
    out = str(tmp_path / "x.labels")
    L.write(out)
    assert filecmp.cmp(out, c["labels"], shallow=False)


def test_label_read_layout(P, O):
    c = label_case("directed60")
    L = P.Labeling.read(c["labels"])
    lines = open(c["labels"]).read().split("\n")
    n = int(lines[0])
    assert L.n() == n
    for v in (0, 7, n - 1):
        for side in (0, 1):
            h, d = L.label(v, side)
            toks = list(map(int, lines[1 + 2 * v + side].split()))
            assert toks[0] == len(h)
            assert toks[1::2] == list(h) and toks[2::2] == list(d)


def test_avg_label_matches_reference_formula(P):
    c = label_case("grid12")
    L = P.Labeling.read(c["labels"])
    toks = open(c["labels"]).read().split("\n")
    n = int(toks[0])
    total = sum(int(t.split()[0]) for t in toks[1:1 + 2 * n])
    assert abs(L.get_avg() - total / n / 2) < 1e-12


def test_truncated_label_file(P, tmp_path):
    p = tmp_path / "bad.labels"
    p.write_text("3\n1 0 0\n1 0 0\n")
    with pytest.raises(P.CHLError) as e:
        P.Labeling.read(str(p))
    assert e.value.status == P.CHL_ERR_FORMAT


def test_order_roundtrip(P, tmp_path):
    o = np.random.default_rng(1).permutation(1000).astype(np.uint32)
    p = str(tmp_path / "o.order")
    P.Order.write(p, o)
    assert open(p).read().split("\n")[0] == "1000"
    assert np.array_equal(P.Order.read(p), o)


def test_reference_order_file_reads(P):
    c = label_case("grid12")
    o = P.Order.read(c["order"])
    assert sorted(o.tolist()) == list(range(len(o)))


def test_query_file(P, tmp_path):
    p = tmp_path / "q.txt"
    p.write_text("1 2\n3 4\n5 6")
    q = P.load_query(str(p))
    assert q.tolist() == [[1, 2], [3, 4], [5, 6]]
    (tmp_path / "bad.txt").write_text("1\n")
    with pytest.raises(P.CHLError):
        P.load_query(str(tmp_path / "bad.txt"))
