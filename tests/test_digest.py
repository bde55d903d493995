"""Label / order / graph digests (oracle/chl_digest.h), pinned to the reference.

The benchmark-scale parity test compares GPU builds with digests of the
reference's own labels (tests/golden/scale_digests.json, made by
tests/golden/make_scale_digests.py through oracle/_ref/ref_digest).  These
CPU tests pin the digest itself:
  * the C oracle's digest equals the NumPy restatement, and both equal the
    digest of the reference's golden label files;
  * where oracle/_ref was built, ref_digest (the reference's run_paraPLL)
    prints the digest of the golden label file;
  * the committed config-1 entry (100 x 100 grid) is reproduced by the
    oracle's GLL restatement and the package's seeded generator.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, label_case
from tests.golden import digests as D

CASES = ["grid12", "grid20hw", "rmat8", "directed60", "unit_path"]


def read_label_file(path):
    """hl::Labeling::write's text (shared_memory/labeling.hpp:167-183) as CSR."""
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    p = 1
    off = [0]
    hub, dist = [], []
    for _ in range(2 * n):
        s = int(tok[p])
        p += 1
        vals = np.array(tok[p:p + 2 * s], dtype=np.int64)
        p += 2 * s
        hub.append(vals[0::2])
        dist.append(vals[1::2])
        off.append(off[-1] + s)
    return n, np.array(off, np.uint64), np.concatenate(hub), np.concatenate(dist)


@pytest.mark.parametrize("case", CASES)
def test_digest_of_reference_files(O, case):
    c = label_case(case)
    n, off, hub, dist = read_label_file(c["labels"])
    want = D.label_digest(n, off, hub, dist)
    og = O.OGraph.read_dimacs(c["gr"])
    order = np.loadtxt(c["order"], dtype=np.uint32)[1:]
    L, _ = O.gll(og, order, threads=2)
    assert L.digest() == want
    assert O.order_digest(order) == D.order_digest(order)


def test_digest_is_position_dependent(O):
    c = label_case("grid12")
    n, off, hub, dist = read_label_file(c["labels"])
    base = D.label_digest(n, off, hub, dist)
    # swap two entries of one list: same multiset, other positions
    k = int(off[3])
    h2, d2 = hub.copy(), dist.copy()
    h2[[k, k + 1]] = h2[[k + 1, k]]
    d2[[k, k + 1]] = d2[[k + 1, k]]
    assert D.label_digest(n, off, h2, d2) != base
    # move an entry to the next list
    off2 = off.copy()
    off2[4] += 1
    assert D.label_digest(n, off2, hub, dist) != base
    d3 = dist.copy()
    d3[5] += 1
    assert D.label_digest(n, off, hub, d3) != base


@pytest.mark.parametrize("case", ["grid12", "rmat8", "directed60"])
def test_ref_digest_harness(O, case):
    exe = O.ref_bin("ref_digest")
    if exe is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    c = label_case(case)
    r = subprocess.run([exe, c["gr"], c["order"], "2"], capture_output=True, text=True, check=True)
    line = [x for x in r.stdout.splitlines() if x.startswith("digest ")][-1].split()
    n, off, hub, dist = read_label_file(c["labels"])
    assert int(line[1], 16) == D.label_digest(n, off, hub, dist)


def test_scale_digest_config1_reproduced(P, O):
    with open(os.path.join(GOLDEN, "scale_digests.json")) as f:
        ref = json.load(f)["grid100"]
    g = P.Graph.grid(100, 100, del_frac=0.05, diag_frac=0.01, wmin=1, wmax=1000, seed=1)
    off, head, ln = g.csr(True)
    assert g.get_n() == ref["n"]
    assert f"{D.graph_digest(g.get_n(), off, head, ln):016x}" == ref["graph_digest"]
    og = O.OGraph.from_csr(g.get_n(), off, head, ln)
    order = og.degree_order(ref["order"]["seed"])
    assert f"{O.order_digest(order):016x}" == ref["order_digest"]
    L, _ = O.gll(og, order, threads=4)
    assert f"{L.digest():016x}" == ref["labels_digest"]
    assert L.total() == ref["labels_total"]
