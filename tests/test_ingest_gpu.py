"""GPU DIMACS, METIS, SNAP and edge-list ingestion against the host parsers (which
follow the reference's Graph::read and are pinned to it by test_graph_io.py).

Every file must give the same outcome both ways: the same CSRs in both
directions, the same n, m and symmetry, or the same error.  Files the
reference's DIMACS line rules reject must be handed to the host parsers.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def outcome(P, path, undirected, gpu):
    try:
        if gpu:
            g, used = P.Graph.read_gpu(path, undirected)
        else:
            g, used = P.Graph.read(path, undirected), None
    except P.CHLError as e:
        return ("error", e.status), None
    parts = [g.get_n(), g.get_m(), g.symmetric()]
    for fwd in (True, False):
        off, head, ln = g.csr(fwd)
        parts += [off.tolist(), head.tolist(), ln.tolist()]
    return ("ok", parts), used


def same(P, path, undirected=False, expect_gpu=None):
    a, used = outcome(P, path, undirected, True)
    b, _ = outcome(P, path, undirected, False)
    assert a == b, path
    if expect_gpu is not None:
        if a[0] == "error":
            assert not expect_gpu, path   # errors come from the host parsers
        else:
            assert used == expect_gpu, path
    return a


GOLDEN_GR = sorted(p for ext in ("gr", "txt", "graph")
                   for p in glob.glob(os.path.join(GOLDEN, "**", "*." + ext), recursive=True))


@pytest.mark.parametrize("path", GOLDEN_GR, ids=[os.path.basename(p) for p in GOLDEN_GR])
@pytest.mark.parametrize("undirected", [False, True])
def test_golden_dimacs_files(P, path, undirected):
    # some fixtures are deliberately malformed (the reference rejects them):
    # only the agreement of the two paths is required
    same(P, path, undirected)


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_bytes(text.encode() if isinstance(text, str) else text)
    return str(p)


def test_quirks(P, tmp_path):
    base = "p sp 4 5\na 1 2 7\na 2 3 1\na 3 4 2\na 4 1 9\na 1 2 3\n"
    cases = {
        "plain": (base, True),
        "crlf": (base.replace("\n", "\r\n"), True),
        "comments": ("c hello\n" + base + "c " + "x" * 700 + "\n", True),
        "signs_tabs": ("p sp 4 2\na\t+1  2\t 5\na 3 4 -2\n", True),
        "dup_both_dirs": ("p sp 3 4\na 1 2 5\na 2 1 5\na 1 2 4\na 1 2 4\n", True),
        "self_loop": ("p sp 2 2\na 1 1 3\na 1 2 1\n", True),
        "empty": ("", True),
        "only_comment": ("c nothing\n", True),
        "no_final_newline": (base[:-1], False),
        "long_arc_line": ("p sp 4 1\na 1 2 " + " " * 600 + "3\n", False),
        "arc_before_p": ("a 1 2 3\np sp 4 1\n", False),
        "two_p": ("p sp 4 1\np sp 4 1\na 1 2 3\n", False),
        "blank_line": ("p sp 4 1\n\na 1 2 3\n", False),
        "out_of_range": ("p sp 2 1\na 1 3 1\n", False),
        "bad_token": ("p sp 2 1\na 1 x 1\n", False),
        "nul_byte": (b"p sp 2 1\na 1 2 1\x00\n", False),
        "huge_number": ("p sp 2 1\na 1 2 1234567890123456789012\n", False),
        "edgelist_like": ("0 1 5\n1 2 3\n", True),   # an edge list: read on the GPU as one
    }
    for name, (text, on_gpu) in cases.items():
        p = write(tmp_path, name + ".gr", text)
        for und in (False, True):
            same(P, p, und, expect_gpu=on_gpu)


def test_random_files_and_large_grid(P, tmp_path):
    rng = np.random.default_rng(3)
    for t in range(6):
        n = int(rng.integers(2, 300))
        k = int(rng.integers(1, 3000))
        u = rng.integers(1, n + 1, k)
        v = rng.integers(1, n + 1, k)
        w = rng.integers(-5 if t % 3 == 0 else 1, 60, k)
        lines = [f"c random {t}", f"p sp {n} {k}"] + [f"a {a} {b} {c}" for a, b, c in zip(u, v, w)]
        p = write(tmp_path, f"r{t}.gr", "\n".join(lines) + "\n")
        for und in (False, True):
            same(P, p, und, expect_gpu=True)
    g = P.Graph.grid(300, 300, highways=100, seed=4)
    p = str(tmp_path / "grid.gr")
    g.write(p)
    r = same(P, p, False, expect_gpu=True)
    assert r[0] == "ok" and r[1][0] == g.get_n()


def test_snap_quirks(P, tmp_path):
    # files whose first non-blank byte is '#' are parsed on the GPU as SNAP;
    # the ones the reference's SNAP rules reject go to the host parsers,
    # which report the error
    hdr = "# Nodes: 4 Edges: 3\n"
    cases = {
        "plain": (hdr + "0 1\n1 2\n2 3\n", True),
        "tabs_crlf_junk": ("# Nodes:\t4   Edges: 3\r\n0\t1\r\n1 2 junk\r\n2 3\r\n", True),
        "comments_no_final_newline": ("# title\n#Nodes:3 Edges:2\n# more\n0 1\n1 2", True),
        "dups_and_loops": (hdr + "0 1\n1 0\n0 1\n2 2\n3 0\n", True),
        "signs": (hdr + "+0 +2\n", True),
        "truncated_ids": (hdr + "4294967297 2\n", True),
        "long_comment": ("# " + "x" * 700 + "\n" + hdr + "0 2\n", True),
        "long_header_line": ("# Nodes: 4 Edges: 1" + " " * 600 + "\n0 2\n", True),
        "hash_only": ("#\n", True),
        "no_header": ("# hello\n0 1\n", False),
        "two_headers": (hdr + hdr + "0 1\n", False),
        "header_after_arc": ("# x\n0 1\n" + hdr, False),
        "out_of_range": (hdr + "0 5\n", False),
        "negative": (hdr + "-1 2\n", False),
        "one_number": (hdr + "0\n", False),
        "empty_line": (hdr + "\n0 2\n", False),
        "long_data_line": (hdr + "0 " + " " * 600 + "2\n", False),
        "leading_blank_line": ("  \n" + hdr + "0 2\n", False),
        "nul_byte": (("# Nodes: 4 Edges: 1\n0 1\x00\n").encode(), False),
        "huge_number": (hdr + "0 1234567890123456789012\n", False),
    }
    for name, (text, on_gpu) in cases.items():
        p = write(tmp_path, name + ".txt", text)
        for und in (False, True):
            same(P, p, und, expect_gpu=on_gpu)


def test_random_snap_files(P, tmp_path):
    rng = np.random.default_rng(5)
    for t in range(6):
        n = int(rng.integers(2, 400))
        k = int(rng.integers(1, 4000))
        u = rng.integers(0, n, k)
        v = rng.integers(0, n, k)
        lines = ["# Directed graph (each unordered pair of nodes is saved once)",
                 f"# Nodes: {n} Edges: {k}", "# FromNodeId\tToNodeId"]
        lines += [f"{a}\t{b}" for a, b in zip(u, v)]
        p = write(tmp_path, f"s{t}.txt", "\n".join(lines) + ("\n" if t % 2 else ""))
        for und in (False, True):
            r = same(P, p, und, expect_gpu=True)
            assert r[0] == "ok" and r[1][0] == n


def test_edgelist_quirks(P, tmp_path):
    # a file DIMACS and SNAP reject on its first line is an edge list when the
    # host's METIS reader rejects a prefix of it
    cases = {
        "plain": ("0 1 5\n1 2 3\n2 0 4\n", True),
        "unit_weights": ("0 1 1\n1 2 1\n2 0 1\n", True),
        "no_final_newline": ("0 1 5\n1 0 2", True),
        "crlf_tabs": ("0\t1\t5\r\n1 0 2\r\n", True),
        "trailing_comment": ("0 1 5 % comment\n", True),
        "ids_past_32_bits": ("4294967296 1 5\n1 4294967296 2\n", True),
        "leading_space": (" 0 1 5\n1 0 2\n", True),
        "loops_and_dups": ("0 0 3\n0 1 5\n0 1 2\n1 0 7\n", True),
        "weight_10": ("0 1 10\n1 0 11\n", True),
        "negative_weight": ("0 1 -4\n1 0 2\n", True),
        "negative_id": ("-1 0 3\n0 1 2\n", False),
        "blank_line": ("0 1 5\n\n1 0 2\n", False),
        "long_line": ("0 1 " + " " * 600 + "5\n", False),
        "sparse_ids": ("0 1 5\n1 7 3\n", False),
        "nul_byte": (b"0 1 5\x00\n1 0 2\n", False),
        "huge_number": ("0 1 5\n1 0 1234567890123456789012\n", False),
    }
    for name, (text, on_gpu) in cases.items():
        p = write(tmp_path, name + ".txt", text)
        for und in (False, True):
            same(P, p, und, expect_gpu=on_gpu)


def test_random_edgelist_files(P, tmp_path):
    rng = np.random.default_rng(9)
    for t in range(6):
        n = int(rng.integers(2, 500))
        k = int(rng.integers(n, 5000))
        ids = np.concatenate([np.arange(n), rng.integers(0, n, 2 * k - n)])
        rng.shuffle(ids)
        u, v = ids[:k], ids[k:]
        w = rng.integers(-3 if t % 3 == 0 else 1, 100, k)
        w[0] = int(rng.integers(2, 10))   # a first line METIS rejects (format code w)
        lines = [f"{a} {b} {c}" for a, b, c in zip(u, v, w)]
        p = write(tmp_path, f"e{t}.txt", "\n".join(lines) + ("\n" if t % 2 else ""))
        for und in (False, True):
            r = same(P, p, und, expect_gpu=True)
            assert r[0] == "ok" and r[1][0] == n


def test_metis_on_gpu(P, tmp_path):
    """METIS files are read on the GPU (comment lines included); a comment
    after a number, which joins two lines in the reference's reader, and
    files whose header the reference rejects are left to the host."""
    cases = {
        "empty_weighted": ("0 5 1\n", True),
        "two_numbers": ("0 1\n", True),
        "plain": ("3 2\n2\n1 3\n2\n", True),
        "comments": ("% a METIS file\n%\n3 2\n  % indented comment\n2\n1 3\n% last\n2\n", True),
        "arc_lengths": ("3 3 1\n2 7 3 4\n1 7\n1 4\n", True),
        "vertex_sizes": ("3 2 100\n5 2\n6 1 3\n7 2\n", True),
        "vertex_weights_ncon": ("3 2 11 2\n1 1 2 5\n1 1 1 5 3 6\n1 1 2 6\n", True),
        "all_fields": ("3 2 111 1\n9 1 2 5\n9 1 1 5 3 6\n9 1 2 6\n", True),
        "no_final_newline": ("3 2\n2\n1 3\n2", True),
        "crlf_tabs": ("3 2\r\n2\r\n1\t3\r\n2\r\n", True),
        "blank_lines": ("4 1\n2\n1\n\n\n", True),
        "long_line": ("3 3\n2 3" + " " * 900 + "\n1 3\n1 2\n", True),
        "comment_after_number": ("3 2\n2 % x\n1 3\n2\n", False),
        "bad_fmt": ("3 2 2\n2\n1 3\n2\n", False),
        "missing_length": ("3 3 1\n2\n1 7\n1 4\n", False),
        "too_many_lines": ("2 1\n2\n1\n1\n", False),
        "stray_byte": ("3 2\n2\n1 x\n2\n", False),
    }
    for name, (text, on_gpu) in cases.items():
        p = write(tmp_path, name + ".graph", text)
        for und in (False, True):
            same(P, p, und, expect_gpu=on_gpu)


def test_fuzz_files_agree(P, tmp_path):
    """The 400 seeded edge-case files of the parser fuzz (every format): the
    GPU path and the host parsers give the same graph or the same error."""
    from test_graph_io import _fuzz_files
    for i, data in enumerate(_fuzz_files(2024, 400)):
        p = write(tmp_path, f"z{i}.txt", data)
        for und in (False, True):
            same(P, p, und)
