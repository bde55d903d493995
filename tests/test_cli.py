"""The hhl command line: reference flags, messages, byte-identical labels."""
import filecmp
import os
import subprocess

import numpy as np
import pytest

from conftest import label_case, ROOT

HHL = os.path.join(ROOT, "plant_gb300", "hhl")


@pytest.fixture(scope="module")
def hhl(P):
    assert os.path.exists(HHL), "hhl CLI not built"
    return HHL


def test_missing_order_message(hhl, tmp_path):
    c = label_case("grid12")
    r = subprocess.run([hhl, "-g", c["gr"], "-o", str(tmp_path / "none.order")], capture_output=True, text=True)
    assert r.returncode == 1
    assert "ERROR: couldn't open order file named" in r.stdout
    assert r.stdout.startswith(hhl + " -g ")   # argv echo first, as the reference


def test_unreadable_graph_message(hhl, tmp_path):
    c = label_case("grid12")
    bad = tmp_path / "bad.gr"
    bad.write_text("this is not a graph\n")
    r = subprocess.run([hhl, "-g", str(bad), "-o", c["order"], "-p", "2"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "Unable to read graph from raw" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["grid12", "rmat8", "directed60"])
def test_cli_labels_byte_identical(hhl, case, tmp_path):
    c = label_case(case)
    out = str(tmp_path / "cli.labels")
    r = subprocess.run([hhl, "-g", c["gr"], "-o", c["order"], "-p", "4", "-s", "32", "-l", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Average label size after gll is" in r.stdout
    assert filecmp.cmp(out, c["labels"], shallow=False)


@pytest.mark.gpu
def test_cli_query_file(hhl, tmp_path):
    c = label_case("grid20hw")
    r = subprocess.run([hhl, "-g", c["gr"], "-o", c["order"], "-qm", "1", "-rq", c["pairs"]],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().split("\n")
    exp = open(c["dist"]).read().strip().split("\n")
    assert lines[-len(exp):] == exp
