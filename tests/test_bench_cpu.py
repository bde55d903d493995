"""bench.py host logic that needs no GPU: the committed sequential PLL traces
are found for the benchmark workloads, and they count the labels the GPU
builds of those workloads produced (same graph, same order)."""
import argparse

import pytest


@pytest.mark.parametrize("kw,labels", [
    (dict(workload="grid", side=1024, highways=2000, sources=256, scale=20), 1591229142),
    (dict(workload="grid", side=512, highways=500, sources=256, scale=20), 214724306),
    (dict(workload="rmat", side=1024, highways=2000, sources=256, scale=20), 505364790),
])
def test_committed_trace_matches_workload(kw, labels):
    import bench
    t = bench.profile_trace(argparse.Namespace(**kw))
    assert t is not None
    assert t["labels"] == labels
    assert t["algorithmic_bytes"] == 8 * (t["list_entries"] + t["settled_out_arcs"] + t["labels"])


def test_no_trace_for_other_workloads():
    import bench
    args = argparse.Namespace(workload="grid", side=300, highways=7, sources=256, scale=20)
    assert bench.profile_trace(args) is None
