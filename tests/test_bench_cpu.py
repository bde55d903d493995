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


def test_oracle_generators_equal_the_package_generators(P, O):
    """The reference arm builds its workload with the oracle's restatement of
    the seeded generators: the graphs must be the package's, arc for arc."""
    from tests.golden import digests as D
    for args in [(30, 30, 0.05, 0.01, 1, 1000, 20, 10, 150.0, 5), (64, 48, 0.1, 0.05, 3, 50, 40, 12, 150.0, 9)]:
        g = P.Graph.grid(args[0], args[1], del_frac=args[2], diag_frac=args[3], wmin=args[4], wmax=args[5],
                         highways=args[6], hw_steps=args[7], hw_factor=args[8], seed=args[9])
        og = O.OGraph.grid(*args)
        assert D.graph_digest(g.get_n(), *g.csr(True)) == D.graph_digest(og.n, *og.csr(1))
    g = P.Graph.rmat(11, 16, 0.57, 0.19, 0.19, seed=3)
    og = O.OGraph.rmat(11, 16, 0.57, 0.19, 0.19, 3)
    assert D.graph_digest(g.get_n(), *g.csr(True)) == D.graph_digest(og.n, *og.csr(1))


def test_superstep_replays_reproduce_the_build(O):
    """Replaying every recorded superstep from its committed state keeps
    exactly the labels the whole build kept."""
    import numpy as np
    og = O.OGraph.grid(60, 60, 0.05, 0.01, 1, 1000, 10, 16, 150.0, 2)
    order = og.betweenness_order(32, 2)
    L, secs, ends, step_secs = O.gll_steps(og, order, 4, sf=2)
    assert len(ends) > 3 and ends[-1] == og.n and len(step_secs) == len(ends)
    starts = np.concatenate([[0], ends[:-1]])
    rp = O.Replay(og, order, L, 4)
    kept = sum(rp.run(int(a), int(a), int(b))[0] for a, b in zip(starts, ends))
    assert kept == L.total()


def test_pps_sample_is_unbiased_on_known_sizes():
    import numpy as np
    import bench
    rng = np.random.default_rng(0)
    sizes = np.array([5.0, 1.0, 0.5, 3.0, 0.1, 2.0, 0.0])
    times = sizes * np.linspace(0.5, 1.5, len(sizes))   # time per unit size drifts over the build
    for target, strata in ((2.0, 1), (6.0, 3), (100.0, 6)):
        est = []
        for _ in range(4000):
            plan = bench.pps_sample(sizes, target, rng)
            assert len(plan) <= strata
            assert all(sizes[i] > 0 for i, _ in plan)
            est.append(sum(times[i] / pi for i, pi in plan))
        assert abs(np.mean(est) / times.sum() - 1) < 0.02
    # every live superstep once when the target affords them all: exact
    plan = bench.pps_sample(sizes, 100.0, rng)
    assert sorted(i for i, _ in plan) == [0, 1, 2, 3, 4, 5] and all(pi == 1.0 for _, pi in plan)


def test_reference_arm_loads_no_product_code(tmp_path):
    """bench.py --impl reference runs the oracle only: no plant_gb300 import,
    no libchl.so mapped, and a line with the reference fields."""
    import json
    import os
    import subprocess
    import sys
    from conftest import ROOT
    code = (
        "import sys, json, bench\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--side', '40', '--highways', '4', '--sources', '16',"
        " '--steps', '2', '--warmup', '1', '--cpu-seconds', '0.2']\n"
        "bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'plant_imported': 'plant_gb300' in sys.modules, 'libchl_mapped': 'libchl' in maps}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[-1]
    assert line["impl"] == "reference" and line["value"] > 0 and line["config"]["same_config"]
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert 0.01 < line["full_build"]["estimate_over_full"] < 100   # a tiny graph: timing noise only
    assert probe == {"plant_imported": False, "libchl_mapped": False}
