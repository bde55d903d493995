"""Digests of the reference's labels on the benchmark-scale workloads.

The label files of these builds are many GB, so instead of files this
script commits digests (oracle/chl_digest.h) to scale_digests.json:

  * the graph (forward CSR, from the seeded generator of the package),
  * the order, computed by the CPU oracle's restatement of the plain order,
  * the labels built by the reference's own run_paraPLL
    (shared_memory/akiba.hpp:132-217, called as shared_memory/hhl.cpp:65
    does, `-p <threads> -s 32`) through oracle/_ref/ref_digest, which is
    compiled from the reference sources by oracle/Makefile.

Runs where the reference sources are present (x86 host; minutes per
workload).  Usage: python tests/golden/make_scale_digests.py [name ...]
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import plant_gb300 as P  # noqa: E402
from tests.golden import digests as D  # noqa: E402

OUT = os.path.join(HERE, "scale_digests.json")

# name -> (generator call, order kind, order seed); the benchmark's workloads
WORKLOADS = {
    "grid100": ("grid", dict(rows=100, cols=100, seed=1), "degree", 1),
    "grid1024_hw2000_bc256": ("grid", dict(rows=1024, cols=1024, highways=2000, hw_steps=64, hw_factor=150.0,
                                           seed=1), "betweenness256", 1),
    "rmat20": ("rmat", dict(scale=20, ef=16, a=0.57, b=0.19, c=0.19, seed=1), "degree", 1),
}


def make_graph(kind, kw):
    if kind == "grid":
        return P.Graph.grid(kw["rows"], kw["cols"], del_frac=0.05, diag_frac=0.01, wmin=1, wmax=1000,
                            highways=kw.get("highways", 0), hw_steps=kw.get("hw_steps", 64),
                            hw_factor=kw.get("hw_factor", 150.0), seed=kw["seed"])
    return P.Graph.rmat(kw["scale"], kw["ef"], kw["a"], kw["b"], kw["c"], seed=kw["seed"])


def run(name, threads):
    kind, kw, okind, oseed = WORKLOADS[name]
    t0 = time.time()
    g = make_graph(kind, kw)
    n = g.get_n()
    off, head, ln = g.csr(True)
    gd = D.graph_digest(n, off, head, ln)
    og = O.OGraph.from_csr(n, off, head, ln)
    order = og.degree_order(oseed) if okind == "degree" else og.betweenness_order(256, oseed)
    od = O.order_digest(order)
    t1 = time.time()
    with tempfile.TemporaryDirectory(prefix="chl_scale_") as d:
        gp, op = os.path.join(d, "g.gr"), os.path.join(d, "g.order")
        g.write(gp)
        P.Order.write(op, order)
        r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_digest"), gp, op, str(threads), "32"],
                           capture_output=True, text=True, check=True)
    t2 = time.time()
    m = re.search(r"digest ([0-9a-f]{16}) n (\d+) total (\d+) avg ([0-9.]+)", r.stdout)
    tm = re.search(r"total time = ([0-9.e+-]+)", r.stdout)
    if not m or int(m.group(2)) != n:
        raise RuntimeError("ref_digest output: " + r.stdout[-400:])
    return {"generator": {"kind": kind, **kw}, "order": {"kind": okind, "seed": oseed},
            "n": n, "arcs": int(len(head)), "graph_digest": f"{gd:016x}", "order_digest": f"{od:016x}",
            "labels_digest": m.group(1), "labels_total": int(m.group(3)), "avg_label": float(m.group(4)),
            "reference": {"binary": "ref_digest (run_paraPLL, sf 32)", "threads": threads,
                          "total_time_s": float(tm.group(1)) if tm else None,
                          "setup_s": round(t1 - t0, 1), "wall_s": round(t2 - t1, 1)}}


def main():
    names = sys.argv[1:] or list(WORKLOADS)
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    data["digest"] = "oracle/chl_digest.h, version 1"
    for name in names:
        data[name] = run(name, os.cpu_count() or 1)
        print(name, json.dumps(data[name]), flush=True)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main()
