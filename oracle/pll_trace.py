"""Sequential PLL trace of a benchmark workload: the algorithmic bytes of the
build roofline.

Roots are taken one at a time in rank order and every tree prunes with the
complete labels of the higher-ranked hubs (og_pll_trace).  The roofline's
bytes are 8 per entry of every settled vertex's label list, 8 per out-arc of
every settled vertex and 8 per label written.  The counts depend only on the
graph and the order, not on any GPU schedule, so they are computed once per
workload and committed as profiles/pll_trace_<workload>.json, which bench.py
reads.

Test infrastructure: this runs the oracle (single-threaded C), never the GPU
engine.  The graph and the order are bench.py's own workload, built by the
oracle's restatements of the package's seeded generators and of the degree /
betweenness orders (identical graphs and orders, checked by digest).

    python oracle/pll_trace.py                           # 1024x1024 grid
    python oracle/pll_trace.py --workload rmat --scale 20
    python oracle/pll_trace.py --side 512 --highways 500
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this folder comes first on the path and would shadow the
# `oracle` package with its own oracle.py
sys.path = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") not in (HERE, ROOT)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="grid", choices=["grid", "rmat"])
    ap.add_argument("--side", type=int, default=1024)
    ap.add_argument("--highways", type=int, default=2000)
    ap.add_argument("--sources", type=int, default=256)
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--out", default=None, help="output JSON (default: profiles/pll_trace_<workload>.json)")
    args = ap.parse_args()

    import bench
    from oracle import oracle as O

    og, order = bench.oracle_workload(O, args)
    _, head, _ = og.csr(True)
    t0 = time.time()
    tr = O.pll_trace(og, order)
    secs = time.time() - t0
    out = {"workload": bench.workload_name(args), "vertices": og.n, "graph_arcs": int(len(head)),
           "trace_seconds": round(secs, 1), **tr,
           "command": "python oracle/pll_trace.py " + " ".join(sys.argv[1:])}
    path = args.out or os.path.join(ROOT, "profiles", "pll_trace_" + bench.workload_slug(args) + ".json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
