"""Regenerate the golden fixtures from the reference itself.

Runs in a container that holds the reference sources (the reference
binaries are built by oracle/Makefile into oracle/_ref):
  * graphs/<file>.u<0|1>.dump : hl::Graph::read's adjacency for each small
    graph file, printed by oracle/_ref/graphdump (built against the
    reference's shared_memory/graph.hpp), undirected = 0 and 1;
  * labels/<case>.{gr,order,labels} : the reference GLL binary
    (shared_memory/hhl, `-p 2 -s 32`) on small seeded graphs;
  * labels/<case>.pairs / .dist : query pairs and the answers of the
    reference's Labeling::query (oracle/_ref/labelquery).
Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import plant_gb300 as P  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def dump_graphs():
    gdir = os.path.join(HERE, "graphs")
    for f in sorted(os.listdir(gdir)):
        if f.endswith(".dump"):
            continue
        for u in (0, 1):
            r = subprocess.run([os.path.join(REF, "graphdump"), os.path.join(gdir, f), str(u)],
                               capture_output=True, text=True, check=True)
            with open(os.path.join(gdir, f"{f}.u{u}.dump"), "w") as fh:
                fh.write(r.stdout)


def random_directed(n, m, seed):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, m, dtype=np.uint32)
    dst = rng.integers(0, n, m, dtype=np.uint32)
    keep = src != dst
    w = rng.integers(1, 20, m, dtype=np.int32)
    return P.Graph.from_arcs(n, src[keep], dst[keep], w[keep])


def label_cases():
    ldir = os.path.join(HERE, "labels")
    os.makedirs(ldir, exist_ok=True)
    cases = {
        "grid12": (P.Graph.grid(12, 12, seed=11), "degree", 21),
        "grid20hw": (P.Graph.grid(20, 20, highways=12, hw_steps=8, seed=12), "betweenness", 22),
        "rmat8": (P.Graph.rmat(8, 8, seed=13), "degree", 23),
        "directed60": (random_directed(60, 240, 14), "degree", 24),
        "unit_path": (P.Graph.from_arcs(6, [0, 1, 2, 3, 4], [1, 2, 3, 4, 5], [1, 1, 1, 1, 1], True),
                      "degree", 25),
    }
    for name, (g, kind, seed) in cases.items():
        base = os.path.join(ldir, name)
        g.write(base + ".gr")
        og = O.OGraph.read_dimacs(base + ".gr")
        order = og.degree_order(seed) if kind == "degree" else og.betweenness_order(32, seed)
        P.Order.write(base + ".order", order)
        subprocess.run([os.path.join(REF, "hhl"), "-g", base + ".gr", "-o", base + ".order", "-p", "2",
                        "-l", base + ".labels"], capture_output=True, check=True)
        n = len(order)
        rng = np.random.default_rng(seed)
        pairs = rng.integers(0, n, (500, 2))
        np.savetxt(base + ".pairs", pairs, fmt="%d")
        r = subprocess.run([os.path.join(REF, "labelquery"), base + ".labels", base + ".pairs"],
                           capture_output=True, text=True, check=True)
        with open(base + ".dist", "w") as fh:
            fh.write(r.stdout)


if __name__ == "__main__":
    if not os.path.exists(os.path.join(REF, "hhl")):
        sys.exit("oracle/_ref is not built (needs the reference sources): make -C oracle ref")
    dump_graphs()
    label_cases()
    print("golden fixtures written")
