"""Schedule autotuner for the label build.

The build's speed depends on four schedule knobs: the roots in the first
superstep, the superstep growth factor, the label budget per superstep, and
the queue size at which a tree's queue is split into near and far parts.
The labels never depend on them (canonical labels are unique for an order),
and the labels of the hubs of rank < R are final once the roots below R are
processed, so every candidate is timed on the same exact work: a prefix build of the roots of rank < R (``root_limit``).  The search is
coordinate descent over the four knobs; the winner is cached in a JSON file
keyed by graph statistics, so graphs of the same kind skip the search.

No reference counterpart: the reference's superstep size is the fixed label
budget ``-s`` (shared_memory/hhl.cpp:65).
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import Graph, build

DEFAULT_CACHE = os.environ.get(
    "CHL_AUTOTUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "plant_gb300", "autotune.json"))

FIRST = (0, 256, 1024, 4096)      # 0: the built-in choice from graph statistics
GROWTH = (0.0, 0.5, 1.0, 2.0)     # 0.0: built-in
SF = (0.0, 32.0, 128.0, 1024.0)   # label budget per superstep (x n); 0.0: built-in
QSPLIT = (0, 1, 512, 4096)        # near/far queue split size; 0: built-in, 1: off


def graph_key(g: Graph) -> str:
    """Statistics the schedule depends on: size class, mean degree, degree
    skew and directedness."""
    n = max(1, g.get_n())
    d = g.degrees(True).astype(np.float64)
    mean = float(d.mean()) if d.size else 0.0
    skew = float(d.max()) / mean if mean > 0 else 0.0
    return "{}-n2^{}-deg{}-skew{}".format("sym" if g.symmetric() else "dir", int(round(math.log2(n))),
                                          int(round(mean)), "heavy" if skew > 32 else "flat")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(g: Graph, order, fraction: float = 0.02, min_roots: int = 4096, repeats: int = 1,
         cache: str | None = DEFAULT_CACHE, force: bool = False, log=None, **build_kw) -> dict:
    """Best (first_superstep, growth, sf, queue_split) for g;
    cached by graph_key."""
    key = graph_key(g)
    data = _load(cache) if cache else {}
    if not force and key in data:
        return dict(data[key]["config"])
    n = g.get_n()
    R = int(min(n, max(min_roots, fraction * n)))
    timings = {}

    def cost(cfg):
        k = json.dumps(cfg, sort_keys=True)
        if k not in timings:
            best = math.inf
            for _ in range(repeats):
                L = build(g, order, root_limit=R, **cfg, **build_kw)
                best = min(best, L.stats()["build_ms"])
                del L
            timings[k] = best
            if log:
                log(f"autotune {key} {cfg}: {best:.1f} ms for roots < {R}")
        return timings[k]

    cfg = {"first_superstep": 0, "growth": 0.0, "sf": 0.0, "queue_split": 0}
    t0 = time.perf_counter()
    for knob, values in (("first_superstep", FIRST), ("growth", GROWTH), ("sf", SF), ("queue_split", QSPLIT)):
        best_v = min(values, key=lambda v: cost({**cfg, knob: v}))
        cfg[knob] = best_v
    result = {"config": cfg, "prefix_roots": R, "prefix_ms": cost(cfg),
              "search_s": time.perf_counter() - t0, "candidates": len(timings)}
    if cache:
        data = _load(cache)
        data[key] = result
        _store(cache, data)
    return dict(cfg)


def tuned_build(g: Graph, order, cache: str | None = DEFAULT_CACHE, log=None, **build_kw):
    """build() with the cached (or freshly tuned) schedule for g."""
    cfg = tune(g, order, cache=cache, log=log, **build_kw)
    return build(g, order, **cfg, **build_kw)
