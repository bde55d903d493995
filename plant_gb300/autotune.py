"""Schedule autotuner for the label build.

The build's speed depends on seven schedule knobs: the roots in the first
superstep, the superstep growth factor, the label budget per superstep, the
queue size at which a tree's queue is split into near and far parts, the
window size and warps per tree of the first superstep's label-correcting
trees, and the PLaNT-to-GLL phase switch ratio.  The labels never depend on them (canonical labels are unique for an
order), and the labels of the hubs of rank < R are final once the roots below
R are processed, so every candidate is timed on the same exact work: a prefix
build of the roots of rank < R (``root_limit``; the whole build when
``fraction`` is 1).  The search is coordinate descent over the knobs; the
winner is cached in a JSON file keyed by the graph's class, so graphs of the
same kind skip the search.

The library reads the winners too: ``write_table`` writes them as the text
table that ``chl_build`` consults when ``autotune`` is set (options left at 0
take the class's value).  ``tuned_schedules.txt`` beside the library ships
the schedules measured on GB300 for the benchmark graphs' classes.

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
WTARGET = (0, 1, 256, 1024, 4096) # first-superstep window size; 0: built-in, 1: settle rounds
WWARPS = (0, 4, 8)                # warps per first-superstep tree; 0: built-in
PS = (0.0, 8.0, 64.0, 1024.0)     # hybrid phase switch ratio; 0.0: built-in
KNOBS = (("first_superstep", FIRST), ("growth", GROWTH), ("sf", SF), ("queue_split", QSPLIT),
         ("window_target", WTARGET), ("window_warps", WWARPS), ("ps", PS))
SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned_schedules.txt")


def graph_key(g: Graph) -> str:
    """The graph's class (chl_graph_class): directedness, log2 n, mean
    out-degree, degree skew -- the statistics the schedule depends on."""
    return g.graph_class()


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
    """Best schedule knobs (KNOBS) for g; cached by graph_key."""
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
                L = build(g, order, root_limit=R if R < n else 0, autotune=0, **cfg, **build_kw)
                best = min(best, L.stats()["build_ms"])
                del L
            timings[k] = best
            if log:
                log(f"autotune {key} {cfg}: {best:.1f} ms for roots < {R}")
        return timings[k]

    cfg = {"first_superstep": 0, "growth": 0.0, "sf": 0.0, "queue_split": 0, "window_target": 0, "window_warps": 0,
           "ps": 0.0}
    t0 = time.perf_counter()
    for knob, values in KNOBS:
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


def table_line(key: str, cfg: dict) -> str:
    """One line of the library's tuned-schedule table."""
    return "{} {} {} {} {} {} {} {}".format(key, int(cfg["first_superstep"]), float(cfg["growth"]),
                                            float(cfg["sf"]), int(cfg["queue_split"]),
                                            int(cfg.get("window_target", 0)), int(cfg.get("window_warps", 0)),
                                            float(cfg.get("ps", 0.0)))


def write_table(path: str = SHIPPED, cache: str | None = DEFAULT_CACHE, entries: dict | None = None) -> None:
    """Merge the cached winners (or `entries`: key -> config) into the text
    table chl_build reads: one line per graph class, replacing that class's
    line if present."""
    new = dict(entries) if entries is not None else {k: v["config"] for k, v in _load(cache).items()}
    lines = []
    try:
        with open(path) as f:
            for line in f:
                k = line.split()[0] if line.strip() and not line.startswith("#") else None
                if k is None or k not in new:
                    lines.append(line.rstrip("\n"))
    except OSError:
        lines = ["# graph-class first_superstep growth sf queue_split window_target window_warps ps",
                 "# written by plant_gb300/autotune.py (write_table); read by chl_build when autotune is set"]
    lines += [table_line(k, c) for k, c in sorted(new.items())]
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        f.write("\n".join(lines) + "\n")
    os.replace(tmp, path)
