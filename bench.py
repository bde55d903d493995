#!/usr/bin/env python3
"""Benchmark: canonical hub label build on a ~1M-vertex road-like grid.

Workload (the metric's configuration): 1024 x 1024 perturbed 4-neighbour
grid (5% edges deleted, largest component, 1% diagonal shortcuts, lengths
uniform in [1, 1000]) plus 2,000 highway edges at most 64 grid steps long
(length round(150 x Manhattan)); ranking = sampled betweenness from 256
seeded sources computed on the GPU (untimed set-up).  One step = one full
label build (all roots, canonical labels) with the graph resident in HBM.

  value  : labels/s of the device-timed builds (CUDA events on the build
           stream; the label CSR alone is several GB, far above L2, so no
           flush is needed between steps)
  e2e    : labels/s through the C ABI from host buffers: graph + order
           upload, build, and the labels read back to host memory, timed on
           the host around each step
  roofline: tree kernel, algorithmic bytes / tree-kernel time.  The bytes
           are sequential PLL's (roots one at a time in rank order, each
           tree pruned with the complete labels of higher-ranked hubs):
           8 B per entry of every settled vertex's label list, per out-arc
           of every settled vertex and per label written, counted once per
           workload by oracle/pll_trace.py into profiles/pll_trace_*.json;
           without such a file, the closed form over the labelled vertices
           (a lower bound) stands in
  cpu_baseline: the CPU restatement of the reference GLL (OpenMP, all host
           cores), estimated for the whole build from replays of a sample of
           its supersteps, each from its committed state (the complete labels
           are the GPU's, identical to the CPU's)

--impl reference times that CPU restatement (the reference itself does not
build on this host: shared_memory/akiba.hpp includes <immintrin.h>, x86 only,
and its sources are not present on the GPU host) with no product code
loaded: the oracle generates the same graph and order, builds the whole
labeling once (set-up), and every step replays a sample of its supersteps.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "CHL label build throughput (canonical labels, 1024x1024 road-like grid, betweenness order)"
METRIC_RMAT = "CHL label build throughput (canonical labels, RMAT scale 20, degree order)"
UNIT = "labels/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--side", type=int, default=1024)
    ap.add_argument("--highways", type=int, default=2000)
    ap.add_argument("--sources", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-full", action="store_true",
                    help="also time the CPU GLL restatement on the WHOLE build (minutes) and "
                         "check its labels against the GPU's")
    ap.add_argument("--workload", default="grid", choices=["grid", "rmat"],
                    help="grid: 1024x1024 road-like grid (default); rmat: RMAT scale 20, degree order")
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--verbose", type=int, default=0, help="2: per-superstep lines on stderr")
    ap.add_argument("--max-warps", type=int, default=0,
                    help="cap on concurrent trees (bounds the per-tree workspace, e.g. for profiler captures)")
    ap.add_argument("--ingest", action="store_true",
                    help="graph ingestion: host parsers against the GPU path on DIMACS and SNAP files "
                         "of the grid workload")
    ap.add_argument("--serve", action="store_true",
                    help="also run the open-loop serving test (Poisson arrivals) on the grid labels")
    ap.add_argument("--no-rmat", action="store_true",
                    help="skip the RMAT-20 leg (GLL vs hybrid builds, queries, serving) of the default run")
    ap.add_argument("--serve-qps", type=float, default=2e8, help="offered pair rate (pairs/s)")
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    ap.add_argument("--rank", action="store_true",
                    help="learned ranking: train on small labelings, evaluate against the plain order")
    ap.add_argument("--rank-graphs", type=int, default=256)
    ap.add_argument("--rank-epochs", type=int, default=12)
    ap.add_argument("--rank-eval", default="rmat21,grid1448",
                    help="comma list of evaluation graphs: rmatS or gridSIDE")
    ap.add_argument("--rank-save", default="", help="write the trained parameters (.npy) here")
    ap.add_argument("--rank-load", default="", help="skip training: load parameters (.npy)")
    return ap.parse_args()


def max_over_ranks(x, dist):
    """The largest x over all ranks (every rank gets it); x itself on one."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(ws, labels_per_rank, ms_step):
    """Whole-job labels/s: every rank builds the whole labeling (replicas),
    timed by the slowest rank."""
    return ws * labels_per_rank / (ms_step / 1e3)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class Clocks:
    """Samples nvidia-smi during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        sm = []
        mx = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
            except ValueError:
                continue
            for nm, v in zip(names, r[3:7]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per algorithmic byte of the tree kernel, from the committed
    ncu capture of a smaller grid (scaled to this workload's launches)."""
    p = os.path.join(ROOT, "profiles", "batch_kernel_traffic_grid512.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


def profile_trace(args):
    """Sequential PLL work counts of this workload (oracle/pll_trace.py), or
    None when no trace is committed for it."""
    p = os.path.join(ROOT, "profiles", "pll_trace_" + workload_slug(args) + ".json")
    try:
        with open(p) as f:
            t = json.load(f)
    except Exception:
        return None
    return t if t.get("workload") == workload_name(args) else None


def make_workload(P, args):
    """The graph (host-side seeded generator) and its order, computed on the
    GPU."""
    if args.workload == "rmat":
        g = P.Graph.rmat(args.scale, 16, 0.57, 0.19, 0.19, seed=1)
        return g, P.Order.degree(g, seed=1)
    g = P.Graph.grid(args.side, args.side, del_frac=0.05, diag_frac=0.01, wmin=1, wmax=1000,
                     highways=args.highways, hw_steps=64, hw_factor=150.0, seed=1)
    return g, P.Order.betweenness(g, args.sources, seed=1)


def workload_slug(args):
    """File-name form of the workload (profiles/pll_trace_<slug>.json)."""
    if args.workload == "rmat":
        return f"rmat{args.scale}"
    return f"grid{args.side}_hw{args.highways}_bc{args.sources}"


def reference_key(args):
    """Entry of tests/golden/scale_digests.json for this workload."""
    if args.workload == "rmat":
        return f"rmat{args.scale}"
    return f"grid{args.side}_hw{args.highways}_bc{args.sources}"


def workload_name(args):
    if args.workload == "rmat":
        return f"rmat{args.scale} ef16 (0.57,0.19,0.19,0.05), degree order"
    return f"grid{args.side}x{args.side}+hw{args.highways}, betweenness({args.sources})"


def cpu_full(g, order, L):
    """Whole CPU GLL build (restatement of run_paraPLL, all host cores);
    returns (seconds, labels, identical_to_gpu)."""
    from oracle import oracle as O
    off, head, ln = g.csr(True)
    og = O.OGraph.from_csr(g.get_n(), off, head, ln)
    ref, secs = O.gll(og, order, threads=os.cpu_count() or 1)
    a = L.export()
    b = ref.export(g.get_n())
    same = all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))
    return secs, int(ref.total()), bool(same)


def oracle_workload(O, args):
    """The workload built by the CPU oracle alone: its restatements of the
    package's seeded generators (og_gen_grid / og_gen_rmat, identical graphs)
    and of the plain orders.  The reference arm uses this and loads no
    product code."""
    if args.workload == "rmat":
        og = O.OGraph.rmat(args.scale, 16, 0.57, 0.19, 0.19, 1)
        return og, og.degree_order(1)
    og = O.OGraph.grid(args.side, args.side, 0.05, 0.01, 1, 1000, args.highways, 64, 150.0, 1)
    return og, og.betweenness_order(args.sources, 1)


def pps_sample(sizes, target, rng):
    """Stratified sample of supersteps: the supersteps are split into S
    contiguous strata of about equal total size, S about the number of
    supersteps the expected cost `target` affords at their mean size, and
    one superstep is drawn from each stratum with probability proportional
    to its size.  Returns [(index, pi)]; the Horvitz-Thompson sum of
    t_i / pi_i over the sample is an unbiased estimate of the whole build's
    sum of t_i.  Contiguous strata take out the drift of the time per label
    over a build (later supersteps prune more per label), which an
    unstratified draw of a few supersteps turns into variance."""
    sizes = np.asarray(sizes, np.float64)
    live = np.nonzero(sizes > 0)[0]
    if len(live) == 0:
        return []
    total = float(sizes[live].sum())
    mean = total / len(live)
    S = int(min(len(live), max(1, round(target / mean))))
    if S == len(live):
        return [(int(i), 1.0) for i in live]
    cum = np.cumsum(sizes[live])
    # stratum of each live superstep: by the midpoint of its size interval
    mid = cum - sizes[live] / 2.0
    strata = np.minimum((mid / total * S).astype(np.int64), S - 1)
    plan = []
    for s_ in range(S):
        idx = live[strata == s_]
        if len(idx) == 0:
            continue
        w = sizes[idx]
        p = w / w.sum()
        j = int(rng.choice(len(idx), p=p))
        plan.append((int(idx[j]), float(p[j])))
    return plan


def replay_rate(rp, labels_total, starts, ends, sizes, target, steps, warmup, seed=12345):
    """CPU GLL build rate from superstep replays: every step replays a
    stratified PPS sample of whole supersteps (pps_sample) with each one's
    committed state taken from the complete labels, and estimates the whole
    build's time by Horvitz-Thompson.  Returns (rate, per-step estimates,
    replay seconds per step, supersteps replayed per step)."""
    rng = np.random.default_rng(seed)
    ests, walls, counts = [], [], []
    for it in range(warmup + steps):
        plan = pps_sample(sizes, target, rng)
        est = wall = 0.0
        for i, pi in plan:
            _, t = rp.run(int(starts[i]), int(starts[i]), int(ends[i]))
            est += t / pi
            wall += t
        if it >= warmup:
            ests.append(est)
            walls.append(wall)
            counts.append(len(plan))
    return labels_total / float(np.mean(ests)), ests, walls, counts


def supersteps_from_labels(hub_count_by_rank, N, sf=32.0):
    """Superstep boundaries a CPU GLL build (run_paraPLL with label_limit =
    sf * N, shared_memory/akiba.hpp:152-185) would have, estimated from the
    final label counts per hub rank (the CPU counts its labels before the
    clean, so its supersteps are somewhat shorter)."""
    cum = np.cumsum(np.asarray(hub_count_by_rank, np.float64))
    limit = sf * N
    ends = []
    start_labels = 0.0
    r = 0
    while r < N:
        e = int(np.searchsorted(cum, start_labels + limit, side="left")) + 1
        e = max(r + 1, min(N, e))
        ends.append(e)
        start_labels = cum[e - 1]
        r = e
    return np.asarray(ends, np.int64)


def build_work_bytes(L, g):
    """Sequential-PLL bytes of the labelled vertices, from list sizes: a list
    of length k at vertex u (side s, built by trees walking direction 1-s)
    costs sum_{j<k} (8*outdeg(u) + 8*j + 8)."""
    sizes = L.list_sizes().astype(np.float64).reshape(-1, 2)
    deg_fwd = g.degrees(True).astype(np.float64)
    deg_rev = g.degrees(False).astype(np.float64)
    tot = 0.0
    for side, deg in ((0, deg_fwd), (1, deg_rev)):
        k = sizes[:, side]
        tot += float(np.sum(8.0 * k * deg + 8.0 * k * (k - 1) / 2.0 + 8.0 * k))
    return tot


def schedule_used(g):
    """The tuned-schedule table line chl_build applies to g (autotune on), or
    the built-in defaults when the table has no line for g's class."""
    cls = g.graph_class()
    path = os.environ.get("CHL_SCHEDULES") or os.path.join(ROOT, "plant_gb300", "tuned_schedules.txt")
    try:
        with open(path) as f:
            for line in f:
                t = line.split()
                if t and not line.startswith("#") and t[0] == cls:
                    keys = ("first_superstep", "growth", "sf", "queue_split", "window_target", "window_warps", "ps")
                    return {"class": cls, "source": os.path.basename(path),
                            "table": dict(zip(keys, (float(x) for x in t[1:])))}
    except OSError:
        pass
    return {"class": cls, "source": "built-in defaults"}


def reference_digests():
    """Digests of the reference's own labels on the benchmark workloads
    (tests/golden/scale_digests.json, written by
    tests/golden/make_scale_digests.py from run_paraPLL's output)."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "scale_digests.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def parity(L, key):
    """The device digest of L against the reference's digest of the same
    workload: equal digests mean byte-identical label files."""
    ref = reference_digests().get(key)
    got = f"{L.digest():016x}"
    if ref is None:
        return {"labels_digest": got, "labels_checksum_match": None, "reference": "no digest committed"}
    return {"labels_digest": got, "reference_digest": ref["labels_digest"],
            "labels_checksum_match": got == ref["labels_digest"] and L.stats()["labels"] == ref["labels_total"],
            "reference": "run_paraPLL (shared_memory/akiba.hpp:132-217), -s 32, digest of its Labeling"}


def rmat_leg(P, args, serve_seconds):
    """RMAT scale 20 (ef 16, degree order): device-timed builds in hybrid
    (PLaNT then pruned supersteps) and GLL mode, both checked against the
    reference digest, then queries and the open-loop serving test on the
    labels.  Part of the default run."""
    g = P.Graph.rmat(20, 16, 0.57, 0.19, 0.19, seed=1)
    order = P.Order.degree(g, seed=1)
    n = g.get_n()
    g.to_device()
    out = {"workload": "rmat20 ef16 (0.57,0.19,0.19,0.05), degree order, full build", "vertices": n,
           "arcs": int(g.out_arcs()), "schedule": schedule_used(g)}
    for name, mode in (("hybrid", P.MODE_HYBRID), ("gll", P.MODE_GLL)):
        P.build(g, order, mode=mode)
        st = []
        for _ in range(3):
            L = P.build(g, order, mode=mode)
            st.append(L.stats())
        ms = float(np.mean([x["build_ms"] for x in st]))
        out[name] = {"build_ms": ms, "tree_ms": float(np.mean([x["tree_ms"] for x in st])),
                     "labels": st[-1]["labels"], "labels_per_s": st[-1]["labels"] / (ms / 1e3),
                     "avg_label": st[-1]["avg_label"], "supersteps": st[-1]["supersteps"],
                     "plant_roots": st[-1]["plant_roots"], "parity": parity(L, "rmat20")}
        if name == "gll":
            del L
        else:
            Lh = L
    out["gll_over_hybrid_build"] = out["gll"]["build_ms"] / out["hybrid"]["build_ms"]
    qk = 1 << 22
    q_ms, q_bytes = P.query_bench(Lh, qk, iters=20, seed=7)
    qh_ms, _ = P.query_bench(Lh, qk, iters=20, seed=7, hot=1000)
    out["query"] = {"pairs": qk, "qps": qk / (q_ms / 1e3), "achieved_gbs": q_bytes / (q_ms / 1e3) / 1e9,
                    "hot_qps": qk / (qh_ms / 1e3)}
    if serve_seconds > 0:
        out["serving"] = serve_test(P, Lh, n, args.serve_qps, serve_seconds)
    del Lh
    g.release_device()
    return out


def serve_test(P, L, n, qps, seconds, seed=11):
    """Open-loop Poisson request stream against the continuous-batching
    server: request sizes log-uniform in [1, 65536] pairs, 10% of the pairs
    drawn from a fixed hot set of 1,000 pairs.  Arrivals follow the offered
    pair rate; latency is submit-to-completion measured by the server."""
    rng = np.random.default_rng(seed)
    hot = rng.integers(0, n, (1000, 2)).astype(np.uint32)
    srv = P.Server(L, max_inflight_pairs=1 << 24, max_requests=1 << 16, max_batch_pairs=1 << 21)
    sizes, reqs = [], []
    total = 0
    while total < qps * seconds:
        k = int(np.exp(rng.uniform(0, np.log(65536.0))))
        k = max(1, min(65536, k))
        q = rng.integers(0, n, (k, 2)).astype(np.uint32)
        nh = rng.binomial(k, 0.1)
        if nh:
            q[:nh] = hot[rng.integers(0, 1000, nh)]
        reqs.append(q)
        sizes.append(k)
        total += k
        if len(reqs) >= 200000:
            break
    mean_k = float(np.mean(sizes))
    rate = qps / mean_k                       # requests per second
    gaps = rng.exponential(1.0 / rate, len(reqs))
    lat = [None] * len(reqs)
    ids = [None] * len(reqs)
    import queue as _q
    pend = _q.Queue()

    kept = {}

    def waiter():
        while True:
            item = pend.get()
            if item is None:
                return
            i, rid = item
            out, l = srv.wait(rid, len(reqs[i]))
            lat[i] = l
            if i % 97 == 0:
                kept[i] = out

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    t0 = time.perf_counter()
    nxt = t0
    for i, q in enumerate(reqs):
        nxt += gaps[i]
        while True:
            now = time.perf_counter()
            if now >= nxt:
                break
            time.sleep(min(0.0005, nxt - now))
        ids[i] = srv.submit(q)
        pend.put((i, ids[i]))
    pend.put(None)
    th.join()
    t1 = time.perf_counter()
    st = srv.stats()
    srv.close()
    # answers of every 97th request against the batch query on the same labels
    same = all(np.array_equal(v, P.query(L, reqs[i])) for i, v in kept.items())
    la = np.array(lat, np.float64)
    return {"offered_pairs_per_s": qps, "requests": len(reqs), "pairs": int(total),
            "achieved_pairs_per_s": total / (t1 - t0), "p50_ms": float(np.percentile(la, 50)),
            "p99_ms": float(np.percentile(la, 99)), "mean_request_pairs": mean_k,
            "launches": st["launches"], "hot_fraction": 0.1, "answers_checked": len(kept),
            "answers_equal_batch_query": bool(same)}


def run_reference(args, ws, rank):
    """The reference's CPU path (the oracle's byte-identical restatement of
    run_paraPLL, all host cores) on the same workload, with no product code
    loaded.  Set-up (untimed): the graph and order from the oracle's own
    generators, one whole CPU build, which records its supersteps.  Each
    step then replays a probability-proportional-to-size sample of whole
    supersteps from their recorded committed state (oracle Replay) and
    estimates the whole build's time; the value is the labels of the whole
    build over the mean estimate."""
    if rank != 0:
        return
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    t0 = time.time()
    og, order = oracle_workload(O, args)
    t_gen = time.time() - t0
    L, full_secs, ends, step_secs = O.gll_steps(og, order, threads)
    labels = int(L.total())
    starts = np.concatenate([[0], ends[:-1]])
    rp = O.Replay(og, order, L, threads)
    target = max(1.0, min(args.cpu_seconds, 75.0 / max(1, args.steps + args.warmup)))
    rate, ests, walls, counts = replay_rate(rp, labels, starts, ends, step_secs, target, args.steps, args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(walls)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (the oracle's restatement of the seeded generators)",
            "config": {"workload": workload_name(args) + ", full build", "vertices": int(og.n),
                       "same_config": True},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": (f"per step, a stratified PPS sample of whole supersteps (mean {np.mean(counts):.1f} of "
                                        f"{len(ends)}) of the GLL restatement (run_paraPLL, sf 32) replayed from "
                                        "their committed state; Horvitz-Thompson estimate of the whole build")},
            "full_build": {"seconds": full_secs, "labels": labels, "labels_per_s": labels / full_secs,
                           "supersteps": int(len(ends)), "estimate_over_full": float(np.mean(ests)) / full_secs,
                           "step_estimates_over_full": [round(x / full_secs, 3) for x in ests]},
            "setup_s": {"workload": round(t_gen, 1), "full_build": round(full_secs, 1)},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank):
    import plant_gb300 as P
    P.lib()
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    g, order = make_workload(P, args)
    n = g.get_n()
    g.to_device()

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        L = P.build(g, order, max_warps=args.max_warps)
        del L
    barrier()
    stats = []
    t0 = time.time()
    with Clocks() as ck:
        for _ in range(args.steps):
            L = P.build(g, order, verbose=args.verbose, max_warps=args.max_warps)
            stats.append(L.stats())
    wall = time.time() - t0
    barrier()
    build_ms = [s["build_ms"] for s in stats]
    tree_ms = [s["tree_ms"] for s in stats]
    labels = stats[-1]["labels"]
    ms_step = max_over_ranks(float(np.mean(build_ms)), dist)
    value = job_throughput(ws, labels, ms_step)
    # algorithmic bytes of a build: the sequential PLL trace of this workload
    # when one is committed, else the closed form over the labelled vertices
    # (a lower bound: pruned visits left out)
    labelled = build_work_bytes(L, g)
    trace = profile_trace(args)
    work = float(trace["algorithmic_bytes"]) if trace else labelled
    avg_tree_ms = float(np.mean(tree_ms))
    per_launch_tree = avg_tree_ms / max(1, stats[-1]["tree_launches"])
    peak, peak_kind = peaks()
    achieved = work / (avg_tree_ms / 1e3) / 1e9
    traffic = profile_traffic()
    # queries on the resident labels (uniform pairs, device resident)
    qk = 1 << 22
    q_ms, q_bytes = P.query_bench(L, qk, iters=20, seed=7)
    qps = qk / (q_ms / 1e3)
    # hot set: every pair one of 1,000 fixed pairs (label lists L2-resident)
    qh_ms, qh_bytes = P.query_bench(L, qk, iters=20, seed=7, hot=1000)
    # e2e through the C ABI from host buffers
    g.release_device()
    off, head, ln = g.csr(True)
    h2d = off.nbytes + head.nbytes + ln.nbytes + order.nbytes
    if not g.symmetric():
        off0, head0, ln0 = g.csr(False)
        h2d += off0.nbytes + head0.nbytes + ln0.nbytes
    e2e_s = []
    d2h = 0
    for _ in range(max(1, args.steps)):
        t = time.time()
        L2 = P.build(g, order, max_warps=args.max_warps)
        o2, h2, d2 = L2.export()
        e2e_s.append(time.time() - t)
        d2h = o2.nbytes + h2.nbytes + d2.nbytes
        del L2, o2, h2, d2
    e2e = ws * labels / float(np.mean(e2e_s))
    launches = int(stats[-1]["kernel_launches"])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "config": {"workload": workload_name(args) + ", full build",
                   "vertices": n, "arcs": int(g.out_arcs()), "l2": "inputs larger than L2 (label CSR of several GB)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "clocks": ck.summary(),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": (work / max(1, stats[-1]["tree_launches"])
                                 * traffic["dram_per_trace_byte" if trace else "dram_per_labelled_byte"]
                                 if traffic and ("dram_per_trace_byte" in traffic or not trace) else None),
                     "traffic_note": ("bytes per launch, scaled from " + traffic["workload"] + " (ncu)"
                                      if traffic else None),
                     "kernel": "batch_kernel", "algorithmic_bytes_per_build": work,
                     "work_model": ("sequential PLL trace, profiles/pll_trace_" + workload_slug(args) + ".json"
                                    if trace else "labelled vertices only (closed form, lower bound)"),
                     "labelled_bytes_per_build": labelled,
                     "pll_scanned_bytes_per_build": (float(trace["scanned_bytes"]) if trace else None),
                     "tree_ms_per_build": avg_tree_ms, "tree_launches": stats[-1]["tree_launches"],
                     "ms_per_launch": per_launch_tree},
        "build": {"build_s": ms_step / 1e3, "avg_label": stats[-1]["avg_label"], "labels": labels,
                  "supersteps": stats[-1]["supersteps"], "tree_ms": avg_tree_ms,
                  "commit_ms": float(np.mean([s["commit_ms"] for s in stats])),
                  "visits": stats[-1]["visits"], "label_reads": stats[-1]["label_reads"],
                  "wall_s_per_step": wall / args.steps},
        "query": {"pairs": qk, "qps": qps, "ms_per_batch": q_ms, "bytes_per_batch": q_bytes,
                  "achieved_gbs": q_bytes / (q_ms / 1e3) / 1e9,
                  "roofline_frac": (q_bytes / (q_ms / 1e3) / 1e9) / peak,
                  "hot_qps": qk / (qh_ms / 1e3), "hot_set": 1000,
                  "hot_achieved_gbs": qh_bytes / (qh_ms / 1e3) / 1e9},
    }
    line["parity"] = parity(L, reference_key(args))
    line["schedule"] = schedule_used(g)
    if rank == 0 and args.workload == "grid" and not args.no_rmat:
        line["rmat20"] = rmat_leg(P, args, args.serve_seconds)
    if rank == 0 and not args.no_cpu:
        # CPU GLL rate: replays of a PPS sample of CPU supersteps (boundaries
        # estimated from the labels), each from its committed state, the
        # complete labels being the GPU's (identical to the CPU's)
        from oracle import oracle as O
        o2, h2, d2 = L.export()
        ol = O.OLabels.from_csr(n, o2, h2, d2)
        del o2, h2, d2
        off, head, ln = g.csr(True)
        og = O.OGraph.from_csr(n, off, head, ln)
        threads = os.cpu_count() or 1
        per_rank = L.hub_freq(order)[order]
        ends = supersteps_from_labels(per_rank, n)
        starts = np.concatenate([[0], ends[:-1]])
        sizes = np.add.reduceat(per_rank.astype(np.float64), starts)
        rp = O.Replay(og, order, ol, threads)
        # sizes are labels; scale them to seconds with a first replay, of
        # the first superstep, which then counts whole (inclusion 1)
        _, t1 = rp.run(int(starts[0]), int(starts[0]), int(ends[0]))
        per_label = t1 / max(sizes[0], 1.0)
        rest = sizes * per_label
        rest[0] = 0.0
        _, ests, walls, counts = replay_rate(rp, labels, starts, ends, rest,
                                             max(1.0, args.cpu_seconds - t1), 1, 0)
        est = t1 + float(np.mean(ests))
        rate = labels / est
        del rp
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": (f"the first superstep whole plus a stratified PPS sample of "
                                           f"{np.mean(counts):.0f} more of {len(ends)} (boundaries estimated from "
                                           "the labels at 32 n per superstep) of the GLL restatement, replayed "
                                           "from their committed state; Horvitz-Thompson estimate of the whole "
                                           "build"),
                                "seconds": float(np.sum(walls)) + t1}
        pairs = P.generate_query(1 << 20, n, seed=7)
        ol.query(pairs[:1024])
        t = time.time()
        ol.query(pairs)
        cq = time.time() - t
        line["query"]["cpu_qps"] = len(pairs) / cq
        line["query"]["cpu_cores"] = os.cpu_count()
        del ol
    if rank == 0 and args.serve:
        line["serving"] = serve_test(P, L, n, args.serve_qps, args.serve_seconds)
    if rank == 0 and args.cpu_full:
        L3 = P.build(g, order)
        secs, lab, same = cpu_full(g, order, L3)
        line["cpu_full_build"] = {"seconds": secs, "labels": lab, "labels_per_s": lab / secs,
                                  "cores": os.cpu_count(), "identical_to_gpu": same,
                                  "what": "CPU GLL restatement (run_paraPLL, sf 32), whole build"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def eval_graph(P, spec):
    """Evaluation graph by name: rmatS (ef 16) or gridSIDE (highways n/500)."""
    if spec.startswith("rmat"):
        return P.Graph.rmat(int(spec[4:]), 16, 0.57, 0.19, 0.19, seed=2021)
    side = int(spec[4:])
    return P.Graph.grid(side, side, highways=side * side // 500, hw_steps=64, hw_factor=150.0, seed=2021)


def run_rank(args):
    """Learned ranking: hub-frequency targets from GPU labelings of seeded
    small graphs, GPU training, then the learned and the plain order compared
    on unseen large graphs (labels exact under both)."""
    import plant_gb300 as P
    from plant_gb300 import ranking
    from oracle import oracle as O
    out = {"metric": "learned ranking vs plain order (average label size, GPU build time)",
           "unit": "avg label entries per vertex side", "higher_is_better": False,
           "data": "synthetic (seeded generators)", "n_gpus": 1}
    if args.rank_load:
        net = P.RankNet.load(args.rank_load)
        out["training"] = {"loaded": os.path.basename(args.rank_load)}
    else:
        t0 = time.time()
        samples = ranking.training_set(args.rank_graphs, seed=1)
        t_label = time.time() - t0
        net = P.RankNet(3, seed=1)
        rep = ranking.train(net, samples, epochs=args.rank_epochs)
        out["training"] = {"graphs": len(samples), "label_s": t_label, "epochs": rep.epochs,
                           "steps": rep.steps, "train_s": rep.seconds,
                           "loss_first_epoch": rep.first_epoch_loss, "loss_last_epoch": rep.last_epoch_loss,
                           "vertices": int(sum(s_.graph.get_n() for s_ in samples))}
        del samples
        if args.rank_save:
            net.save(args.rank_save)
    evals = []
    for spec in [x for x in args.rank_eval.split(",") if x]:
        g = eval_graph(P, spec)
        n = g.get_n()
        g.to_device()
        t = time.time()
        plain = ranking.plain_order(g, seed=1)
        t_plain = time.time() - t
        t = time.time()
        learned = net.order(g, seed=1)
        t_learned = time.time() - t
        Lp = P.build(g, plain)
        sp = Lp.stats()
        Ll = P.build(g, learned)
        sl = Ll.stats()
        # exactness: both labelings answer 1M sampled pairs identically, and a
        # few pairs equal plain Dijkstra on the CPU
        pairs = P.generate_query(1 << 20, n, seed=5)
        same = bool(np.array_equal(P.query(Lp, pairs), P.query(Ll, pairs)))
        off, head, ln = g.csr(True)
        og = O.OGraph.from_csr(n, off, head, ln)
        few = pairs[:8]
        dj = [og.dijkstra(int(u))[int(v)] for u, v in few]
        dq = P.query(Ll, few)
        dj_ok = bool(all(int(a) == int(b) for a, b in zip(dj, dq)))
        evals.append({"graph": spec, "vertices": n, "arcs": int(g.out_arcs()),
                      "plain": {"kind": "degree" if ranking.is_heavy_tailed(g) else "betweenness(256)",
                                "avg_label": sp["avg_label"], "build_ms": sp["build_ms"], "order_s": t_plain},
                      "learned": {"avg_label": sl["avg_label"], "build_ms": sl["build_ms"], "order_s": t_learned},
                      "label_ratio": sl["avg_label"] / sp["avg_label"],
                      "build_ratio": sl["build_ms"] / sp["build_ms"],
                      "used": "learned" if sl["avg_label"] <= sp["avg_label"] else "plain",
                      "queries_agree_1M": same, "dijkstra_pairs_agree": dj_ok})
        del Lp, Ll
        g.release_device()
        print(json.dumps(evals[-1]), file=sys.stderr, flush=True)
    out["evaluation"] = evals
    out["value"] = float(np.mean([e["label_ratio"] for e in evals])) if evals else None
    out["value_meaning"] = "mean learned/plain average-label ratio (<= 1: the learned order is used)"
    print(json.dumps(out), flush=True)


def run_ingest(args):
    """Graph ingestion: the grid workload written as a DIMACS and as a SNAP
    file, each read twice by the host parsers (chl_graph_load) and twice by
    the GPU path (chl_graph_load_gpu) in one process; the CSRs of the two
    paths are compared."""
    import shutil
    import tempfile
    import plant_gb300 as P
    g = P.Graph.grid(args.side, args.side, highways=args.highways, seed=1)
    d = tempfile.mkdtemp(prefix="chl_ingest_")
    try:
        files = {"dimacs": os.path.join(d, "g.gr"), "snap": os.path.join(d, "g.txt")}
        g.write(files["dimacs"])
        off, head, _ = g.csr(True)
        src = np.repeat(np.arange(g.get_n(), dtype=np.int64), np.diff(off.astype(np.int64)))
        with open(files["snap"], "w") as f:
            f.write(f"# Nodes: {g.get_n()} Edges: {len(head)}\n# FromNodeId\tToNodeId\n")
            np.savetxt(f, np.stack([src, head.astype(np.int64)], 1), fmt="%d\t%d")
        tiny = os.path.join(d, "t.gr")
        with open(tiny, "w") as f:
            f.write("p sp 2 1\na 1 2 1\n")
        P.Graph.read_gpu(tiny)   # CUDA context set-up outside the timings
        out = {"metric": "graph ingestion time (file to CSR)", "unit": "s", "higher_is_better": False,
               "data": "synthetic (seeded generator)",
               "config": {"workload": f"grid{args.side}x{args.side}+hw{args.highways}",
                          "vertices": g.get_n(), "arcs": int(len(head))}}
        for fmt, path in files.items():
            res = {"bytes": os.path.getsize(path)}
            got = {}
            for way in ("host", "gpu"):
                ts = []
                for _ in range(2):
                    t0 = time.perf_counter()
                    if way == "host":
                        got[way] = P.Graph.read(path)
                    else:
                        got[way], used = P.Graph.read_gpu(path)
                        res["parsed_on_gpu"] = bool(used)
                    ts.append(round(time.perf_counter() - t0, 4))
                res[way + "_s"] = ts
            res["identical"] = all(np.array_equal(a, b) for fwd in (True, False)
                                   for a, b in zip(got["host"].csr(fwd), got["gpu"].csr(fwd)))
            res["speedup_second_read"] = round(res["host_s"][1] / max(res["gpu_s"][1], 1e-9), 1)
            out[fmt] = res
        print(json.dumps(out), flush=True)
    finally:
        shutil.rmtree(d, ignore_errors=True)


def main():
    args = parse()
    if args.rank:
        run_rank(args)
        return
    if args.ingest:
        run_ingest(args)
        return
    global METRIC
    if args.workload == "rmat":
        METRIC = METRIC_RMAT
    ws, rank = dist_info()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank)


if __name__ == "__main__":
    main()
