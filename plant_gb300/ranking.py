"""Vertex ranking for CHL: the plain GPU orders and the learned one.

* ``plain_order``: degree order for heavy-tailed graphs, sampled betweenness
  (Brandes from 256 seeded sources) for road-like ones, both on the GPU.
* ``training_set`` / ``train``: the learned ranking is fitted to per-vertex
  hub frequencies (how many label entries name the vertex as their hub) of
  GPU labelings of many small seeded graphs, half RMAT and half perturbed
  grids, labelled under their plain order.
* ``select_order``: the learned order is used only when the labels it
  produces are no larger on average than the plain order's; both labelings
  are exact, so the choice changes label size and build time only.

No reference counterpart: the reference reads a precomputed order file
(shared_memory/hhl.cpp:36-37; README.md:24 names the outside tools).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import Graph, Order, RankNet, build

HEAVY_TAIL_RATIO = 16.0   # max degree / mean degree above this: degree order


def is_heavy_tailed(g: Graph) -> bool:
    d = g.degrees(True).astype(np.float64)
    if not g.symmetric():
        d = d + g.degrees(False)
    mean = d.mean() if d.size else 0.0
    return bool(mean > 0 and d.max() / mean > HEAVY_TAIL_RATIO)


def plain_order(g: Graph, seed: int = 1, sources: int = 256) -> np.ndarray:
    """Degree order for heavy-tailed graphs, else sampled betweenness."""
    if is_heavy_tailed(g):
        return Order.degree(g, seed)
    return Order.betweenness(g, sources, seed)


def hub_target(labels, order) -> np.ndarray:
    """Standardised log1p hub frequency per vertex (the regression target)."""
    f = np.log1p(labels.hub_freq(order).astype(np.float64))
    sd = f.std()
    return ((f - f.mean()) / (sd if sd > 1e-12 else 1.0)).astype(np.float32)


@dataclass
class Sample:
    name: str
    graph: Graph
    target: np.ndarray
    avg_label: float


def training_graph(i: int, seed: int = 1) -> tuple[str, Graph]:
    """The i-th seeded training graph: 2^12..2^15 vertices, even i RMAT
    (a, b, c = 0.57, 0.19, 0.19, 16 arcs per vertex), odd i a perturbed grid
    with highways."""
    scale = 12 + (i // 2) % 4
    s = seed * 1000003 + i
    if i % 2 == 0:
        return f"rmat{scale}_{i}", Graph.rmat(scale, 16, 0.57, 0.19, 0.19, seed=s)
    side = int(round(math.sqrt(1 << scale)))
    hw = max(1, (side * side) // 500)
    return f"grid{side}_{i}", Graph.grid(side, side, highways=hw, hw_steps=max(2, side // 8), seed=s)


def training_set(count: int = 256, seed: int = 1, log=None) -> list[Sample]:
    """Label `count` seeded small graphs on the GPU under their plain order."""
    out = []
    for i in range(count):
        name, g = training_graph(i, seed)
        order = plain_order(g, seed=1)
        L = build(g, order)
        out.append(Sample(name, g, hub_target(L, order), L.get_avg()))
        g.release_device()
        if log:
            log(f"labelled {name}: n={g.get_n()} avg={L.get_avg():.2f}")
        del L
    return out


@dataclass
class TrainReport:
    epochs: int
    steps: int
    seconds: float
    first_epoch_loss: float
    last_epoch_loss: float
    losses: list = field(default_factory=list)


def train(net: RankNet, samples: list[Sample], epochs: int = 20, lr: float = 2e-3,
          lr_final: float = 2e-4, seed: int = 1, feature_seed: int = 1) -> TrainReport:
    """Adam over the samples in a seeded shuffled order each epoch, learning
    rate decayed geometrically from lr to lr_final."""
    rng = np.random.default_rng(seed)
    losses = []
    steps = 0
    t0 = time.perf_counter()
    total = max(1, epochs * len(samples) - 1)
    for e in range(epochs):
        acc = 0.0
        for j in rng.permutation(len(samples)):
            rate = lr * (lr_final / lr) ** (steps / total)
            acc += net.train_step(samples[j].graph, samples[j].target, rate, feature_seed)
            steps += 1
        losses.append(acc / max(1, len(samples)))
    return TrainReport(epochs, steps, time.perf_counter() - t0, losses[0] if losses else 0.0,
                       losses[-1] if losses else 0.0, losses)


@dataclass
class Choice:
    order: np.ndarray
    labels: object
    learned: bool
    plain_avg: float
    learned_avg: float
    plain_ms: float
    learned_ms: float


def select_order(g: Graph, net: RankNet, plain=None, seed: int = 1, **build_kw) -> Choice:
    """Build under the plain and the learned order; keep the learned labels
    only if their average size is no larger."""
    if plain is None:
        plain = plain_order(g, seed)
    Lp = build(g, plain, **build_kw)
    sp = Lp.stats()
    learned = net.order(g, seed)
    Ll = build(g, learned, **build_kw)
    sl = Ll.stats()
    use = sl["avg_label"] <= sp["avg_label"]
    return Choice(learned if use else np.asarray(plain, np.uint32), Ll if use else Lp, bool(use),
                  sp["avg_label"], sl["avg_label"], sp["build_ms"], sl["build_ms"])
