"""CPU restatement of the learned-ranking network (features, forward, backward).

TEST INFRASTRUCTURE ONLY: the checker for the GPU network's features,
scores and gradients; nothing in the product imports it.  The network has no
counterpart in the reference (which reads its order from a file,
shared_memory/hhl.cpp:36-37), so parity here is against this restatement of
the network's own definition, with two settings:

* ``emulate=True`` rounds to BF16 at exactly the points where the GPU stores
  or feeds BF16 (h_l, m_l, GEMM weights, dz before the GEMMs): the remaining
  difference is FP32 accumulation order, so the gradients agree closely;
* ``emulate=False`` is the plain FP64 network: it bounds what BF16 costs and,
  checked against central finite differences, pins the backward formulas.

Graph inputs are CSR arrays: off_out/head_out (out-arcs) and off_in/head_in
(in-arcs); deg(v) = out + in arcs.
"""
from __future__ import annotations

import numpy as np

H = 64
NF = 3
K2 = 2 * H
CLUSTER_SAMPLES = 16
CLUSTER_SCAN = 256
M64 = (1 << 64) - 1


def param_count(layers: int) -> int:
    return NF * H + H + layers * (K2 * H + H) + H + 1


def unpack(p: np.ndarray, layers: int):
    """W0[3,H], b0[H], [(W_l[2H,H], b_l[H])], wout[H], bout[1]."""
    p = np.asarray(p, np.float64)
    i = 0

    def take(k, shape):
        nonlocal i
        a = p[i:i + k].reshape(shape)
        i += k
        return a

    W0 = take(NF * H, (NF, H))
    b0 = take(H, (H,))
    Ls = [(take(K2 * H, (K2, H)), take(H, (H,))) for _ in range(layers)]
    wout = take(H, (H,))
    bout = take(1, (1,))
    assert i == p.size
    return W0, b0, Ls, wout, bout


def pack(W0, b0, Ls, wout, bout) -> np.ndarray:
    parts = [W0.ravel(), b0.ravel()]
    for W, b in Ls:
        parts += [W.ravel(), b.ravel()]
    parts += [wout.ravel(), np.asarray(bout).ravel()]
    return np.concatenate(parts)


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _mix(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def raw_features(off_out, head_out, off_in, seed: int) -> np.ndarray:
    """[log1p deg, log1p 2-hop degree sum, sampled clustering] per vertex."""
    off_out = np.asarray(off_out, np.int64)
    off_in = np.asarray(off_in, np.int64)
    head_out = np.asarray(head_out, np.int64)
    n = off_out.size - 1
    outd = np.diff(off_out)
    deg = outd + np.diff(off_in)
    x = np.zeros((n, NF), np.float32)
    for v in range(n):
        b, e = off_out[v], off_out[v + 1]
        two = float(deg[head_out[b:e]].sum()) if e > b else 0.0
        cc = 0.0
        d = int(e - b)
        if d >= 2:
            hit = 0
            for k in range(CLUSTER_SAMPLES):
                h = _mix(seed ^ ((v * 0x100000001B3 + k) & M64))
                i = h % d
                j = (h >> 32) % (d - 1)
                if j >= i:
                    j += 1
                a, c = int(head_out[b + i]), int(head_out[b + j])
                ab = off_out[a]
                ae = min(off_out[a + 1], ab + CLUSTER_SCAN)
                if np.any(head_out[ab:ae] == c):
                    hit += 1
            cc = hit / CLUSTER_SAMPLES
        x[v, 0] = np.float32(np.log1p(float(deg[v])))
        x[v, 1] = np.float32(np.log1p(two))
        x[v, 2] = np.float32(cc)
    return x


def standardise(x: np.ndarray) -> np.ndarray:
    """Per-column (x - mean) / population sd, in float64, stored as float32."""
    x = np.asarray(x, np.float32)
    n = x.shape[0]
    out = np.zeros_like(x)
    for k in range(x.shape[1]):
        col = x[:, k].astype(np.float64)
        mean = col.sum() / n if n else 0.0
        sd = np.sqrt(((col - mean) ** 2).sum() / n) if n > 1 else 0.0
        inv = 1.0 / sd if sd > 1e-12 else 0.0
        out[:, k] = ((col - mean) * inv).astype(np.float32)
    return out


def features(off_out, head_out, off_in, seed: int) -> np.ndarray:
    return standardise(raw_features(off_out, head_out, off_in, seed))


class _Csr:
    def __init__(self, off_out, head_out, off_in, head_in):
        self.off_out = np.asarray(off_out, np.int64)
        self.head_out = np.asarray(head_out, np.int64)[: self.off_out[-1]]
        self.n = self.off_out.size - 1
        outd = np.diff(self.off_out)
        self.src_out = np.repeat(np.arange(self.n), outd)
        # 1/outdeg as the GPU forms it: an FP32 reciprocal
        self.inv = np.zeros(self.n)
        nz = outd > 0
        self.inv[nz] = (np.float32(1.0) / outd[nz].astype(np.float32)).astype(np.float64)

    def mean_out(self, h):
        """m(v) = mean of h over v's out-neighbours (0 without any)."""
        s = np.zeros_like(h)
        np.add.at(s, self.src_out, h[self.head_out])
        return s * self.inv[:, None]

    def mean_out_T(self, g):
        """Adjoint of mean_out: out(u) = sum over arcs v->u of g(v) / outdeg(v)."""
        out = np.zeros_like(g)
        np.add.at(out, self.head_out, (g * self.inv[:, None])[self.src_out])
        return out


def forward(p, layers, x, csr: _Csr, emulate: bool):
    """Returns scores and the cache for backward."""
    q = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    W0, b0, Ls, wout, bout = unpack(p, layers)
    x = np.asarray(x, np.float64)
    z0 = x @ W0 + b0
    h = [q(np.maximum(z0, 0.0))]
    ms = [None]
    for W, b in Ls:
        m = q(csr.mean_out(h[-1]))
        A = np.concatenate([h[-1], m], axis=1)
        z = A @ q(W) + b
        ms.append(m)
        h.append(q(np.maximum(z, 0.0)))
    s = h[-1] @ wout + bout[0]
    return s, (x, h, ms)


def loss_and_grad(p, layers, x, csr: _Csr, y, emulate: bool):
    """MSE loss mean((s - y)^2) and its gradient (float64, packed layout)."""
    q = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    W0, b0, Ls, wout, bout = unpack(p, layers)
    s, (x, h, ms) = forward(p, layers, x, csr, emulate)
    n = s.size
    y = np.asarray(y, np.float64)
    r = s - y
    loss = float((r * r).sum() / n)
    ds = 2.0 * r / n
    gwout = h[-1].T @ ds
    gbout = np.array([ds.sum()])
    dh = np.outer(ds, wout)
    gLs = [None] * layers
    for l in range(layers, 0, -1):
        W, _ = Ls[l - 1]
        dz = dh * (h[l] > 0)
        dzq = q(dz)
        A = np.concatenate([h[l - 1], ms[l]], axis=1)
        gW = A.T @ dzq
        gb = dz.sum(axis=0)
        gLs[l - 1] = (gW, gb)
        dA = dzq @ q(W).T
        dh = dA[:, :H] + csr.mean_out_T(dA[:, H:])
    dz0 = dh * (h[0] > 0)
    gW0 = x.T @ dz0
    gb0 = dz0.sum(axis=0)
    return loss, pack(gW0, gb0, gLs, gwout, gbout)


def csr_of(off_out, head_out, off_in, head_in) -> _Csr:
    return _Csr(off_out, head_out, off_in, head_in)


def init_params(layers: int, seed: int) -> np.ndarray:
    """Glorot-uniform weights, zero biases (any generator: used by tests that
    set the GPU network's parameters explicitly)."""
    rng = np.random.default_rng(seed)

    def g(fi, fo, shape):
        lim = np.sqrt(6.0 / (fi + fo))
        return rng.uniform(-lim, lim, shape)

    W0 = g(NF, H, (NF, H))
    Ls = [(g(K2, H, (K2, H)), np.zeros(H)) for _ in range(layers)]
    return pack(W0, np.zeros(H), Ls, g(H, 1, (H,)), np.zeros(1)).astype(np.float32)
