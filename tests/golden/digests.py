"""NumPy restatement of the digests in oracle/chl_digest.h (test helpers).

Graphs use the label layout with one list per vertex: list v holds the
forward arcs of v as (head, length) in CSR order.  All arithmetic is modulo
2^64 (NumPy uint64 arrays wrap).
"""
from __future__ import annotations

import numpy as np

C_N = np.uint64(0x243F6A8885A308D3)
C_L = np.uint64(0x13198A2E03707344)
C_E = np.uint64(0xA4093822299F31D0)
C_O = np.uint64(0x082EFA98EC4E6C89)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def mix(z):
    """SplitMix64's finaliser on a uint64 array (copy)."""
    z = np.array(z, dtype=np.uint64, copy=True)
    z ^= z >> np.uint64(30)
    z *= _M1
    z ^= z >> np.uint64(27)
    z *= _M2
    z ^= z >> np.uint64(31)
    return z


def _wsum(x) -> int:
    return int(np.sum(np.asarray(x, np.uint64), dtype=np.uint64))


def _head(n) -> int:
    return int(mix(np.array([n], np.uint64) + C_N)[0])


def _lists_sum(nlists, off, a, b) -> int:
    """Sum of the list and entry terms of `nlists` lists whose entries are
    (a[k], b[k]) for k in off[i] .. off[i+1]."""
    off = np.asarray(off, np.uint64)
    sizes = np.diff(off)
    base = mix(np.arange(nlists, dtype=np.uint64) + C_L)
    total = _wsum(mix(base ^ sizes))
    m = int(off[-1])
    if m:
        owner = np.repeat(np.arange(nlists, dtype=np.int64), sizes.astype(np.int64))
        pos = np.arange(m, dtype=np.uint64) - off[:-1][owner]
        val = (np.asarray(a, np.uint64)[:m] << np.uint64(32)) | (
            np.asarray(b, np.int64)[:m].astype(np.uint64) & np.uint64(0xFFFFFFFF))
        total += _wsum(mix(base[owner] ^ mix(pos + C_E) ^ val))
    return total


def label_digest(n, off, hub, dist) -> int:
    """Digest of a labeling exported as CSR over lists 2v + side."""
    return (_head(n) + _lists_sum(2 * n, off, hub, dist)) % (1 << 64)


def graph_digest(n, off, head, length) -> int:
    """Digest of a graph's forward CSR: list v = the out-arcs (head, length)
    of v in stored order."""
    return (_head(n) + _lists_sum(n, off, head, length)) % (1 << 64)


def order_digest(order) -> int:
    o = np.asarray(order, np.uint64)
    t = _head(len(o)) + _wsum(mix(mix(np.arange(len(o), dtype=np.uint64) + C_O) ^ o))
    return t % (1 << 64)
