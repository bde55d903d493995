"""ctypes binding of the CPU oracle (liboracle.so, built from chl_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker / baseline, never by the
product.  The reference binaries of oracle/_ref exist only where the
reference sources were present when oracle/Makefile ran (x86 build host).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# the reference checkout: $CHL_REFERENCE, else a directory named `reference`
# beside this repository (absent on hosts that only run the prebuilt tests)
REF_SRC = os.environ.get("CHL_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_I32P = C.POINTER(C.c_int32)
_U64P = C.POINTER(C.c_uint64)
_F64P = C.POINTER(C.c_double)

_SIG = {
    "og_read_dimacs": (_P, [C.c_char_p]),
    "og_from_arcs": (_P, [C.c_uint32, C.c_size_t, _U32P, _U32P, _I32P]),
    "og_n": (C.c_uint32, [_P]),
    "og_arcs": (C.c_uint64, [_P, C.c_int]),
    "og_export": (None, [_P, C.c_int, _U64P, _U32P, _I32P]),
    "og_free": (None, [_P]),
    "ol_free": (None, [_P]),
    "ol_total": (C.c_uint64, [_P]),
    "ol_avg": (C.c_double, [_P]),
    "ol_export": (None, [_P, _U64P, _U32P, _I32P]),
    "ol_import": (_P, [C.c_uint32, _U64P, _U32P, _I32P]),
    "ol_write": (C.c_int, [_P, C.c_char_p]),
    "ol_query": (C.c_int32, [_P, C.c_uint32, C.c_uint32]),
    "ol_query_batch": (None, [_P, _U32P, C.c_size_t, _I32P, C.c_int]),
    "og_dijkstra": (None, [_P, C.c_uint32, C.c_int, _I32P]),
    "og_gll": (_P, [_P, _U32P, C.c_uint32, C.c_int, C.c_uint64, _F64P]),
    "og_gll_steps": (_P, [_P, _U32P, C.c_uint32, C.c_int, C.c_uint64, _F64P, C.c_uint32, _U32P, _U32P, _F64P]),
    "og_replay_new": (_P, [_P, _U32P, C.c_uint32, C.c_int, _P]),
    "og_replay_free": (None, [_P]),
    "og_replay_run": (C.c_uint64, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _F64P]),
    "og_pll_trace": (None, [_P, _U32P, C.c_uint32, _U64P]),
    "og_plant_all": (_P, [_P, _U32P, C.c_uint32, _U32P, _U32P]),
    "og_canonical_check": (C.c_uint64, [_P, _U32P, _P]),
    "og_degree_order": (None, [_P, C.c_uint64, _U32P]),
    "og_bc_sources": (None, [C.c_uint32, C.c_uint32, C.c_uint64, _U32P]),
    "og_betweenness": (None, [_P, _U32P, C.c_uint32, _F64P]),
    "og_betweenness_order": (None, [_P, C.c_uint32, C.c_uint64, _U32P]),
    "ol_digest": (C.c_uint64, [_P]),
    "og_gen_grid": (_P, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_uint32,
                         C.c_uint32, C.c_double, C.c_uint64]),
    "og_gen_rmat": (_P, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64]),
    "og_order_digest": (C.c_uint64, [_U32P, C.c_uint32]),
}

_lib = None


def build() -> str:
    """Compile liboracle.so (and oracle/_ref when the reference is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if os.path.isdir(os.path.join(REF_SRC, "shared_memory")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def ref_bin(name: str):
    p = os.path.join(REF_DIR, name)
    return p if os.path.exists(p) else None


def _u32(a):
    return np.ascontiguousarray(a, np.uint32)


class OGraph:
    def __init__(self, h):
        if not h:
            raise ValueError("oracle could not read graph")
        self.h = C.c_void_p(h)

    @classmethod
    def read_dimacs(cls, path):
        return cls(lib().og_read_dimacs(os.fsencode(path)))

    @classmethod
    def from_csr(cls, n, off, head, length):
        """Graph whose forward arcs are the given CSR (reverse arcs mirrored)."""
        off = np.asarray(off, np.uint64)
        src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off).astype(np.int64))
        h = _u32(head)
        w = np.ascontiguousarray(length, np.int32)
        return cls(lib().og_from_arcs(n, len(src), src.ctypes.data_as(_U32P), h.ctypes.data_as(_U32P),
                                      w.ctypes.data_as(_I32P)))

    @classmethod
    def grid(cls, rows, cols, del_frac=0.05, diag_frac=0.01, wmin=1, wmax=1000, highways=0, hw_steps=64,
             hw_factor=150.0, seed=1):
        """The package's seeded road-like grid (og_gen_grid), built on the CPU."""
        return cls(lib().og_gen_grid(rows, cols, del_frac, diag_frac, wmin, wmax, highways, hw_steps, hw_factor,
                                     seed))

    @classmethod
    def rmat(cls, scale, ef=16, a=0.57, b=0.19, c=0.19, seed=1):
        """The package's seeded RMAT graph (og_gen_rmat), built on the CPU."""
        return cls(lib().og_gen_rmat(scale, ef, a, b, c, seed))

    @property
    def n(self):
        return lib().og_n(self.h)

    def csr(self, side):
        m = lib().og_arcs(self.h, side)
        off = np.zeros(self.n + 1, np.uint64)
        head = np.zeros(max(m, 1), np.uint32)
        ln = np.zeros(max(m, 1), np.int32)
        lib().og_export(self.h, side, off.ctypes.data_as(_U64P), head.ctypes.data_as(_U32P),
                        ln.ctypes.data_as(_I32P))
        return off, head[:m], ln[:m]

    def dijkstra(self, src, forward=True):
        d = np.zeros(self.n, np.int32)
        lib().og_dijkstra(self.h, src, int(forward), d.ctypes.data_as(_I32P))
        return d

    def degree_order(self, seed):
        o = np.zeros(self.n, np.uint32)
        lib().og_degree_order(self.h, seed, o.ctypes.data_as(_U32P))
        return o

    def betweenness_order(self, sources, seed):
        o = np.zeros(self.n, np.uint32)
        lib().og_betweenness_order(self.h, sources, seed, o.ctypes.data_as(_U32P))
        return o

    def betweenness(self, sources, seed):
        src = np.zeros(sources, np.uint32)
        lib().og_bc_sources(self.n, sources, seed, src.ctypes.data_as(_U32P))
        bc = np.zeros(self.n, np.float64)
        lib().og_betweenness(self.h, src.ctypes.data_as(_U32P), sources, bc.ctypes.data_as(_F64P))
        return bc

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.og_free(self.h)
            self.h = None


class OLabels:
    def __init__(self, h):
        self.h = C.c_void_p(h)

    @classmethod
    def from_csr(cls, n, off, hub, dist):
        off = np.ascontiguousarray(off, np.uint64)
        hub = _u32(hub)
        dist = np.ascontiguousarray(dist, np.int32)
        return cls(lib().ol_import(n, off.ctypes.data_as(_U64P), hub.ctypes.data_as(_U32P),
                                   dist.ctypes.data_as(_I32P)))

    def total(self):
        return lib().ol_total(self.h)

    def avg(self):
        return lib().ol_avg(self.h)

    def export(self, n):
        t = self.total()
        off = np.zeros(2 * n + 1, np.uint64)
        hub = np.zeros(max(t, 1), np.uint32)
        dist = np.zeros(max(t, 1), np.int32)
        lib().ol_export(self.h, off.ctypes.data_as(_U64P), hub.ctypes.data_as(_U32P), dist.ctypes.data_as(_I32P))
        return off, hub[:t], dist[:t]

    def digest(self):
        """Label digest (oracle/chl_digest.h) of these labels."""
        return int(lib().ol_digest(self.h))

    def write(self, path):
        if lib().ol_write(self.h, os.fsencode(path)):
            raise IOError(path)

    def query(self, pairs, threads=None):
        p = _u32(np.asarray(pairs).reshape(-1, 2))
        out = np.zeros(len(p), np.int32)
        lib().ol_query_batch(self.h, p.ctypes.data_as(_U32P), len(p), out.ctypes.data_as(_I32P),
                             threads or os.cpu_count() or 1)
        return out

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ol_free(self.h)
            self.h = None


def order_digest(order) -> int:
    """Order digest (oracle/chl_digest.h)."""
    o = _u32(order)
    return int(lib().og_order_digest(o.ctypes.data_as(_U32P), len(o)))


def gll(g: OGraph, order, threads=None, sf=32):
    o = _u32(order)
    secs = C.c_double()
    n = len(o)
    h = lib().og_gll(g.h, o.ctypes.data_as(_U32P), n, threads or os.cpu_count() or 1, int(sf * n),
                     C.byref(secs))
    return OLabels(h), secs.value


def gll_steps(g: OGraph, order, threads=None, sf=32, max_steps=1 << 16):
    """gll() that also returns its supersteps: (labels, secs, ends, step_secs);
    superstep k covers roots [ends[k-1], ends[k])."""
    o = _u32(order)
    secs = C.c_double()
    n = len(o)
    ends = np.zeros(max_steps, np.uint32)
    ss = np.zeros(max_steps, np.float64)
    ns = C.c_uint32()
    h = lib().og_gll_steps(g.h, o.ctypes.data_as(_U32P), n, threads or os.cpu_count() or 1, int(sf * n),
                           C.byref(secs), max_steps, C.byref(ns), ends.ctypes.data_as(_U32P),
                           ss.ctypes.data_as(_F64P))
    k = min(ns.value, max_steps)
    return OLabels(h), secs.value, ends[:k].copy(), ss[:k].copy()


class Replay:
    """Re-runs root ranges of one superstep of a GLL build with that
    superstep's committed state taken from the complete labels
    (og_replay_run)."""

    def __init__(self, g: OGraph, order, complete: OLabels, threads=None):
        self._order = _u32(order)
        self._g, self._complete = g, complete   # kept alive for the C side
        self.threads = threads or os.cpu_count() or 1
        self.h = C.c_void_p(lib().og_replay_new(g.h, self._order.ctypes.data_as(_U32P), len(self._order),
                                                self.threads, complete.h))

    def run(self, s_begin, r_begin, r_end):
        """(labels kept, seconds) of roots [r_begin, r_end) of the superstep
        that starts at root s_begin."""
        secs = C.c_double()
        kept = lib().og_replay_run(self.h, s_begin, r_begin, r_end, C.byref(secs))
        return int(kept), secs.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.og_replay_free(self.h)
            self.h = None


def pll_trace(g: OGraph, order) -> dict:
    """Sequential PLL work counts (og_pll_trace): settled vertices, label
    entries scanned by prune tests (to the first witness), arcs relaxed,
    labels written, and the build roofline's algorithmic bytes: 8 B per
    entry of every settled vertex's list, per out-arc of every settled
    vertex and per label written.  Single-threaded."""
    o = _u32(order)
    out = (C.c_uint64 * 8)()
    lib().og_pll_trace(g.h, o.ctypes.data_as(_U32P), len(o), out)
    return {"settled": out[0], "label_reads": out[1], "arcs": out[2], "labels": out[3],
            "scanned_bytes": out[4], "list_entries": out[5], "settled_out_arcs": out[6],
            "algorithmic_bytes": out[7]}


def plant_all(g: OGraph, order):
    o = _u32(order)
    n = len(o)
    ts = np.zeros(n, np.uint32)
    lc = np.zeros(n, np.uint32)
    h = lib().og_plant_all(g.h, o.ctypes.data_as(_U32P), n, ts.ctypes.data_as(_U32P), lc.ctypes.data_as(_U32P))
    return OLabels(h), ts, lc


def canonical_check(g: OGraph, order, labels: OLabels) -> int:
    o = _u32(order)
    return int(lib().og_canonical_check(g.h, o.ctypes.data_as(_U32P), labels.h))
