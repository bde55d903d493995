"""plant_gb300 -- GB300-native canonical hub labeling (CHL).

Python mirror of the reference's `hl` C++ interface, over the C ABI in
include/chl.h (libchl.so, hand-written CUDA for sm_103a):

  reference (namespace hl)                         here
  Graph::read(file, undirected)   graph.hpp:327    Graph.read(path, undirected)
  Order::read / Order::write      ordering.hpp:37  Order.read / Order.write
  run_paraPLL(g, order, ...)      akiba.hpp:132    run_paraPLL(g, order, sf=32)
  run(g, order, ..., ps, ...)     (distributed)    run(g, order, phase_switch=1024)
  Labeling::query(u, v)           labeling.hpp:56  Labeling.query(u, v)
  Labeling::write / read          labeling.hpp:167 Labeling.write / Labeling.read
  Labeling::get_avg               labeling.hpp:153 Labeling.get_avg()
  batchLocalQuery / hl::query     query_funcs.hpp  query(labels, pairs)

There is no CPU fallback: if libchl.so is missing or no CUDA device is
usable, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libchl.so")

CHL_OK = 0
CHL_ERR_IO = 1
CHL_ERR_FORMAT = 2
CHL_ERR_OOM = 3
CHL_ERR_TIMEOUT = 4
CHL_ERR_INVALID = 5
CHL_ERR_CUDA = 6
INFTY = 2147483647

MODE_HYBRID, MODE_GLL, MODE_PLANT = 0, 1, 2


class CHLError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        super().__init__(f"{what}: {_status_str(status)}" + (f" ({detail})" if detail else ""))
        self.status = status


class BuildOpts(C.Structure):
    _fields_ = [("mode", C.c_int32), ("sf", C.c_double), ("ps", C.c_double),
                ("autotune", C.c_int32), ("use_graphs", C.c_int32), ("verbose", C.c_int32),
                ("first_superstep", C.c_uint32), ("growth", C.c_double),
                ("max_warps", C.c_uint32), ("root_limit", C.c_uint32),
                ("superstep_extend", C.c_int32), ("label_cap", C.c_uint32), ("queue_split", C.c_int32),
                ("window_target", C.c_uint32), ("window_warps", C.c_uint32), ("reserved", C.c_uint32 * 1)]


class BuildStats(C.Structure):
    _fields_ = [("build_ms", C.c_double), ("tree_ms", C.c_double), ("sort_ms", C.c_double),
                ("commit_ms", C.c_double), ("h2d_ms", C.c_double), ("labels", C.c_uint64),
                ("visits", C.c_uint64), ("label_reads", C.c_uint64), ("arcs", C.c_uint64),
                ("supersteps", C.c_uint32), ("plant_roots", C.c_uint32),
                ("tree_launches", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("avg_label", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerOpts(C.Structure):
    _fields_ = [("max_inflight_pairs", C.c_uint32), ("max_requests", C.c_uint32),
                ("max_batch_pairs", C.c_uint32), ("reserved", C.c_uint32 * 5)]


_lib: Optional[C.CDLL] = None

_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_I32P = C.POINTER(C.c_int32)
_U64P = C.POINTER(C.c_uint64)
_F32P = C.POINTER(C.c_float)

# name -> (restype, argtypes)
SIGNATURES = {
    "chl_status_str": (C.c_char_p, [C.c_int]),
    "chl_last_error": (C.c_char_p, []),
    "chl_graph_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P)]),
    "chl_graph_load_gpu": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P), C.POINTER(C.c_int)]),
    "chl_graph_from_arcs": (C.c_int, [C.c_uint32, C.c_size_t, _U32P, _U32P, _I32P, C.c_int, C.POINTER(_P)]),
    "chl_graph_from_csr": (C.c_int, [C.c_uint32, _U64P, _U32P, _I32P, C.c_int, C.POINTER(_P)]),
    "chl_graph_write_dimacs": (C.c_int, [_P, C.c_char_p]),
    "chl_graph_n": (C.c_uint32, [_P]),
    "chl_graph_m": (C.c_uint64, [_P]),
    "chl_graph_out_arcs": (C.c_uint64, [_P]),
    "chl_graph_symmetric": (C.c_int, [_P]),
    "chl_graph_degree": (C.c_uint32, [_P, C.c_uint32]),
    "chl_graph_arcs": (C.c_int, [_P, C.c_uint32, C.c_int, _U32P, _I32P, C.c_uint32, _U32P]),
    "chl_graph_degrees": (C.c_int, [_P, C.c_int, _U32P]),
    "chl_graph_export": (C.c_int, [_P, C.c_int, _U64P, _U32P, _I32P]),
    "chl_graph_to_device": (C.c_int, [_P]),
    "chl_graph_release_device": (C.c_int, [_P]),
    "chl_graph_free": (None, [_P]),
    "chl_gen_grid": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_int32, C.c_int32,
                               C.c_uint32, C.c_uint32, C.c_double, C.c_uint64, C.POINTER(_P)]),
    "chl_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                               C.POINTER(_P)]),
    "chl_order_load": (C.c_int, [C.c_char_p, C.POINTER(_U32P), _U32P]),
    "chl_order_write": (C.c_int, [C.c_char_p, _U32P, C.c_uint32]),
    "chl_order_free": (None, [_U32P]),
    "chl_order_degree": (C.c_int, [_P, C.c_uint64, _U32P]),
    "chl_order_betweenness": (C.c_int, [_P, C.c_uint32, C.c_uint64, _U32P]),
    "chl_build_opts_default": (None, [C.POINTER(BuildOpts)]),
    "chl_build": (C.c_int, [_P, _U32P, C.c_uint32, C.POINTER(BuildOpts), C.POINTER(_P)]),
    "chl_graph_class": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "chl_build_get_stats": (C.c_int, [_P, C.POINTER(BuildStats)]),
    "chl_labels_write": (C.c_int, [_P, C.c_char_p]),
    "chl_labels_read": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "chl_avg_label": (C.c_double, [_P]),
    "chl_labels_n": (C.c_uint32, [_P]),
    "chl_labels_total": (C.c_uint64, [_P]),
    "chl_labels_get": (C.c_int, [_P, C.c_uint32, C.c_int, _U32P, _I32P, C.c_uint32, _U32P]),
    "chl_labels_list_sizes": (C.c_int, [_P, _U32P]),
    "chl_labels_export": (C.c_int, [_P, _U64P, _U32P, _I32P]),
    "chl_labels_import": (C.c_int, [C.c_uint32, _U64P, _U32P, _I32P, C.POINTER(_P)]),
    "chl_labels_hub_freq": (C.c_int, [_P, _U32P, _U32P]),
    "chl_labels_digest": (C.c_int, [_P, _U64P]),
    "chl_labels_save": (C.c_int, [_P, C.c_char_p]),
    "chl_labels_load": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "chl_labels_free": (None, [_P]),
    "chl_query_batch": (C.c_int, [_P, _U32P, C.c_size_t, _I32P, _P]),
    "chl_query_batch_noalloc": (C.c_int, [_P, _U32P, C.c_size_t, _I32P, _P]),
    "chl_query_batch_device": (C.c_int, [_P, _P, C.c_size_t, _P, _P]),
    "chl_query_bench": (C.c_int, [_P, C.c_size_t, C.c_uint64, C.c_int, C.c_uint32, C.POINTER(C.c_double), _U64P]),
    "chl_query_generate": (C.c_int, [_U32P, C.c_size_t, C.c_uint32, C.c_uint64]),
    "chl_query_load": (C.c_int, [C.c_char_p, C.POINTER(_U32P), C.POINTER(C.c_size_t)]),
    "chl_server_opts_default": (None, [C.POINTER(ServerOpts)]),
    "chl_server_create": (C.c_int, [_P, C.POINTER(ServerOpts), C.POINTER(_P)]),
    "chl_server_submit": (C.c_int, [_P, _U32P, C.c_size_t, _U64P]),
    "chl_server_wait": (C.c_int, [_P, C.c_uint64, _I32P, C.c_double, C.POINTER(C.c_double)]),
    "chl_server_stats": (C.c_int, [_P, _U64P, _U64P, _U64P]),
    "chl_server_blocked": (C.c_int, [_P, _U32P]),
    "chl_server_free": (None, [_P]),
    "chl_gnn_create": (C.c_int, [C.c_uint32, C.c_uint64, C.POINTER(_P)]),
    "chl_gnn_param_count": (C.c_size_t, [_P]),
    "chl_gnn_get_params": (C.c_int, [_P, _F32P]),
    "chl_gnn_set_params": (C.c_int, [_P, _F32P]),
    "chl_gnn_features": (C.c_int, [_P, C.c_uint64, _F32P]),
    "chl_gnn_predict": (C.c_int, [_P, _P, C.c_uint64, _F32P]),
    "chl_gnn_grad": (C.c_int, [_P, _P, C.c_uint64, _F32P, C.POINTER(C.c_double), _F32P]),
    "chl_gnn_train_step": (C.c_int, [_P, _P, C.c_uint64, _F32P, C.c_float, C.POINTER(C.c_double)]),
    "chl_gnn_order": (C.c_int, [_P, _P, C.c_uint64, _U32P]),
    "chl_gnn_free": (None, [_P]),
}


def lib() -> C.CDLL:
    """Load libchl.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise CHLError(CHL_ERR_CUDA, "libchl.so not built", "run plant_gb300.buildlib.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _status_str(s: int) -> str:
    try:
        return lib().chl_status_str(s).decode()
    except Exception:
        return f"status {s}"


def _check(status: int, what: str) -> None:
    if status != CHL_OK:
        detail = lib().chl_last_error().decode(errors="replace")
        raise CHLError(status, what, detail)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


# ------------------------------------------------------------------ graph
class Graph:
    """hl::Graph: adjacency after the reference's arc merge."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    @classmethod
    def read(cls, path: str, undirected: bool = False) -> "Graph":
        h = C.c_void_p()
        _check(lib().chl_graph_load(os.fsencode(path), int(undirected), C.byref(h)), f"read {path}")
        return cls(h)

    @classmethod
    def read_gpu(cls, path: str, undirected: bool = False):
        """Graph::read with DIMACS files parsed on the GPU; returns (graph,
        parsed_on_gpu).  Other formats go through the host parsers."""
        h = C.c_void_p()
        used = C.c_int(0)
        _check(lib().chl_graph_load_gpu(os.fsencode(path), int(undirected), C.byref(h), C.byref(used)),
               f"read {path}")
        return cls(h), bool(used.value)

    @classmethod
    def from_arcs(cls, n: int, src, dst, length, undirected: bool = False) -> "Graph":
        s, d = _u32(src), _u32(dst)
        w = np.ascontiguousarray(length, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().chl_graph_from_arcs(n, len(s), _ptr(s, _U32P), _ptr(d, _U32P), _ptr(w, _I32P),
                                         int(undirected), C.byref(h)), "graph from arcs")
        return cls(h)

    @classmethod
    def from_csr(cls, n: int, off, head, length, undirected: bool = False) -> "Graph":
        """Graph from an out-arc CSR (off[n+1], head, length), merged like
        from_arcs."""
        o = np.ascontiguousarray(off, dtype=np.uint64)
        if len(o) != n + 1:
            raise CHLError(CHL_ERR_INVALID, "graph from csr", "off must have n + 1 entries")
        hd = _u32(head)
        w = np.ascontiguousarray(length, dtype=np.int32)
        if len(hd) < int(o[-1]) or len(w) < int(o[-1]):
            raise CHLError(CHL_ERR_INVALID, "graph from csr", "head/length shorter than off[n]")
        h = C.c_void_p()
        _check(lib().chl_graph_from_csr(n, _ptr(o, _U64P), _ptr(hd, _U32P), _ptr(w, _I32P), int(undirected),
                                        C.byref(h)), "graph from csr")
        return cls(h)

    @classmethod
    def grid(cls, rows, cols, del_frac=0.05, diag_frac=0.01, wmin=1, wmax=1000, highways=0,
             hw_steps=64, hw_factor=150.0, seed=1) -> "Graph":
        h = C.c_void_p()
        _check(lib().chl_gen_grid(rows, cols, del_frac, diag_frac, wmin, wmax, highways, hw_steps,
                                  hw_factor, seed, C.byref(h)), "grid generator")
        return cls(h)

    @classmethod
    def rmat(cls, scale, ef=16, a=0.57, b=0.19, c=0.19, seed=1) -> "Graph":
        h = C.c_void_p()
        _check(lib().chl_gen_rmat(scale, ef, a, b, c, seed, C.byref(h)), "rmat generator")
        return cls(h)

    def write(self, path: str) -> None:
        _check(lib().chl_graph_write_dimacs(self._h, os.fsencode(path)), f"write {path}")

    def get_n(self) -> int:
        return lib().chl_graph_n(self._h)

    def get_m(self) -> int:
        return lib().chl_graph_m(self._h)

    def out_arcs(self) -> int:
        return lib().chl_graph_out_arcs(self._h)

    def graph_class(self) -> str:
        """Class of the graph in the tuned-schedule table (chl_graph_class)."""
        buf = C.create_string_buffer(128)
        _check(lib().chl_graph_class(self._h, buf, len(buf)), "graph class")
        return buf.value.decode()

    def symmetric(self) -> bool:
        return bool(lib().chl_graph_symmetric(self._h))

    def get_degree(self, v: int) -> int:
        return lib().chl_graph_degree(self._h, v)

    def arcs(self, v: int, forward: bool = True):
        cnt = C.c_uint32()
        _check(lib().chl_graph_arcs(self._h, v, int(forward), None, None, 0, C.byref(cnt)), "arcs")
        h = np.zeros(cnt.value, np.uint32)
        w = np.zeros(cnt.value, np.int32)
        _check(lib().chl_graph_arcs(self._h, v, int(forward), _ptr(h, _U32P), _ptr(w, _I32P),
                                    cnt.value, C.byref(cnt)), "arcs")
        return h, w

    def csr(self, forward: bool = True):
        """(off, head, len) numpy arrays of one direction."""
        n = self.get_n()
        off = np.zeros(n + 1, np.uint64)
        _check(lib().chl_graph_export(self._h, int(forward), _ptr(off, _U64P), None, None), "export")
        m = int(off[-1])
        head = np.zeros(max(m, 1), np.uint32)
        ln = np.zeros(max(m, 1), np.int32)
        _check(lib().chl_graph_export(self._h, int(forward), _ptr(off, _U64P), _ptr(head, _U32P),
                                      _ptr(ln, _I32P)), "export")
        return off, head[:m], ln[:m]

    def degrees(self, forward: bool = True) -> np.ndarray:
        d = np.zeros(self.get_n(), np.uint32)
        _check(lib().chl_graph_degrees(self._h, int(forward), _ptr(d, _U32P)), "degrees")
        return d

    def to_device(self) -> None:
        _check(lib().chl_graph_to_device(self._h), "graph to device")

    def release_device(self) -> None:
        _check(lib().chl_graph_release_device(self._h), "graph release")

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.chl_graph_free(self._h)
            self._h = None


# ------------------------------------------------------------------ order
class Order:
    """hl::Order: order[i] is the vertex of rank i."""

    @staticmethod
    def read(path: str) -> np.ndarray:
        p = _U32P()
        n = C.c_uint32()
        _check(lib().chl_order_load(os.fsencode(path), C.byref(p), C.byref(n)), f"read {path}")
        try:
            return np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.uint32)
        finally:
            lib().chl_order_free(p)

    @staticmethod
    def write(path: str, order) -> None:
        o = _u32(order)
        _check(lib().chl_order_write(os.fsencode(path), _ptr(o, _U32P), len(o)), f"write {path}")

    @staticmethod
    def degree(g: Graph, seed: int = 1) -> np.ndarray:
        o = np.zeros(g.get_n(), np.uint32)
        _check(lib().chl_order_degree(g._h, seed, _ptr(o, _U32P)), "degree order")
        return o

    @staticmethod
    def betweenness(g: Graph, sources: int = 256, seed: int = 1) -> np.ndarray:
        o = np.zeros(g.get_n(), np.uint32)
        _check(lib().chl_order_betweenness(g._h, sources, seed, _ptr(o, _U32P)), "betweenness order")
        return o


# ------------------------------------------------------------------ labels
class Labeling:
    """hl::Labeling: canonical labels, resident in device memory."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def read(cls, path: str) -> "Labeling":
        h = C.c_void_p()
        _check(lib().chl_labels_read(os.fsencode(path), C.byref(h)), f"read {path}")
        return cls(h)

    @classmethod
    def from_csr(cls, n: int, off, hub, dist) -> "Labeling":
        o = np.ascontiguousarray(off, np.uint64)
        hb = _u32(hub)
        d = np.ascontiguousarray(dist, np.int32)
        h = C.c_void_p()
        _check(lib().chl_labels_import(n, _ptr(o, _U64P), _ptr(hb, _U32P), _ptr(d, _I32P), C.byref(h)),
               "labels import")
        return cls(h)

    def write(self, path: str) -> None:
        _check(lib().chl_labels_write(self._h, os.fsencode(path)), f"write {path}")

    def save(self, path: str) -> None:
        """Binary CSR file (fast cold start; see load)."""
        _check(lib().chl_labels_save(self._h, os.fsencode(path)), f"save {path}")

    @classmethod
    def load(cls, path: str) -> "Labeling":
        h = C.c_void_p()
        _check(lib().chl_labels_load(os.fsencode(path), C.byref(h)), f"load {path}")
        return cls(h)

    def get_avg(self) -> float:
        return lib().chl_avg_label(self._h)

    def n(self) -> int:
        return lib().chl_labels_n(self._h)

    def total(self) -> int:
        return lib().chl_labels_total(self._h)

    def label(self, v: int, side: int):
        cnt = C.c_uint32()
        _check(lib().chl_labels_get(self._h, v, side, None, None, 0, C.byref(cnt)), "label")
        h = np.zeros(cnt.value, np.uint32)
        d = np.zeros(cnt.value, np.int32)
        _check(lib().chl_labels_get(self._h, v, side, _ptr(h, _U32P), _ptr(d, _I32P), cnt.value,
                                    C.byref(cnt)), "label")
        return h, d

    def export(self):
        """(off[2n+1], hub, dist) host CSR over lists 2v+side."""
        n = self.n()
        off = np.zeros(2 * n + 1, np.uint64)
        t = self.total()
        hub = np.zeros(max(t, 1), np.uint32)
        dist = np.zeros(max(t, 1), np.int32)
        _check(lib().chl_labels_export(self._h, _ptr(off, _U64P), _ptr(hub, _U32P), _ptr(dist, _I32P)),
               "export")
        return off, hub[:t], dist[:t]

    def list_sizes(self) -> np.ndarray:
        """sizes[2v+side] = |L(v, side)|."""
        z = np.zeros(2 * self.n(), np.uint32)
        _check(lib().chl_labels_list_sizes(self._h, _ptr(z, _U32P)), "list sizes")
        return z

    def stats(self) -> dict:
        s = BuildStats()
        _check(lib().chl_build_get_stats(self._h, C.byref(s)), "stats")
        return s.as_dict()

    def digest(self) -> int:
        """64-bit fingerprint of the label file's content, computed on the
        device (chl_labels_digest)."""
        d = C.c_uint64()
        _check(lib().chl_labels_digest(self._h, C.byref(d)), "label digest")
        return int(d.value)

    def hub_freq(self, order) -> np.ndarray:
        o = _u32(order)
        f = np.zeros(self.n(), np.uint32)
        _check(lib().chl_labels_hub_freq(self._h, _ptr(o, _U32P), _ptr(f, _U32P)), "hub freq")
        return f

    def query(self, u: int, v: int) -> int:
        """Labeling::query(u, v, f=true): d(u -> v), INFTY if no common hub."""
        return int(query(self, np.array([[u, v]], np.uint32))[0])

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.chl_labels_free(self._h)
            self._h = None


def build(g: Graph, order, mode: int = MODE_HYBRID, sf: float = 0.0, ps: float = 0.0,
          verbose: int = 0, max_warps: int = 0, autotune: int = 1,
          first_superstep: int = 0, growth: float = 0.0,
          use_graphs: Optional[int] = None, root_limit: int = 0,
          superstep_extend: int = 0, label_cap: int = 0, queue_split: int = 0,
          window_target: int = 0, window_warps: int = 0) -> Labeling:
    o = _u32(order)
    opts = BuildOpts()
    lib().chl_build_opts_default(C.byref(opts))
    opts.mode = mode
    opts.sf = sf
    opts.ps = ps
    opts.verbose = verbose
    opts.max_warps = max_warps
    opts.autotune = autotune
    opts.first_superstep = first_superstep
    opts.growth = growth
    if use_graphs is not None:
        opts.use_graphs = use_graphs
    opts.root_limit = root_limit
    opts.superstep_extend = superstep_extend
    opts.label_cap = label_cap
    opts.window_target = window_target
    opts.window_warps = window_warps
    opts.queue_split = queue_split
    h = C.c_void_p()
    _check(lib().chl_build(g._h, _ptr(o, _U32P), len(o), C.byref(opts), C.byref(h)), "build")
    return Labeling(h)


def run_paraPLL(g: Graph, order, sf: float = 32.0, verbose: int = 0) -> Labeling:
    """hl::run_paraPLL (shared_memory/akiba.hpp:132): GLL supersteps of sf*N labels."""
    return build(g, order, mode=MODE_GLL, sf=sf, verbose=verbose)


def run(g: Graph, order, phase_switch: float = 1024.0, sf: float = 32.0, verbose: int = 0) -> Labeling:
    """hl::run (distributed_memory/akiba.hpp:190): PLaNT trees, then GLL."""
    return build(g, order, mode=MODE_HYBRID, ps=phase_switch, sf=sf, verbose=verbose)


def query(labels: Labeling, pairs) -> np.ndarray:
    """batchLocalQuery: pairs is (k, 2) of (u, v); returns d(u -> v) int32."""
    p = _u32(np.asarray(pairs).reshape(-1, 2))
    out = np.zeros(len(p), np.int32)
    _check(lib().chl_query_batch(labels._h, _ptr(p, _U32P), len(p), _ptr(out, _I32P), None), "query")
    return out


def query_bench(labels: Labeling, k: int, iters: int = 10, seed: int = 1, hot: int = 0):
    """(ms per launch, algorithmic bytes per launch) of k device-resident pairs
    (uniform, or drawn from `hot` fixed pairs)."""
    ms = C.c_double()
    b = C.c_uint64()
    _check(lib().chl_query_bench(labels._h, k, seed, iters, hot, C.byref(ms), C.byref(b)), "query bench")
    return ms.value, b.value


def generate_query(k: int, n: int, seed: int = 1) -> np.ndarray:
    p = np.zeros((k, 2), np.uint32)
    _check(lib().chl_query_generate(_ptr(p, _U32P), k, n, seed), "generate_query")
    return p


def load_query(path: str) -> np.ndarray:
    p = _U32P()
    k = C.c_size_t()
    _check(lib().chl_query_load(os.fsencode(path), C.byref(p), C.byref(k)), f"read {path}")
    try:
        return np.ctypeslib.as_array(p, shape=(k.value, 2)).copy() if k.value else np.zeros((0, 2), np.uint32)
    finally:
        lib().chl_order_free(p)


class Server:
    """Continuous-batching query server over resident labels."""

    def __init__(self, labels: Labeling, max_inflight_pairs: int = 1 << 22, max_requests: int = 1 << 16,
                 max_batch_pairs: int = 1 << 20):
        o = ServerOpts()
        lib().chl_server_opts_default(C.byref(o))
        o.max_inflight_pairs = max_inflight_pairs
        o.max_requests = max_requests
        o.max_batch_pairs = max_batch_pairs
        self._labels = labels
        self._h = C.c_void_p()
        _check(lib().chl_server_create(labels._h, C.byref(o), C.byref(self._h)), "server create")

    def submit(self, pairs) -> int:
        p = _u32(np.asarray(pairs).reshape(-1, 2))
        rid = C.c_uint64()
        _check(lib().chl_server_submit(self._h, _ptr(p, _U32P), len(p), C.byref(rid)), "submit")
        self._last_k = len(p)
        return rid.value

    def wait(self, rid: int, k: int, timeout_ms: float = -1.0):
        out = np.zeros(k, np.int32)
        lat = C.c_double()
        _check(lib().chl_server_wait(self._h, rid, _ptr(out, _I32P), timeout_ms, C.byref(lat)), "wait")
        return out, lat.value

    def blocked(self) -> int:
        """Callers blocked in submit (admission) or wait."""
        x = C.c_uint32()
        _check(lib().chl_server_blocked(self._h, C.byref(x)), "server blocked")
        return x.value

    def stats(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().chl_server_stats(self._h, C.byref(a), C.byref(b), C.byref(c)), "stats")
        return {"launches": a.value, "pairs": b.value, "requests": c.value}

    def close(self):
        # the handle is dropped before it is freed: no method call starts on
        # a server that is being freed
        h, self._h = self._h, None
        if h:
            lib().chl_server_free(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RankNet:
    """Learned vertex ranking (message-passing network on the GPU).

    No reference counterpart: the reference reads its order from a file
    (shared_memory/hhl.cpp:36-37) made by outside tools (README.md:24).
    """

    HIDDEN = 64
    FEATURES = 3

    def __init__(self, layers: int = 3, seed: int = 1):
        self.layers = layers
        self._h = C.c_void_p()
        _check(lib().chl_gnn_create(layers, seed, C.byref(self._h)), "gnn create")

    def param_count(self) -> int:
        return int(lib().chl_gnn_param_count(self._h))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        _check(lib().chl_gnn_get_params(self._h, _ptr(p, _F32P)), "gnn get params")
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.param_count():
            raise ValueError("parameter vector has the wrong length")
        _check(lib().chl_gnn_set_params(self._h, _ptr(p, _F32P)), "gnn set params")

    @staticmethod
    def features(g: Graph, seed: int = 1) -> np.ndarray:
        x = np.zeros((g.get_n(), RankNet.FEATURES), np.float32)
        _check(lib().chl_gnn_features(g._h, seed, _ptr(x, _F32P)), "gnn features")
        return x

    def predict(self, g: Graph, seed: int = 1) -> np.ndarray:
        s = np.zeros(g.get_n(), np.float32)
        _check(lib().chl_gnn_predict(self._h, g._h, seed, _ptr(s, _F32P)), "gnn predict")
        return s

    def grad(self, g: Graph, target, seed: int = 1):
        t = np.ascontiguousarray(target, np.float32)
        if t.size != g.get_n():
            raise ValueError("target must have one value per vertex")
        loss = C.c_double()
        gr = np.zeros(self.param_count(), np.float32)
        _check(lib().chl_gnn_grad(self._h, g._h, seed, _ptr(t, _F32P), C.byref(loss), _ptr(gr, _F32P)), "gnn grad")
        return loss.value, gr

    def train_step(self, g: Graph, target, lr: float = 1e-3, seed: int = 1) -> float:
        t = np.ascontiguousarray(target, np.float32)
        if t.size != g.get_n():
            raise ValueError("target must have one value per vertex")
        loss = C.c_double()
        _check(lib().chl_gnn_train_step(self._h, g._h, seed, _ptr(t, _F32P), lr, C.byref(loss)), "gnn train")
        return loss.value

    def save(self, path: str) -> None:
        """Parameters as a .npy float32 vector (load with the same layer count)."""
        np.save(path, self.get_params())

    @classmethod
    def load(cls, path: str, layers: int = 3) -> "RankNet":
        p = np.load(path).astype(np.float32)
        net = cls(layers)
        net.set_params(p)
        return net

    @classmethod
    def pretrained(cls) -> "RankNet":
        """The 3-layer network trained on hub frequencies of 256 small GPU
        labelings (``bench.py --rank``), shipped with the package."""
        return cls.load(os.path.join(_HERE, "ranknet_l3.npy"), layers=3)

    def order(self, g: Graph, seed: int = 1) -> np.ndarray:
        o = np.zeros(g.get_n(), np.uint32)
        _check(lib().chl_gnn_order(self._h, g._h, seed, _ptr(o, _U32P)), "gnn order")
        return o

    def close(self):
        if self._h:
            lib().chl_gnn_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
