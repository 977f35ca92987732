"""GB300-native SCAN structural graph clustering (the GPUSCAN++ hot path, rebuilt).

Python mirror of the C-ABI in include/scan_gb300.h, over ctypes.  The compute path is the
CUDA library libscan_gb300.so; this module only marshals numpy arrays.  If the library is
missing, importing succeeds but every call raises (there is no CPU fallback).

Reference surface mirrored (GPUSCAN++):
  Graph(dir)                      -> Graph.load(dir)               (Graph.cpp:147-223)
  CheckInputGraph                 -> Graph.validate()              (Graph.cpp:270-288)
  getEidAndEdgeList(g, Eu, Ev)    -> Graph.orient_reference()      (Graph.cpp:52-141)
  GPUScan(g, Eu, Ev, eps, miu)    -> GPUScan(...) / Graph.run(...) (GPUScan.h:7, GPUScan.cu:800-1009)
  main's "Cluster Number"         -> count_clusters(label)         (main.cpp:83-111)
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass
from pathlib import Path

import numpy as np

__all__ = [
    "ScanError", "Graph", "ScanStats", "GPUScan", "count_clusters", "library_path", "load_library",
    "cores_noalloc", "Server", "Batch", "convert_edge_list", "PRED_EXACT", "PRED_REF_F64", "SMALL_SERIAL", "SMALL_BATCHED", "SMALL_SEARCH", "ROLE_OUTLIER", "ROLE_HUB", "ROLE_BORDER", "ROLE_CORE", "EXPORTED_SYMBOLS",
]

PRED_EXACT = 0
PRED_REF_F64 = 1
# small-pivot intersection strategies of the similarity plan
SMALL_SERIAL, SMALL_BATCHED, SMALL_SEARCH = 0, 1, 2
ROLE_OUTLIER, ROLE_HUB, ROLE_BORDER, ROLE_CORE = 0, 1, 2, 3

_PKG = Path(__file__).resolve().parent
_LIB_PATH = _PKG / "_build" / "libscan_gb300.so"

STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "i/o error", 3: "bad graph format", 4: "cuda error",
                5: "out of memory", 6: "graph too large", 7: "device-side check failed"}


class ScanError(RuntimeError):
    """A C-ABI call returned a non-zero scan_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class ScanStats(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in (
        "n", "num_edges", "num_cores", "num_clusters", "num_hubs", "num_outliers", "num_borders",
        "num_similar_edges", "pred_disagreements", "multi_cluster_borders")] + [
        (name, C.c_double) for name in ("ms_h2d", "ms_orient", "ms_similarity", "ms_cluster", "ms_d2h", "ms_total")] + [
        ("ms_cn_kernel", C.c_double * 5), ("cn_work_items", C.c_uint64 * 5),
        ("kernel_launches", C.c_uint32), ("reserved", C.c_uint32), ("cn_words", C.c_uint64),
        ("cn_edges_counted", C.c_uint64)]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            if name == "reserved":
                continue
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, C.Array) else v
        return out


class QueryResult(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int32), ("graph_id", C.c_uint32), ("queue_ms", C.c_double),
                ("latency_ms", C.c_double), ("device_ms", C.c_double), ("num_cores", C.c_uint64),
                ("num_clusters", C.c_uint64), ("num_similar_edges", C.c_uint64)]


class BatchStats(C.Structure):
    _fields_ = [("ms_device", C.c_double), ("ms_total", C.c_double)] + [
        (name, C.c_uint64) for name in ("num_graphs", "num_vertices", "num_edges", "num_cores", "num_clusters")] + [
        ("graph_kernels", C.c_uint32), ("long_words", C.c_uint32), ("target_probes", C.c_uint64),
        ("tuned_similarity_ms", C.c_double), ("small_deg", C.c_uint32), ("small_strategy", C.c_uint32),
        ("hub_min_deg", C.c_uint32), ("chunk_max", C.c_uint32)]


class ServerCounters(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in ("submitted", "admitted", "completed", "failed", "pending",
                                                "in_flight", "graphs", "budget_bytes", "kernel_launches")]


_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)
_vp = C.c_void_p

# name -> (restype, argtypes); every symbol declared in include/scan_gb300.h
_SIGS = {
    "scan_last_error": (C.c_char_p, []),
    "scan_status_string": (C.c_char_p, [C.c_int]),
    "scan_version": (C.c_char_p, []),
    "scan_graph_load": (C.c_int, [C.c_char_p, C.POINTER(_vp)]),
    "scan_graph_save": (C.c_int, [_vp, C.c_char_p]),
    "scan_graph_from_csr": (C.c_int, [_u64p, _u32p, C.c_uint64, C.c_uint64, C.POINTER(_vp)]),
    "scan_graph_from_csr32": (C.c_int, [_u32p, _u32p, C.c_uint64, C.c_uint64, C.POINTER(_vp)]),
    "scan_graph_free": (None, [_vp]),
    "scan_graph_num_vertices": (C.c_uint64, [_vp]),
    "scan_graph_num_directed": (C.c_uint64, [_vp]),
    "scan_graph_max_degree": (C.c_uint32, [_vp]),
    "scan_graph_offsets": (_u64p, [_vp]),
    "scan_graph_adjacency": (_u32p, [_vp]),
    "scan_graph_validate": (C.c_int, [_vp, C.c_int]),
    "scan_graph_upload": (C.c_int, [_vp, C.c_int]),
    "scan_graph_release_device": (C.c_int, [_vp]),
    "scan_graph_upload_streamed": (C.c_int, [_vp, C.c_int, C.c_uint64, _u64p]),
    "scan_graph_device_bytes": (C.c_uint64, [_vp]),
    "scan_release_cached_memory": (None, []),
    "scan_set_cached_memory_limit": (None, [C.c_uint64]),
    "scan_cached_memory_bytes": (C.c_uint64, [C.c_int]),
    "scan_set_loop_limits": (None, [C.c_int64, C.c_int32]),
    "scan_gen_rmat": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64, C.POINTER(_vp)]),
    "scan_gen_chung_lu": (C.c_int, [C.c_uint64, C.c_double, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(_vp)]),
    "scan_gen_sbm": (C.c_int, [C.c_uint64, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                               C.POINTER(_vp)]),
    "scan_orient_reference": (C.c_int, [_vp, _u32p, _i32p, _i32p]),
    "scan_run": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_int, C.c_int, _i32p, _u8p, C.POINTER(ScanStats)]),
    "scan_common_neighbors": (C.c_int, [_vp, C.c_int, _u32p, C.POINTER(ScanStats)]),
    "scan_memberships": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_int, C.c_int, _i32p, _i32p, C.c_uint64,
                                   C.POINTER(C.c_uint64)]),
    "scan_gpuscan_compat": (_i32p, [C.c_int64, C.c_int64, _i32p, _u32p, _u32p, _i32p, _i32p, C.c_double, C.c_int]),
    "scan_count_clusters": (C.c_uint64, [_i32p, C.c_uint64]),
    "scan_convert_edge_list": (C.c_int, [C.c_char_p, C.c_char_p, _u64p, _u64p]),
    "scan_eps_to_decimal": (C.c_int, [C.c_double, C.c_char_p, C.c_size_t]),
    "scan_graph_autotune": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_uint32), _u64p]),
    "scan_graph_plan": (C.c_int, [_vp, _u32p, _u32p, _u32p, _u32p]),
    "scan_graph_set_plan": (C.c_int, [_vp, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
    "scan_cores_noalloc": (C.c_int, [_vp, C.c_uint32, _vp, _vp, _vp, C.c_uint64, C.c_char_p, C.c_int, C.c_int, _vp,
                                     _vp]),
    "scan_batch_create": (C.c_int, [C.POINTER(_vp), C.c_uint32, C.c_int, C.c_int, C.POINTER(_vp)]),
    "scan_batch_run": (C.c_int, [_vp, C.POINTER(C.c_char_p), _i32p, C.c_int, C.POINTER(_i32p), C.POINTER(_u8p),
                                 C.POINTER(BatchStats)]),
    "scan_batch_free": (None, [_vp]),
    "scan_server_create": (C.c_int, [C.c_int, C.c_uint64, C.c_uint32, C.POINTER(_vp)]),
    "scan_server_add_graph": (C.c_int, [_vp, _vp, C.POINTER(C.c_uint32)]),
    "scan_server_submit": (C.c_int, [_vp, C.c_uint32, C.c_char_p, C.c_int, C.c_int, _i32p, _u8p,
                                     C.POINTER(C.c_uint64)]),
    "scan_server_wait": (C.c_int, [_vp, C.c_uint64, C.POINTER(QueryResult)]),
    "scan_server_poll": (C.c_int, [_vp, C.c_uint64, C.POINTER(C.c_int)]),
    "scan_server_get_counters": (C.c_int, [_vp, C.POINTER(ServerCounters)]),
    "scan_server_replay": (C.c_int, [_vp, C.c_uint64, _u32p, C.POINTER(C.c_char_p), _i32p, _i32p,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), _i32p, C.POINTER(C.c_double)]),
    "scan_server_destroy": (None, [_vp]),
}
EXPORTED_SYMBOLS = tuple(_SIGS)

_lib = None


def library_path() -> Path:
    return _LIB_PATH


def load_library() -> C.CDLL:
    """Load libscan_gb300.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise ScanError(4, f"{_LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(_LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


_libc = None


def _libc_free(addr: int) -> None:
    """free() of a result the library malloc'd (the drop-in GPUScan's int32[n])."""
    global _libc
    if _libc is None:
        _libc = C.CDLL(None)
        _libc.free.argtypes = [C.c_void_p]
        _libc.free.restype = None
    _libc.free(addr)


def _check(status: int) -> None:
    if status != 0:
        raise ScanError(status, load_library().scan_last_error().decode())


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def _eps_text(eps) -> bytes:
    if isinstance(eps, (bytes, str)):
        return eps.encode() if isinstance(eps, str) else eps
    buf = C.create_string_buffer(48)
    _check(load_library().scan_eps_to_decimal(float(eps), buf, 48))
    return buf.value


@dataclass
class ScanResult:
    label: np.ndarray   # int32[n]: cluster id (smallest core id) / -1 hub / -2 outlier
    role: np.ndarray    # uint8[n]: 0 outlier, 1 hub, 2 border, 3 core
    stats: dict


class Graph:
    """A CSR graph owned by the library (host copy, plus a device copy once uploaded)."""

    def __init__(self, handle: int):
        self._h = _vp(handle)

    # -- construction ---------------------------------------------------------------------
    @classmethod
    def load(cls, folder: str | os.PathLike) -> "Graph":
        h = _vp()
        _check(load_library().scan_graph_load(str(folder).encode(), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_csr(cls, offsets: np.ndarray, adj: np.ndarray) -> "Graph":
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        a = np.ascontiguousarray(adj, dtype=np.uint32)
        if a.size == 0:
            a = np.zeros(1, dtype=np.uint32)
        h = _vp()
        _check(load_library().scan_graph_from_csr(_ptr(off, C.c_uint64), _ptr(a, C.c_uint32), off.size - 1,
                                                  int(off[-1]), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_edges(cls, n: int, edges) -> "Graph":
        """Undirected edge pairs -> symmetric, deduplicated, sorted CSR (self-loops dropped)."""
        e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
        e = e[e[:, 0] != e[:, 1]]
        both = np.concatenate([e, e[:, ::-1]]) if e.size else np.zeros((0, 2), np.int64)
        both = np.unique(both, axis=0)
        off = np.zeros(n + 1, dtype=np.uint64)
        if both.size:
            np.add.at(off, both[:, 0] + 1, 1)
        off = np.cumsum(off, dtype=np.uint64)
        return cls.from_csr(off, both[:, 1].astype(np.uint32) if both.size else np.zeros(0, np.uint32))

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1) -> "Graph":
        h = _vp()
        _check(load_library().scan_gen_rmat(scale, edge_factor, a, b, c, seed, C.byref(h)))
        return cls(h.value)

    @classmethod
    def chung_lu(cls, n: int, exponent: float, target_edges: int, max_degree: int, seed: int = 1) -> "Graph":
        h = _vp()
        _check(load_library().scan_gen_chung_lu(n, exponent, target_edges, max_degree, seed, C.byref(h)))
        return cls(h.value)

    @classmethod
    def sbm(cls, n: int, blocks: int, p_in: float, p_out: float, max_avg_degree: float = 64.0,
            seed: int = 1) -> "Graph":
        h = _vp()
        _check(load_library().scan_gen_sbm(n, blocks, p_in, p_out, max_avg_degree, seed, C.byref(h)))
        return cls(h.value)

    def close(self) -> None:
        if self._h:
            load_library().scan_graph_free(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- properties -----------------------------------------------------------------------
    @property
    def n(self) -> int:
        return load_library().scan_graph_num_vertices(self._h)

    @property
    def m(self) -> int:
        return load_library().scan_graph_num_directed(self._h)

    @property
    def num_edges(self) -> int:
        return self.m // 2

    @property
    def max_degree(self) -> int:
        return load_library().scan_graph_max_degree(self._h)

    def offsets(self) -> np.ndarray:
        p = load_library().scan_graph_offsets(self._h)
        return np.ctypeslib.as_array(p, shape=(self.n + 1,)).copy()

    def adjacency(self) -> np.ndarray:
        if self.m == 0:
            return np.zeros(0, np.uint32)
        p = load_library().scan_graph_adjacency(self._h)
        return np.ctypeslib.as_array(p, shape=(self.m,)).copy()

    def degrees(self) -> np.ndarray:
        return np.diff(self.offsets()).astype(np.int64)

    # -- host operations ------------------------------------------------------------------
    def save(self, folder: str | os.PathLike) -> None:
        Path(folder).mkdir(parents=True, exist_ok=True)
        _check(load_library().scan_graph_save(self._h, str(folder).encode()))

    def validate(self, check_symmetry: bool = True) -> None:
        _check(load_library().scan_graph_validate(self._h, int(check_symmetry)))

    def orient_reference(self):
        """(eid[m], edge_u[E], edge_v[E]) exactly as getEidAndEdgeList builds them."""
        eid = np.zeros(max(self.m, 1), np.uint32)
        eu = np.zeros(max(self.num_edges, 1), np.int32)
        ev = np.zeros(max(self.num_edges, 1), np.int32)
        _check(load_library().scan_orient_reference(self._h, _ptr(eid, C.c_uint32), _ptr(eu, C.c_int32),
                                                    _ptr(ev, C.c_int32)))
        return eid[: self.m], eu[: self.num_edges], ev[: self.num_edges]

    # -- device operations ----------------------------------------------------------------
    def upload(self, device: int = 0) -> None:
        _check(load_library().scan_graph_upload(self._h, device))

    def upload_streamed(self, device: int = 0, device_budget_bytes: int = 0) -> int:
        """Keep the adjacency in pinned host memory read over the host link; the rest on the
        device under device_budget_bytes (0: no cap).  Returns device bytes used."""
        used = C.c_uint64(0)
        _check(load_library().scan_graph_upload_streamed(self._h, device, device_budget_bytes, C.byref(used)))
        return used.value

    @property
    def device_bytes(self) -> int:
        return load_library().scan_graph_device_bytes(self._h)

    def release_device(self) -> None:
        _check(load_library().scan_graph_release_device(self._h))

    def run(self, eps, mu: int, predicate: int = PRED_EXACT, device: int = 0) -> ScanResult:
        """SCAN(eps, mu) on the GPU; eps as decimal text (or a float, printed shortest)."""
        label = np.empty(self.n, np.int32)
        role = np.empty(self.n, np.uint8)
        st = ScanStats()
        _check(load_library().scan_run(self._h, device, _eps_text(eps), int(mu), int(predicate),
                                       _ptr(label, C.c_int32), _ptr(role, C.c_uint8), C.byref(st)))
        return ScanResult(label, role, st.as_dict())

    def autotune(self, device: int = 0) -> dict:
        """Tune the similarity stage's plan for later runs; returns the chosen plan."""
        ms, lw, tp = C.c_double(0), C.c_uint32(0), C.c_uint64(0)
        _check(load_library().scan_graph_autotune(self._h, device, C.byref(ms), C.byref(lw), C.byref(tp)))
        return dict(self.plan(), similarity_ms=ms.value, long_words=lw.value, target_probes=tp.value)

    def set_plan(self, small_deg: int = 128, small_strategy: int = SMALL_SERIAL, hub_min_deg: int = 6144,
                 chunk_max: int = 6144, device: int = 0) -> None:
        """Pin the similarity plan (uploads the graph first); every plan gives the same results.
        small_strategy: SMALL_SERIAL, SMALL_BATCHED or SMALL_SEARCH."""
        _check(load_library().scan_graph_set_plan(self._h, device, small_deg, int(small_strategy), hub_min_deg,
                                                  chunk_max))

    def plan(self) -> dict:
        """The resident copy's similarity plan (small-pivot cut and strategy, hub threshold, chunk)."""
        v = [C.c_uint32(0) for _ in range(4)]
        _check(load_library().scan_graph_plan(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("small_deg", "small_strategy", "hub_min_deg", "chunk_max"), (x.value for x in v)))

    def common_neighbors(self, device: int = 0):
        """cn[E] in the reference edge order, plus stats."""
        cn = np.empty(max(self.num_edges, 1), np.uint32)
        st = ScanStats()
        _check(load_library().scan_common_neighbors(self._h, device, _ptr(cn, C.c_uint32), C.byref(st)))
        return cn[: self.num_edges], st.as_dict()

    def memberships(self, eps, mu: int, predicate: int = PRED_EXACT, device: int = 0):
        """Sorted (cluster, vertex) pairs: cores once, borders once per cluster."""
        lib = load_library()
        cnt = C.c_uint64(0)
        status = lib.scan_memberships(self._h, device, _eps_text(eps), int(mu), int(predicate), None, None, 0,
                                      C.byref(cnt))
        if status not in (0, 1):
            _check(status)
        k = int(cnt.value)
        cl = np.empty(max(k, 1), np.int32)
        vx = np.empty(max(k, 1), np.int32)
        _check(lib.scan_memberships(self._h, device, _eps_text(eps), int(mu), int(predicate), _ptr(cl, C.c_int32),
                                    _ptr(vx, C.c_int32), k, C.byref(cnt)))
        return cl[:k], vx[:k]


def GPUScan(num_edges: np.ndarray, adj: np.ndarray, eps: float, miu: int, eid=None, Edge_u=None,
            Edge_v=None) -> np.ndarray:
    """The reference's GPUScan(graph_t*, Edge_u, Edge_v, eps, miu) on host arrays.

    num_edges: uint32[n+1] offsets, adj: int32[m].  Returns int32[n] in the reference's
    encoding.  eid/Edge_u/Edge_v are accepted for signature parity and not read.
    """
    lib = load_library()
    off = np.ascontiguousarray(num_edges, dtype=np.uint32)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    if a.size == 0:
        a = np.zeros(1, np.int32)
    n = off.size - 1
    p = lib.scan_gpuscan_compat(n, int(off[-1]), _ptr(a, C.c_int32), _ptr(off, C.c_uint32), None, None, None,
                                float(eps), int(miu))
    if not p:
        raise ScanError(4, lib.scan_last_error().decode())
    # The array views the library's malloc'd result and frees it when collected (no copy).
    out = np.ctypeslib.as_array(p, shape=(n,))
    weakref.finalize(out, _libc_free, C.cast(p, C.c_void_p).value)
    return out


def cores_noalloc(d_offsets: int, n: int, d_edge_u: int, d_edge_v: int, d_cn: int, num_edges: int, eps,
                  mu: int, predicate: int, d_is_core: int, stream: int = 0) -> None:
    """Core flags into caller-owned device memory, allocating nothing (scan_cores_noalloc).

    Every buffer argument is a device address (an int, e.g. a tensor's data_ptr()); the
    work is queued on `stream` and this returns before it completes.  For callers that
    may not allocate device memory themselves; limited to 2^20 vertices.
    """
    _check(load_library().scan_cores_noalloc(d_offsets, n, d_edge_u, d_edge_v, d_cn, num_edges, _eps_text(eps),
                                             int(mu), int(predicate), d_is_core, stream or None))


class Batch:
    """Many graphs with their own (eps, mu), one pass: a disjoint union on the device whose
    similarity and cluster stages run as one captured CUDA graph (scan_batch_*)."""

    def __init__(self, graphs, device: int = 0, autotune: bool = True):
        self._graphs = list(graphs)   # keep the handles alive
        arr = (_vp * len(self._graphs))(*[g._h.value for g in self._graphs])
        h = _vp()
        _check(load_library().scan_batch_create(arr, len(self._graphs), device, int(autotune), C.byref(h)))
        self._h = h

    def run(self, eps, mus, predicate: int = PRED_EXACT):
        """Per-graph (labels, roles) lists and the batch stats dict."""
        k = len(self._graphs)
        texts = (C.c_char_p * k)(*[_eps_text(e) for e in eps])
        mu = np.ascontiguousarray(mus, np.int32)
        labels = [np.empty(g.n, np.int32) for g in self._graphs]
        roles = [np.empty(g.n, np.uint8) for g in self._graphs]
        lp = (_i32p * k)(*[_ptr(x, C.c_int32) for x in labels])
        rp = (_u8p * k)(*[_ptr(x, C.c_uint8) for x in roles])
        st = BatchStats()
        _check(load_library().scan_batch_run(self._h, texts, _ptr(mu, C.c_int32), int(predicate), lp, rp,
                                             C.byref(st)))
        return labels, roles, {name: getattr(st, name) for name, _ in st._fields_}

    def close(self):
        if self._h:
            load_library().scan_batch_free(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """Serving loop over resident graphs with cached common-neighbour counts (scan_server_*).

    Queries run only the cluster stage; they are admitted in arrival order as stream slots
    and the memory budget allow, and run concurrently on the device.
    """

    def __init__(self, device: int = 0, memory_budget_bytes: int = 1 << 30, max_in_flight: int = 8):
        h = _vp()
        _check(load_library().scan_server_create(device, memory_budget_bytes, max_in_flight, C.byref(h)))
        self._h = h
        self._n = {}        # graph id -> vertex count (ids come from the library: add_graph may race)
        self._keep = {}

    def add_graph(self, g: "Graph") -> int:
        gid = C.c_uint32(0)
        _check(load_library().scan_server_add_graph(self._h, g._h, C.byref(gid)))
        self._n[gid.value] = g.n
        return gid.value

    def submit(self, graph_id: int, eps, mu: int, predicate: int = PRED_EXACT):
        """Queue a query; returns its ticket.  Results land in buffers kept until wait()."""
        n = self._n[graph_id]
        label = np.empty(n, np.int32)
        role = np.empty(n, np.uint8)
        t = C.c_uint64(0)
        _check(load_library().scan_server_submit(self._h, graph_id, _eps_text(eps), int(mu), int(predicate),
                                                 _ptr(label, C.c_int32), _ptr(role, C.c_uint8), C.byref(t)))
        self._keep[t.value] = (label, role)
        return t.value

    def wait(self, ticket: int):
        """(label, role, result dict) of a ticket; raises ScanError if the query failed."""
        r = QueryResult()
        status = load_library().scan_server_wait(self._h, ticket, C.byref(r))
        label, role = self._keep.pop(ticket)
        _check(status)
        return label, role, {name: getattr(r, name) for name, _ in r._fields_}

    def poll(self, ticket: int) -> bool:
        d = C.c_int(0)
        _check(load_library().scan_server_poll(self._h, ticket, C.byref(d)))
        return bool(d.value)

    def counters(self) -> dict:
        c = ServerCounters()
        _check(load_library().scan_server_get_counters(self._h, C.byref(c)))
        return {name: getattr(c, name) for name, _ in c._fields_}

    def replay(self, graph_ids, eps, mus, predicates, arrival_ms):
        """Submit query i at arrival_ms[i] (native timing); returns (latency_ms, status, wall_ms)."""
        k = len(graph_ids)
        gid = np.ascontiguousarray(graph_ids, np.uint32)
        mu = np.ascontiguousarray(mus, np.int32)
        pr = np.ascontiguousarray(predicates, np.int32)
        arr = np.ascontiguousarray(arrival_ms, np.float64)
        texts = [_eps_text(e) for e in eps]
        ptrs = (C.c_char_p * max(k, 1))(*texts)
        lat = np.zeros(max(k, 1), np.float64)
        st = np.zeros(max(k, 1), np.int32)
        wall = C.c_double(0)
        _check(load_library().scan_server_replay(self._h, k, _ptr(gid, C.c_uint32), ptrs, _ptr(mu, C.c_int32),
                                                 _ptr(pr, C.c_int32), _ptr(arr, C.c_double), _ptr(lat, C.c_double),
                                                 _ptr(st, C.c_int32), C.byref(wall)))
        return lat[:k], st[:k], wall.value

    def close(self):
        if self._h:
            load_library().scan_server_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def convert_edge_list(edge_list_path, out_dir) -> tuple[int, int]:
    """Edge-list text -> b_degree.bin / b_adj.bin (csr_convert's format); returns (n, E)."""
    Path(out_dir).mkdir(parents=True, exist_ok=True)
    n, e = C.c_uint64(0), C.c_uint64(0)
    _check(load_library().scan_convert_edge_list(str(edge_list_path).encode(), str(out_dir).encode(), C.byref(n),
                                                 C.byref(e)))
    return n.value, e.value


def count_clusters(label: np.ndarray) -> int:
    lab = np.ascontiguousarray(label, dtype=np.int32)
    return int(load_library().scan_count_clusters(_ptr(lab, C.c_int32), lab.size))


def release_cached_memory() -> None:
    """Return every cached device buffer (of freed graphs and drop-in calls) to the driver."""
    load_library().scan_release_cached_memory()


def set_cached_memory_limit(nbytes: int) -> None:
    """Cap the per-device cache of freed device buffers (0 disables it; default 8 GiB)."""
    load_library().scan_set_cached_memory_limit(int(nbytes))


def cached_memory_bytes(device: int = 0) -> int:
    return int(load_library().scan_cached_memory_bytes(device))


def set_loop_limits(union_find_iterations: int = -1, jump_rounds_cap: int = -1) -> None:
    """Testing: shrink the bounded device loops' limits (negative restores the default)."""
    load_library().scan_set_loop_limits(int(union_find_iterations), int(jump_rounds_cap))
