"""ctypes wrapper of the oracle (oracle/scan_oracle.c) and of the reference-kernel harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke(), bench.py's
CPU-baseline leg and bench.py's CPU reference arm, as the checker or the CPU baseline.  The
product package never imports this module.
"""
from __future__ import annotations

import ctypes as C
from fractions import Fraction
from pathlib import Path

import numpy as np

from . import build as _build

_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)

_lib = None
_harness = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(str(path))
        L.oracle_orient.restype = C.c_int64
        L.oracle_orient.argtypes = [C.c_uint64, _u64p, _u32p, _u32p, _u32p]
        L.oracle_eid.restype = C.c_int
        L.oracle_eid.argtypes = [C.c_uint64, _u64p, _u32p, _u32p]
        L.oracle_common_neighbors.restype = None
        L.oracle_common_neighbors.argtypes = [_u64p, _u32p, C.c_uint64, _u32p, _u32p, _u32p]
        L.oracle_ref_f64_similar.restype = C.c_int
        L.oracle_ref_f64_similar.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_double]
        L.oracle_exact_similar.restype = C.c_int
        L.oracle_exact_similar.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64]
        L.oracle_scan.restype = C.c_int
        L.oracle_scan.argtypes = [C.c_uint64, _u64p, _u32p, C.c_int, C.c_double, C.c_uint64, C.c_uint64, C.c_int,
                                  _i32p, _u8p, _u32p, _u64p]
        L.oracle_scan_ex.restype = C.c_int
        L.oracle_scan_ex.argtypes = [C.c_uint64, _u64p, _u32p, C.c_int, C.c_double, C.c_uint64, C.c_uint64, C.c_int,
                                     C.c_uint, _u32p, _i32p, _u8p, _u32p, _u64p]
        L.oracle_check_admissible_ex.restype = C.c_int
        L.oracle_check_admissible_ex.argtypes = [C.c_uint64, _u64p, _u32p, C.c_int, C.c_double, C.c_uint64,
                                                 C.c_uint64, C.c_int, _u32p, _i32p, _u64p]
        L.oracle_rmat_pairs.restype = None
        L.oracle_rmat_pairs.argtypes = [C.c_int, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_uint64, _u64p]
        L.oracle_csr_from_pairs.restype = C.c_int64
        L.oracle_csr_from_pairs.argtypes = [C.c_uint64, _u64p, C.c_uint64, _u64p, _u32p]
        L.oracle_count_stripe.restype = None
        L.oracle_count_stripe.argtypes = [_u64p, _u32p, C.c_uint64, _u32p, _u32p, C.c_uint64, C.c_uint64, C.c_double,
                                          C.c_uint64, C.c_uint64, C.c_uint, _u32p]
        L.oracle_memberships.restype = C.c_int64
        L.oracle_memberships.argtypes = [C.c_uint64, _u64p, _u32p, C.c_int, C.c_double, C.c_uint64, C.c_uint64,
                                         C.c_int, _i32p, _i32p, C.c_uint64]
        L.oracle_check_admissible.restype = C.c_int
        L.oracle_check_admissible.argtypes = [C.c_uint64, _u64p, _u32p, C.c_int, C.c_double, C.c_uint64, C.c_uint64,
                                              C.c_int, _i32p, _u64p]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def eps_params(eps: str) -> tuple[float, int, int]:
    """(double as atof reads it, p, q) for decimal text eps; p > q means eps > 1."""
    f = Fraction(eps.strip().lstrip("+-"))
    return float(eps), f.numerator, f.denominator


def _csr(off, adj):
    off = np.ascontiguousarray(off, dtype=np.uint64)
    adj = np.ascontiguousarray(adj, dtype=np.uint32)
    if adj.size == 0:
        adj = np.zeros(1, np.uint32)
    return off, adj


def orient(off, adj):
    off, adj = _csr(off, adj)
    n = off.size - 1
    E = int(off[-1]) // 2
    eu = np.zeros(max(E, 1), np.uint32)
    ev = np.zeros(max(E, 1), np.uint32)
    r = lib().oracle_orient(n, _p(off, C.c_uint64), _p(adj, C.c_uint32), _p(eu, C.c_uint32), _p(ev, C.c_uint32))
    if r < 0:
        raise ValueError("graph is not symmetric")
    return eu[:E], ev[:E]


def eid(off, adj):
    off, adj = _csr(off, adj)
    n = off.size - 1
    out = np.zeros(max(int(off[-1]), 1), np.uint32)
    if lib().oracle_eid(n, _p(off, C.c_uint64), _p(adj, C.c_uint32), _p(out, C.c_uint32)) < 0:
        raise ValueError("graph is not symmetric")
    return out[: int(off[-1])]


def common_neighbors(off, adj):
    """cn in the reference edge order."""
    off, adj = _csr(off, adj)
    eu, ev = orient(off, adj)
    cn = np.zeros(max(eu.size, 1), np.uint32)
    lib().oracle_common_neighbors(_p(off, C.c_uint64), _p(adj, C.c_uint32), eu.size, _p(eu, C.c_uint32),
                                  _p(ev, C.c_uint32), _p(cn, C.c_uint32))
    return cn[: eu.size]


COUNT_KEYS = ("cores", "clusters", "borders", "hubs", "outliers", "similar_edges", "disagreements", "multi_borders")


def scan(off, adj, eps: str, mu: int, mode: int):
    """(label, role, counts dict) of the oracle; mode 0 exact, 1 ref-f64."""
    off, adj = _csr(off, adj)
    n = off.size - 1
    e, p, q = eps_params(eps)
    label = np.zeros(n, np.int32)
    role = np.zeros(n, np.uint8)
    counts = np.zeros(8, np.uint64)
    if lib().oracle_scan(n, _p(off, C.c_uint64), _p(adj, C.c_uint32), mode, e, p, q, mu, _p(label, C.c_int32),
                         _p(role, C.c_uint8), None, _p(counts, C.c_uint64)) < 0:
        raise ValueError("oracle_scan failed")
    return label, role, dict(zip(COUNT_KEYS, map(int, counts)))


PRUNE = 1   # oracle_scan_ex flag: the reference's degree prune (GPUSCAN++/GPUScan.cu:145) before counting


def scan_ex(off, adj, eps: str, mu: int, mode: int, prune: bool = False, cn=None, want_cn: bool = False):
    """oracle_scan_ex: (label, role, counts dict[, cn used]).  prune skips the edges both
    predicates reject by degree alone (as the reference's __prep_edge does); cn (reference
    edge order) replaces the intersections, so one count serves several (eps, mu)."""
    off, adj = _csr(off, adj)
    n = off.size - 1
    e, p, q = eps_params(eps)
    E = int(off[-1]) // 2
    label = np.zeros(n, np.int32)
    role = np.zeros(n, np.uint8)
    counts = np.zeros(8, np.uint64)
    cn_in = None if cn is None else np.ascontiguousarray(cn, dtype=np.uint32)
    if cn_in is not None and cn_in.size != E:
        raise ValueError(f"cn has {cn_in.size} entries, the graph {E} edges")
    cn_out = np.zeros(max(E, 1), np.uint32) if want_cn else None
    if lib().oracle_scan_ex(n, _p(off, C.c_uint64), _p(adj, C.c_uint32), mode, e, p, q, mu, PRUNE if prune else 0,
                            None if cn_in is None or E == 0 else _p(cn_in, C.c_uint32), _p(label, C.c_int32),
                            _p(role, C.c_uint8), None if cn_out is None else _p(cn_out, C.c_uint32),
                            _p(counts, C.c_uint64)) < 0:
        raise ValueError("oracle_scan_ex failed")
    res = (label, role, dict(zip(COUNT_KEYS, map(int, counts))))
    return res + (cn_out[:E],) if want_cn else res


class StripedPass:
    """One oracle SCAN pass split into bounded steps: count(s, k) intersects the edges
    e = s, s + k, ... (reference edge order, degree prune on), finish() runs the predicate
    and the clustering on the collected counts.  Steps 0..k-1 of one k cover every edge."""

    def __init__(self, off, adj, eps: str, mode: int, prune: bool = True):
        self.off, self.adj = _csr(off, adj)
        self.eu, self.ev = orient(self.off, self.adj)
        self.E = self.eu.size
        self.eps, self.mode, self.flags = eps, mode, PRUNE if prune else 0
        self.e, self.p, self.q = eps_params(eps)
        self.cn = np.zeros(max(self.E, 1), np.uint32)

    def count(self, stripe: int, nstripes: int) -> None:
        lib().oracle_count_stripe(_p(self.off, C.c_uint64), _p(self.adj, C.c_uint32), self.E,
                                  _p(self.eu, C.c_uint32), _p(self.ev, C.c_uint32), stripe, nstripes, self.e, self.p,
                                  self.q, self.flags, _p(self.cn, C.c_uint32))

    def finish(self, mu: int):
        return scan_ex(self.off, self.adj, self.eps, mu, self.mode, cn=self.cn[: self.E])


def rmat(scale: int, edge_factor: int = 16, seed: int = 1, a: float = 0.57, b: float = 0.19, c: float = 0.19):
    """(offsets uint64[n+1], adjacency uint32[m]) of the seeded R-MAT graph, built on the
    CPU: the same graph as the engine's Graph.rmat (both pinned by the same checksums)."""
    n = 1 << scale
    k = edge_factor * n
    pairs = np.empty(k, np.uint64)
    lib().oracle_rmat_pairs(scale, k, a, b, c, seed, _p(pairs, C.c_uint64))
    off = np.empty(n + 1, np.uint64)
    adj = np.empty(max(2 * k, 1), np.uint32)
    m = lib().oracle_csr_from_pairs(n, _p(pairs, C.c_uint64), k, _p(off, C.c_uint64), _p(adj, C.c_uint32))
    if m < 0:
        raise MemoryError("oracle_csr_from_pairs: allocation failed")
    del pairs
    return off, adj[:m].copy()


def memberships(off, adj, eps: str, mu: int, mode: int):
    off, adj = _csr(off, adj)
    n = off.size - 1
    e, p, q = eps_params(eps)
    k = lib().oracle_memberships(n, _p(off, C.c_uint64), _p(adj, C.c_uint32), mode, e, p, q, mu, None, None, 0)
    cl = np.zeros(max(k, 1), np.int32)
    vx = np.zeros(max(k, 1), np.int32)
    lib().oracle_memberships(n, _p(off, C.c_uint64), _p(adj, C.c_uint32), mode, e, p, q, mu, _p(cl, C.c_int32),
                             _p(vx, C.c_int32), k)
    return cl[:k], vx[:k]


def check_admissible(off, adj, eps: str, mu: int, mode: int, cand, cn=None) -> dict:
    """Violations of a reference-style label array against the oracle (see
    oracle_check_admissible_ex); cn (reference edge order) replaces the intersections."""
    off, adj = _csr(off, adj)
    n = off.size - 1
    e, p, q = eps_params(eps)
    c = np.ascontiguousarray(cand, dtype=np.int32)
    viol = np.zeros(4, np.uint64)
    cn_in = None if cn is None else np.ascontiguousarray(cn, dtype=np.uint32)
    if lib().oracle_check_admissible_ex(n, _p(off, C.c_uint64), _p(adj, C.c_uint32), mode, e, p, q, mu,
                                        None if cn_in is None or cn_in.size == 0 else _p(cn_in, C.c_uint32),
                                        _p(c, C.c_int32), _p(viol, C.c_uint64)) < 0:
        raise ValueError("oracle_check_admissible failed")
    return dict(zip(("core", "border", "membership", "hub_rule"), map(int, viol)))


# ---- the reference's own code -----------------------------------------------------------
def reference_orientation_available() -> bool:
    return _build.REF_GRAPH_LIB.exists()


def reference_orient(off, adj):
    """(eid, edge_u, edge_v) from the reference's getEidAndEdgeList (GPUSCAN++/Graph.cpp:52)."""
    L = C.CDLL(str(_build.REF_GRAPH_LIB))
    f = L.ref_get_eid_and_edge_list
    f.restype = None
    f.argtypes = [C.c_long, C.c_long, _i32p, _u32p, _u32p, _i32p, _i32p]
    off32 = np.ascontiguousarray(off, dtype=np.uint32)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    n = off32.size - 1
    m = int(off32[-1])
    a = np.concatenate([a, np.zeros(16, np.int32)])   # the reference allocates m + 16 entries
    e = np.zeros(max(m, 1), np.uint32)
    eu = np.zeros(max(m // 2, 1), np.int32)
    ev = np.zeros(max(m // 2, 1), np.int32)
    f(n, m, _p(a, C.c_int32), _p(off32, C.c_uint32), _p(e, C.c_uint32), _p(eu, C.c_int32), _p(ev, C.c_int32))
    return e[:m], eu[: m // 2], ev[: m // 2]


def reference_kernels_available() -> bool:
    return _build.REF_CUBIN.exists()


def reference_gpuscan_prepare(off, adj):
    """The host inputs GPUScan() takes (GPUSCAN++/main.cpp:52-56): uint32 offsets, int32
    adjacency, eid and the oriented edge list, computed once so repeated calls can be timed."""
    off64, adj32 = _csr(off, adj)
    eu, ev = orient(off64, adj32)
    return {"off32": off64.astype(np.uint32), "adj": adj32.astype(np.int32), "eid": eid(off64, adj32),
            "eu": eu.astype(np.int32), "ev": ev.astype(np.int32), "n": off64.size - 1, "m": int(off64[-1])}


def reference_gpuscan(off, adj, eps: float, mu: int, prepared=None):
    """Run the reference's kernels (its cubin) on device 0; returns (role array, kernel ms)."""
    global _harness
    if _harness is None:
        L = C.CDLL(str(_build.build_harness()))
        L.ref_gpuscan.restype = C.c_int
        L.ref_gpuscan.argtypes = [C.c_char_p, C.c_int64, C.c_int64, _u32p, _i32p, _u32p, _i32p, _i32p, C.c_double,
                                  C.c_int, _i32p, C.POINTER(C.c_float)]
        L.ref_harness_error.restype = C.c_char_p
        _harness = L
    p = prepared if prepared is not None else reference_gpuscan_prepare(off, adj)
    n, m = p["n"], p["m"]
    out = np.zeros(n, np.int32)
    ms = C.c_float(0)
    if _harness.ref_gpuscan(str(_build.REF_CUBIN).encode(), n, m, _p(p["off32"], C.c_uint32), _p(p["adj"], C.c_int32),
                            _p(p["eid"], C.c_uint32), _p(p["eu"], C.c_int32), _p(p["ev"], C.c_int32),
                            float(eps), int(mu), _p(out, C.c_int32), C.byref(ms)) != 0:
        raise RuntimeError("reference harness: " + _harness.ref_harness_error().decode())
    return out, ms.value
