"""CPU tests: the C-ABI library loads and exports its header, host logic (formats, checks,
generators, reference orientation) and the oracle's pins.  No GPU is touched here."""
import ctypes
import json
import re
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

ROOT = Path(__file__).resolve().parent.parent


def header_functions(path: Path) -> set[str]:
    text = path.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(scan_[a-z0-9_]+)\s*\(", text))


def test_library_exports_every_declared_symbol():
    lib = sg.load_library()
    declared = header_functions(ROOT / "include" / "scan_gb300.h")
    assert declared, "no declarations parsed"
    assert declared == set(sg.EXPORTED_SYMBOLS), declared ^ set(sg.EXPORTED_SYMBOLS)
    for name in declared:
        assert hasattr(lib, name), name
    # the C++-linkage drop-in of GPUSCAN++/GPUScan.h:7 (include/gpuscan_compat.h)
    assert hasattr(lib, "_Z7GPUScanP7graph_tPiS1_di")


def test_version_and_status_strings():
    lib = sg.load_library()
    assert lib.scan_version().decode().count(".") == 2
    assert lib.scan_status_string(3).decode() == "bad graph format"


# ---- formats and input checks --------------------------------------------------------------
def write_bin(folder: Path, deg, adj, int_size=4, n=None, m=None):
    folder.mkdir(parents=True, exist_ok=True)
    deg = np.asarray(deg, np.int64)
    n = len(deg) if n is None else n
    m = int(deg.sum()) if m is None else m
    with open(folder / "b_degree.bin", "wb") as f:
        if int_size == 4:
            np.array([4, n, m], np.uint32).tofile(f)
            deg.astype(np.int32).tofile(f)
        else:
            np.array([8], np.int32).tofile(f)
            np.array([n, m], np.uint64).tofile(f)
            deg.astype(np.int64).tofile(f)
    np.asarray(adj, np.uint32).tofile(folder / "b_adj.bin")


def test_save_load_roundtrip(tmp_path):
    g = sg.Graph.rmat(10, 8, seed=3)
    g.save(tmp_path / "g")
    h = sg.Graph.load(tmp_path / "g")
    assert h.n == g.n and h.m == g.m
    assert np.array_equal(h.offsets(), g.offsets())
    assert np.array_equal(h.adjacency(), g.adjacency())
    # the file layout is the reference's: int32 4, uint32 n, uint32 m, int32 deg[n]
    raw = np.fromfile(tmp_path / "g" / "b_degree.bin", dtype=np.int32)
    assert raw[0] == 4 and raw[1] == g.n and raw[2] == g.m
    assert np.array_equal(raw[3:], np.diff(g.offsets()).astype(np.int32))


def test_load_64bit_header(tmp_path):
    write_bin(tmp_path / "w", [1, 2, 1], [1, 0, 2, 1], int_size=8)
    g = sg.Graph.load(tmp_path / "w")
    assert g.n == 3 and g.m == 4
    g.validate()


@pytest.mark.parametrize("case,deg,adj,status", [
    ("self_loop", [2, 1, 1], [0, 1, 0, 0], 3),
    ("unsorted", [2, 1, 1], [2, 1, 0, 0], 3),
    ("duplicate", [2, 1, 1], [1, 1, 0, 0], 3),
    ("id_out_of_range", [1, 1], [5, 0], 3),
])
def test_load_rejects_bad_lists(tmp_path, case, deg, adj, status):
    write_bin(tmp_path / case, deg, adj)
    with pytest.raises(sg.ScanError) as e:
        sg.Graph.load(tmp_path / case)
    assert e.value.status == status


def test_load_rejects_header_mismatch(tmp_path):
    write_bin(tmp_path / "h", [1, 1], [1, 0], m=7)
    with pytest.raises(sg.ScanError) as e:
        sg.Graph.load(tmp_path / "h")
    assert e.value.status == 3 and "sum to" in str(e.value)


def test_load_rejects_truncated_and_missing(tmp_path):
    write_bin(tmp_path / "t", [2, 1, 1], [1, 2, 0])          # adjacency one entry short
    with pytest.raises(sg.ScanError) as e:
        sg.Graph.load(tmp_path / "t")
    assert e.value.status == 2
    with pytest.raises(sg.ScanError) as e:
        sg.Graph.load(tmp_path / "nothing_here")
    assert e.value.status == 2


def test_validate_symmetry():
    off = np.array([0, 2, 2, 2], np.uint64)       # 0 -> 1, 0 -> 2 without the reverse entries
    g = sg.Graph.from_csr(off, np.array([1, 2], np.uint32))
    with pytest.raises(sg.ScanError) as e:
        g.validate(check_symmetry=True)
    assert "symmetric" in str(e.value)
    with pytest.raises(sg.ScanError):                # odd m cannot be symmetric
        sg.Graph.from_csr(np.array([0, 1, 1], np.uint64), np.array([1], np.uint32))


def test_run_argument_errors():
    g = sg.Graph.from_edges(4, [(0, 1), (1, 2)])
    with pytest.raises(sg.ScanError) as e:
        g.run("0.5", 0)
    assert e.value.status == 1
    with pytest.raises(sg.ScanError) as e:
        g.run("half", 2)
    assert e.value.status == 1
    with pytest.raises(sg.ScanError) as e:
        g.run("0.1234567891", 2, sg.PRED_EXACT)     # denominator above 2^30
    assert e.value.status == 1


# ---- generators ---------------------------------------------------------------------------------
def test_rmat_deterministic_and_clean():
    a = sg.Graph.rmat(12, 16, seed=5)
    b = sg.Graph.rmat(12, 16, seed=5)
    c = sg.Graph.rmat(12, 16, seed=6)
    assert np.array_equal(a.adjacency(), b.adjacency())
    assert not np.array_equal(a.adjacency(), c.adjacency())
    a.validate(check_symmetry=True)


def test_rmat16_counts():
    """R-MAT scale 16, edge factor 16, a/b/c/d = .57/.19/.19/.05, seed 1 (golden counts of
    this generator; platform independent: integer thresholds + splitmix64)."""
    g = sg.Graph.rmat(16, 16, seed=1)
    assert (g.n, g.m, g.max_degree) == (65536, 1818922, 9776)
    assert int((g.degrees() == 0).sum()) == 18762


def test_chung_lu_and_sbm():
    g = sg.Graph.chung_lu(20000, 2.1, 100000, 5000, seed=2)
    g.validate(check_symmetry=True)
    assert g.max_degree <= 5000 * 1.5
    s = sg.Graph.sbm(3000, 6, 0.1, 0.001, 64, seed=1)
    s.validate(check_symmetry=True)
    assert s.m > 0


# ---- orientation pins ----------------------------------------------------------------------------
GRAPHS = {
    "rmat10": lambda: sg.Graph.rmat(10, 16, seed=1),
    "rmat12": lambda: sg.Graph.rmat(12, 16, seed=2),
    "sbm": lambda: sg.Graph.sbm(2000, 4, 0.05, 0.002, 64, seed=3),
    "ties": lambda: sg.Graph.from_edges(8, [(i, (i + 1) % 8) for i in range(8)]),
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
def test_orientation_library_equals_oracle(name):
    g = GRAPHS[name]()
    eid, eu, ev = g.orient_reference()
    ou, ov = oracle.orient(g.offsets(), g.adjacency())
    assert np.array_equal(eu, ou.astype(np.int32)) and np.array_equal(ev, ov.astype(np.int32))
    assert np.array_equal(eid, oracle.eid(g.offsets(), g.adjacency()))


@pytest.mark.parametrize("name", sorted(GRAPHS))
def test_orientation_oracle_equals_reference_code(name):
    """Pin: GPUSCAN++/Graph.cpp:52-141 (getEidAndEdgeList) compiled from the reference
    sources gives the oracle's eid/Edge_u/Edge_v bit for bit."""
    if not oracle.reference_orientation_available():
        pytest.skip("reference sources not present on this machine")
    g = GRAPHS[name]()
    re_, reu, rev = oracle.reference_orient(g.offsets(), g.adjacency())
    ou, ov = oracle.orient(g.offsets(), g.adjacency())
    assert np.array_equal(reu, ou.astype(np.int32))
    assert np.array_equal(rev, ov.astype(np.int32))
    assert np.array_equal(re_, oracle.eid(g.offsets(), g.adjacency()))


# ---- predicate pins ------------------------------------------------------------------------------
def ref_f64_py(t, du, dv, eps):
    """GPUSCAN++/GPUScan.cu:145,156,220-221 evaluated with Python floats (IEEE double)."""
    deg_u, deg_v = float(du + 1), float(dv + 1)
    if deg_u < deg_v * eps * eps:
        return 0
    if eps * eps * deg_u * deg_v <= 4.0:
        return 1
    sq = ((t + 2) * (t + 2)) & 0xFFFFFFFF
    sq = sq - (1 << 32) if sq >= (1 << 31) else sq
    return int(not (float(sq) < eps * eps * float(du + 1) * float(dv + 1)))


@pytest.mark.parametrize("eps", ["0.1", "0.2", "0.3", "0.4", "0.5", "0.6", "0.7", "0.8", "0.9"])
def test_predicates_against_python(eps):
    L = oracle.lib()
    e, p, q = oracle.eps_params(eps)
    fr = Fraction(eps)
    rng = np.random.default_rng(int(fr.numerator * 100 + fr.denominator))
    cases = [(t, du, dv) for du in range(1, 40) for dv in range(du, 60, 3) for t in range(0, du, 2)]
    cases += [(int(t), int(du), int(du + dd)) for t, du, dd in
              zip(rng.integers(0, 50000, 300), rng.integers(50000, 100000, 300), rng.integers(0, 100000, 300))]
    for t, du, dv in cases:
        t = min(t, du - 1) if du > 0 else 0
        exact = int(Fraction(t + 2) ** 2 >= fr * fr * (du + 1) * (dv + 1))
        assert L.oracle_exact_similar(t, du, dv, p, q) == exact, (t, du, dv)
        assert L.oracle_ref_f64_similar(t, du, dv, e) == ref_f64_py(t, du, dv, e), (t, du, dv)


def test_exact_and_ref_disagree_at_boundary():
    L = oracle.lib()
    e, p, q = oracle.eps_params("0.4")
    # du = dv = 4, T = 0: exactly 4 >= 0.16 * 25 = 4; in double 0.16000000000000003 * 25 > 4
    assert L.oracle_exact_similar(0, 4, 4, p, q) == 1
    assert L.oracle_ref_f64_similar(0, 4, 4, e) == 0


def test_ref_predicate_int_overflow_wraps():
    # (T+2)^2 above 2^31 wraps negative in the reference's int arithmetic
    assert ref_f64_py(46338, 60000, 60000, 0.5) == 1     # 46340^2 = 2147395600 fits
    assert ref_f64_py(46339, 60000, 60000, 0.5) == 0     # 46341^2 wraps negative
    L = oracle.lib()
    assert L.oracle_ref_f64_similar(46338, 60000, 60000, 0.5) == 1
    assert L.oracle_ref_f64_similar(46339, 60000, 60000, 0.5) == 0
    assert L.oracle_exact_similar(46339, 60000, 60000, 1, 2) == 1


# ---- oracle on hand-derived answers ------------------------------------------------------------
def test_oracle_two_cliques():
    """Two 6-cliques joined by one edge, a vertex (12) touching both, a pendant (13)."""
    a = [(i, j) for i in range(6) for j in range(i + 1, 6)]
    b = [(i, j) for i in range(6, 12) for j in range(i + 1, 12)]
    g = sg.Graph.from_edges(14, a + b + [(5, 6), (12, 0), (12, 7), (13, 3)])
    label, role, counts = oracle.scan(g.offsets(), g.adjacency(), "0.7", 4, 0)
    # clique members are cores; clusters are {0..5} -> 0 and {6..11} -> 6
    assert list(label[:6]) == [0] * 6 and list(label[6:12]) == [6] * 6
    assert (role[:12] == 3).all()
    assert label[12] == -1 and role[12] == 1          # touches both clusters, similar to neither
    assert label[13] == -2 and role[13] == 0          # pendant: degree 1 -> outlier
    assert counts["clusters"] == 2 and counts["cores"] == 12


def test_oracle_cluster_ids_are_min_core():
    g = sg.Graph.rmat(11, 16, seed=8)
    label, role, _ = oracle.scan(g.offsets(), g.adjacency(), "0.4", 3, 0)
    cores = np.flatnonzero(role == 3)
    for c in np.unique(label[cores]):
        members = cores[label[cores] == c]
        assert members.min() == c


# ---- the generators are pinned: the bench graph must be the same on every host -----------
def _graph_sha256(g):
    import hashlib
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(g.offsets(), np.uint64).tobytes())
    h.update(np.ascontiguousarray(g.adjacency(), np.uint32).tobytes())
    return h.hexdigest()


def test_rmat_generator_matches_pinned_checksums():
    pins = json.loads((Path(__file__).parent / "golden" / "rmat_checksums.json").read_text())
    for scale, want in pins["rmat"].items():
        g = sg.Graph.rmat(int(scale), 16, seed=1)
        assert g.m == want["m"]
        assert _graph_sha256(g) == want["sha256"], f"R-MAT scale {scale} changed"
    w = pins["bench_workload"]
    g = sg.Graph.rmat(w["scale"], 16, seed=1)
    assert (g.n, g.m, g.num_edges, g.max_degree) == (w["n"], w["m"], w["undirected_edges"], w["max_degree"])


# ---- the CLI's argument and input errors come before any device work ----------------------
def test_cli_rejects_bad_arguments_and_missing_graphs(tmp_path):
    import subprocess

    from efficientstructuralgraphclusteringongpus_gb300 import build

    cli = str(build.CLI)
    p = subprocess.run([cli, str(tmp_path), "0.5"], capture_output=True, text=True)
    assert p.returncode == 1 and "<Graph folder> <eps> <miu>" in p.stderr
    p = subprocess.run([cli, str(tmp_path), "0.5", "5", "--predicate", "fuzzy"], capture_output=True, text=True)
    assert p.returncode == 1 and "<Graph folder>" in p.stderr
    p = subprocess.run([cli, str(tmp_path / "absent"), "0.5", "5"], capture_output=True, text=True)
    assert p.returncode == 2 and "load failed" in p.stderr
