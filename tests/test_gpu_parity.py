"""CUDA engine vs the oracle: bit-identical labels, roles, counts and common-neighbour counts.

Every test calls the engine through the C-ABI (libscan_gb300.so via ctypes).
"""
import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

pytestmark = pytest.mark.gpu

EXACT, REF = sg.PRED_EXACT, sg.PRED_REF_F64


def assert_same_as_oracle(g, eps, mu, mode):
    res = g.run(eps, mu, predicate=mode)
    label, role, counts = oracle.scan(g.offsets(), g.adjacency(), eps, mu, mode)
    bad = np.flatnonzero(res.label != label)
    assert bad.size == 0, f"eps={eps} mu={mu} mode={mode}: {bad.size} labels differ, first at {bad[:5]}"
    assert np.array_equal(res.role, role)
    st = res.stats
    assert st["num_cores"] == counts["cores"]
    assert st["num_clusters"] == counts["clusters"]
    assert st["num_borders"] == counts["borders"]
    assert st["num_hubs"] == counts["hubs"]
    assert st["num_outliers"] == counts["outliers"]
    assert st["num_similar_edges"] == counts["similar_edges"]
    assert st["pred_disagreements"] == counts["disagreements"]
    assert st["multi_cluster_borders"] == counts["multi_borders"]
    return res


# ---- hand-built graphs ------------------------------------------------------------------
def two_cliques_bridge():
    a = [(i, j) for i in range(6) for j in range(i + 1, 6)]
    b = [(i, j) for i in range(6, 12) for j in range(i + 1, 12)]
    return sg.Graph.from_edges(14, a + b + [(5, 6), (12, 0), (12, 7), (13, 3)])


def star():
    return sg.Graph.from_edges(40, [(0, i) for i in range(1, 40)] + [(1, 2), (2, 3)])


def border_two_clusters():
    # 7-cliques {0..6} and {8..14}; vertex 7 touches 5,6 and 8,9, vertex 15 touches 0 and 14.
    # At eps=0.4, mu=5 both are non-cores similar to cores of both cliques.
    a = [(i, j) for i in range(7) for j in range(i + 1, 7)]
    b = [(i, j) for i in range(8, 15) for j in range(i + 1, 15)]
    return sg.Graph.from_edges(16, a + b + [(7, 5), (7, 6), (7, 8), (7, 9), (15, 0), (15, 14)])


def wheel(spokes):
    rim = [(i, i % spokes + 1) for i in range(1, spokes + 1)]
    return sg.Graph.from_edges(spokes + 1, [(0, i) for i in range(1, spokes + 1)] + rim)


def degree_four_ring():
    # every vertex degree 4, triangle-free: cn = 0, du = dv = 4 -> the eps=0.4 boundary edge
    n = 20
    return sg.Graph.from_edges(n, [(i, (i + 1) % n) for i in range(n)] + [(i, (i + 5) % n) for i in range(n)])


HAND = {"cliques": two_cliques_bridge, "star": star, "border2": border_two_clusters, "ring4": degree_four_ring}


@pytest.mark.parametrize("name", sorted(HAND))
@pytest.mark.parametrize("eps", ["0.2", "0.4", "0.5", "0.7", "0.9", "1.0"])
@pytest.mark.parametrize("mu", [1, 2, 3, 5])
@pytest.mark.parametrize("mode", [EXACT, REF])
def test_hand_built(name, eps, mu, mode):
    assert_same_as_oracle(HAND[name](), eps, mu, mode)


def test_eps_boundary_modes_differ():
    g = degree_four_ring()
    ex = assert_same_as_oracle(g, "0.4", 2, EXACT)
    rf = assert_same_as_oracle(g, "0.4", 2, REF)
    # exact: 2^2 * 25 >= 4 * 25 holds on every edge; the reference's double says no
    assert ex.stats["num_similar_edges"] == g.num_edges
    assert rf.stats["num_similar_edges"] == 0
    assert ex.stats["pred_disagreements"] == g.num_edges


def test_border_in_two_clusters_takes_smallest():
    g = border_two_clusters()
    res = assert_same_as_oracle(g, "0.4", 5, EXACT)
    assert (res.role[[7, 15]] == sg.ROLE_BORDER).all()
    assert res.stats["num_clusters"] == 2 and res.stats["multi_cluster_borders"] == 2
    cl, vx = g.memberships("0.4", 5, EXACT)
    ocl, ovx = oracle.memberships(g.offsets(), g.adjacency(), "0.4", 5, EXACT)
    assert np.array_equal(cl, ocl) and np.array_equal(vx, ovx)
    assert sorted(cl[vx == 7].tolist()) == [0, 8]
    assert res.label[7] == 0 and res.label[15] == 0


def test_isolated_and_empty_edges():
    g = sg.Graph.from_edges(10, [(0, 1)])
    res = assert_same_as_oracle(g, "0.5", 1, EXACT)
    assert (res.label[2:] == -2).all()


# ---- generated graphs -------------------------------------------------------------------
# By default pivots above degree 6,144 take the hub paths (the filter kernel up to 12,288
# entries in one-shot runs, the hot-id bitmap kernel above it and for full counts); "off"
# forces the hash-table classes and the chunked hub path on the same graphs.
@pytest.fixture(params=["default", "off"])
def bitmap(request, monkeypatch):
    if request.param == "default":
        monkeypatch.delenv("SCAN_GB300_BITMAP", raising=False)
    else:
        monkeypatch.setenv("SCAN_GB300_BITMAP", request.param)
    return request.param


@pytest.mark.parametrize("scale,seed", [(8, 1), (10, 2), (12, 3), (14, 4)])
@pytest.mark.parametrize("eps", ["0.2", "0.4", "0.5", "0.6", "0.8"])
@pytest.mark.parametrize("mu", [2, 5, 10])
def test_rmat_both_modes(scale, seed, eps, mu, bitmap):
    g = sg.Graph.rmat(scale, 16, seed=seed)
    assert_same_as_oracle(g, eps, mu, EXACT)
    assert_same_as_oracle(g, eps, mu, REF)


@pytest.mark.parametrize("eps", ["0.05", "0.3", "0.5", "0.7"])
def test_rmat16_chunked_hubs_both_modes(eps, bitmap):
    """R-MAT scale 16 has pivots above the 6144-entry chunk: with the bitmap off they are
    split into id-range chunks."""
    g = sg.Graph.rmat(16, 16, seed=3)
    assert g.max_degree > 6144
    assert_same_as_oracle(g, eps, 3, EXACT)
    assert_same_as_oracle(g, eps, 3, REF)


@pytest.mark.parametrize("leaves", [46337, 46338, 46339, 50000, 70000])
def test_twin_hubs_count_square_wrap(leaves, bitmap):
    """Two adjacent hubs sharing every leaf: T = leaves.  Past T + 2 = 46340 the reference's
    int square wraps and ref-f64 stops calling the edge similar; exact does not."""
    edges = [(0, 1)] + [(0, 2 + i) for i in range(leaves)] + [(1, 2 + i) for i in range(leaves)]
    g = sg.Graph.from_edges(leaves + 2, edges)
    # eps 0 and 0.00001: the reference's 'Y' prune (eps^2 deg_u deg_v <= 4) calls the hub-hub
    # edge similar even where its wrapped square says not
    for eps in ("0", "0.00001", "0.00005", "0.5", "0.99", "1"):
        assert_same_as_oracle(g, eps, 2, EXACT)
        assert_same_as_oracle(g, eps, 2, REF)
        assert_same_as_oracle(g, eps, 1, REF)


@pytest.mark.parametrize("knob", ["default", "tails-free"])
def test_bitmap_with_tails_matches_oracle(knob, monkeypatch):
    """More non-isolated vertices than hot ids: the bitmap kernel keeps the rest of each
    pivot's list (its tail) in the shared-memory table ("tails-free" keeps such graphs on
    the hash classes)."""
    if knob == "default":
        monkeypatch.delenv("SCAN_GB300_BITMAP", raising=False)
    else:
        monkeypatch.setenv("SCAN_GB300_BITMAP", knob)
    g = sg.Graph.chung_lu(1_300_000, 2.1, 6_000_000, 20000, seed=12)
    assert (np.diff(g.offsets()) > 0).sum() > (1 << 20)
    for eps, mu in (("0.3", 3), ("0.5", 5)):
        assert_same_as_oracle(g, eps, mu, EXACT)
        assert_same_as_oracle(g, eps, mu, REF)
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))


def test_rmat16_reference_config():
    """R-MAT scale 16, edge factor 16, eps=0.5, mu=5 (the reference's CPU-runnable case)."""
    g = sg.Graph.rmat(16, 16, seed=1)
    assert_same_as_oracle(g, "0.5", 5, REF)
    assert_same_as_oracle(g, "0.5", 5, EXACT)


@pytest.mark.parametrize("make", [
    lambda: sg.Graph.rmat(12, 16, seed=11),
    lambda: sg.Graph.rmat(16, 16, seed=1),
    lambda: sg.Graph.chung_lu(60000, 2.1, 400000, 30000, seed=5),   # hubs above the chunk size
    lambda: sg.Graph.chung_lu(200000, 2.1, 1500000, 60000, seed=8),
    lambda: sg.Graph.sbm(20000, 16, 0.1, 0.001, 64, seed=2),
    lambda: star(),
    lambda: wheel(20000),                                            # one pivot in several chunks
])
def test_common_neighbors_exact(make, bitmap):
    g = make()
    cn, st = g.common_neighbors()
    ref = oracle.common_neighbors(g.offsets(), g.adjacency())
    assert cn.shape == ref.shape
    bad = np.flatnonzero(cn != ref)
    assert bad.size == 0, f"{bad.size} edges differ"
    assert st["ms_similarity"] > 0


def test_sparse_ids_with_long_empty_runs(bitmap):
    # 300 active vertices 997 ids apart: each 2,048-entry tile's owner map scatters its list
    # starts across runs of ~1,000 empty lists; one active hub spans several tiles
    rng = np.random.default_rng(17)
    active = np.arange(300) * 997
    edges = {(int(a), int(b)) for a, b in zip(rng.choice(active, 9000), rng.choice(active, 9000)) if a < b}
    edges |= {(0, int(b)) for b in active[1:]}
    g = sg.Graph.from_edges(int(active[-1]) + 5, sorted(edges))
    assert g.m > 4 * 2048 and g.max_degree == 299
    for eps in ("0.2", "0.5"):
        assert_same_as_oracle(g, eps, 3, EXACT)
        assert_same_as_oracle(g, eps, 3, REF)
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))


def test_wheel_hub_pipeline(bitmap):
    g = wheel(20000)
    for eps in ("0.01", "0.3"):
        assert_same_as_oracle(g, eps, 2, EXACT)


@pytest.mark.parametrize("n", [5000, 200000])
def test_triangle_strip_one_long_cluster(n):
    # every vertex is a core and the cluster is one long chain: deep union-find forests
    g = sg.Graph.from_edges(n, [(i, i + 1) for i in range(n - 1)] + [(i, i + 2) for i in range(n - 2)])
    res = assert_same_as_oracle(g, "0.3", 2, EXACT)
    assert res.stats["num_clusters"] == 1 and (res.label == 0).all()


def test_chunked_hub_pipeline(bitmap):
    g = sg.Graph.chung_lu(60000, 2.1, 400000, 30000, seed=5)
    assert g.max_degree > 6144          # above the per-CTA chunk: the hub is split
    for eps in ("0.1", "0.3"):
        assert_same_as_oracle(g, eps, 3, EXACT)
        assert_same_as_oracle(g, eps, 3, REF)


@pytest.mark.parametrize("eps", ["0.12", "0.15", "0.18", "0.2", "0.22", "0.25"])
def test_sbm_dense_blocks_near_threshold(eps, bitmap):
    """Blocks of 2,000 at p_in = 0.2: lists of ~400 entries (whole-warp streaming) and
    intra-block similarities near 0.2, so many edges are decided close to the early-stop
    threshold."""
    g = sg.Graph.sbm(16000, 8, 0.2, 0.002, 512, seed=7)
    for mu in (2, 20):
        assert_same_as_oracle(g, eps, mu, EXACT)
        assert_same_as_oracle(g, eps, mu, REF)


def test_sbm_pipeline(bitmap):
    g = sg.Graph.sbm(5000, 8, 0.1, 0.001, 64, seed=3)
    for eps in ("0.3", "0.5", "0.7"):
        for mu in (2, 5, 8):
            assert_same_as_oracle(g, eps, mu, EXACT)


# ---- drop-in surfaces ----------------------------------------------------------------------
def test_gpuscan_compat_matches_oracle():
    g = sg.Graph.rmat(12, 16, seed=5)
    off = g.offsets().astype(np.uint32)
    adj = g.adjacency().astype(np.int32)
    for eps, mu in ((0.5, 5), (0.4, 2), (0.8, 3)):
        out = sg.GPUScan(off, adj, eps, mu)
        label, _, _ = oracle.scan(g.offsets(), g.adjacency(), repr(eps), mu, REF)
        assert np.array_equal(out, label)


@pytest.mark.parametrize("case,off,adj,msg", [
    ("self_loop", [0, 2, 3, 4], [0, 1, 0, 1], "self loop"),
    ("unsorted", [0, 2, 3, 4], [2, 1, 0, 0], "sorted"),
    ("duplicate", [0, 2, 4], [1, 1, 0, 0], "sorted"),
    ("id_range", [0, 1, 2], [7, 0], "neighbour id"),
    ("offsets", [0, 3, 2], [1, 0], "offsets"),
])
def test_drop_in_rejects_bad_graphs_on_device(case, off, adj, msg):
    # GPUScan() does no host-side validation: these are caught by the device checks
    with pytest.raises(sg.ScanError) as e:
        sg.GPUScan(np.array(off, np.uint32), np.array(adj, np.int32), 0.5, 2)
    assert msg in str(e.value)


def test_long_lists_orientation_matches_reference_order():
    # vertices above the long-list threshold take the CTA orientation path
    g = wheel(5000)
    eid, eu, ev = g.orient_reference()
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))


def test_repeat_runs_identical():
    g = sg.Graph.rmat(13, 16, seed=9)
    a = g.run("0.5", 5, EXACT)
    b = g.run("0.5", 5, EXACT)
    assert np.array_equal(a.label, b.label) and np.array_equal(a.role, b.role)


def test_degree_prune_leaves_no_stale_cache(bitmap):
    """A one-shot run skips the edges its eps rules out by degree; those partial counts must
    never be served later as cached counts."""
    g = sg.Graph.rmat(12, 16, seed=6)
    assert_same_as_oracle(g, "0.8", 5, EXACT)          # prunes most hub edges
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))
    assert_same_as_oracle(g, "0.8", 5, REF)
    cl, vx = g.memberships("0.2", 2, EXACT)
    ocl, ovx = oracle.memberships(g.offsets(), g.adjacency(), "0.2", 2, EXACT)
    assert np.array_equal(cl, ocl) and np.array_equal(vx, ovx)
    assert_same_as_oracle(g, "0.2", 2, EXACT)


def prune_boundary_graph(extra):
    # v has degree 15 (dv + 1 = 16); u has degree 3 (du + 1 = 4) with N(u) = {v, a, b} and
    # a, b also adjacent to v, so T(u, v) = 2.  At eps = 1/2: du + 1 = eps^2 (dv + 1) sits
    # exactly on the prune boundary and (T + 2)^2 = eps^2 (du + 1)(dv + 1) = 16: similar.
    v, u, a, b = 0, 1, 2, 3
    edges = [(v, u), (v, a), (v, b), (u, a), (u, b)] + [(v, 4 + i) for i in range(12)]
    edges += [(4 + i, 16 + j) for i in range(12) for j in range(extra)]
    return sg.Graph.from_edges(16 + extra, edges)


@pytest.mark.parametrize("eps", ["0.5", "0.5000001", "0.4999999", "0.25", "1", "1.5", "0"])
@pytest.mark.parametrize("extra", [0, 3])
def test_degree_prune_boundary(eps, extra):
    g = prune_boundary_graph(extra)
    for mode in (EXACT, REF):
        for mu in (1, 2, 3):
            assert_same_as_oracle(g, eps, mu, mode)


def test_memberships_match_oracle():
    g = sg.Graph.rmat(12, 16, seed=4)
    for eps, mu in (("0.3", 3), ("0.5", 5)):
        cl, vx = g.memberships(eps, mu, EXACT)
        ocl, ovx = oracle.memberships(g.offsets(), g.adjacency(), eps, mu, EXACT)
        assert np.array_equal(cl, ocl) and np.array_equal(vx, ovx)


def test_cli_matches_library(tmp_path):
    import subprocess

    from efficientstructuralgraphclusteringongpus_gb300 import build

    g = sg.Graph.rmat(11, 16, seed=6)
    g.save(tmp_path / "g")
    out = tmp_path / "labels.bin"
    p = subprocess.run([str(build.CLI), str(tmp_path / "g"), "0.5", "5", "--out", str(out)], capture_output=True,
                       text=True)
    assert p.returncode == 0, p.stderr
    lab = np.fromfile(out, dtype=np.int32)
    label, _, _ = oracle.scan(g.offsets(), g.adjacency(), "0.5", 5, REF)
    assert np.array_equal(lab, label)
    assert f"Cluster Number: {sg.count_clusters(label)}" in p.stderr


# ---- the reference's own kernels -----------------------------------------------------------
@pytest.mark.parametrize("scale,seed,eps,mu", [(10, 1, "0.5", 5), (12, 2, "0.4", 3), (12, 3, "0.6", 2),
                                               (14, 4, "0.5", 5), (16, 1, "0.5", 5)])
def test_reference_kernels_admissible(scale, seed, eps, mu):
    """The reference's GPU output must be one the oracle admits (cores and core clusters
    identical; each border label one of the oracle's memberships; hub rule consistent)."""
    if not oracle.reference_kernels_available():
        pytest.skip("reference cubin not built (reference sources absent where build() ran)")
    g = sg.Graph.rmat(scale, 16, seed=seed)
    ref, _ = oracle.reference_gpuscan(g.offsets(), g.adjacency(), float(eps), mu)
    viol = oracle.check_admissible(g.offsets(), g.adjacency(), eps, mu, REF, ref)
    assert viol == {"core": 0, "border": 0, "membership": 0, "hub_rule": 0}, viol
    # and our engine's answer is admissible in the same sense
    res = g.run(eps, mu, REF)
    assert oracle.check_admissible(g.offsets(), g.adjacency(), eps, mu, REF, res.label) == viol


# ---- uploads of 16M+ entries arrive in eight chunks checked and oriented as they land ----
def test_chunked_upload_matches_oracle():
    g = sg.Graph.rmat(20, 16, seed=12)
    assert g.m >= (16 << 20)
    assert_same_as_oracle(g, "0.4", 3, REF)
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))


@pytest.mark.parametrize("where", [0.1, 0.125, 0.5, 0.55, 0.999])
@pytest.mark.parametrize("fault", ["id", "self_loop", "order"])
def test_chunked_upload_rejects_bad_entries(where, fault):
    g = sg.Graph.rmat(20, 16, seed=12)
    off = g.offsets().astype(np.uint32)
    adj = g.adjacency().astype(np.int32).copy()
    deg = np.diff(off.astype(np.int64))
    v = int(np.searchsorted(off, int(where * len(adj)), side="right")) - 1
    while deg[v] < 2:
        v += 1
    b = int(off[v])
    if fault == "id":
        adj[b] = g.n + 5
        msg = "neighbour id"
    elif fault == "self_loop":
        adj[b] = v
        msg = "self loop"                      # reported before any order violation it causes
    else:
        adj[b], adj[b + 1] = adj[b + 1], adj[b]
        msg = "sorted"
    with pytest.raises(sg.ScanError) as e:
        sg.GPUScan(off, adj, 0.5, 2)
    assert msg in str(e.value)


# The upload passes work on tiles of 2,048 entries; at a tile's first entry "does a list
# start here" comes from the offsets rather than the tile's owner map.
@pytest.mark.parametrize("scale", [12, 20])           # one chunk; eight chunks
@pytest.mark.parametrize("fault", ["self_loop", "order"])
def test_upload_rejects_bad_entry_at_tile_start(scale, fault):
    g = sg.Graph.rmat(scale, 16, seed=3)
    off = g.offsets().astype(np.uint32)
    adj = g.adjacency().astype(np.int32).copy()
    tile = 2048
    starts = set(off.tolist())
    j = next(k for k in range(tile, len(adj), tile) if k not in starts)   # inside a list
    v = int(np.searchsorted(off, j, side="right")) - 1
    if fault == "self_loop":
        adj[j] = v
        msg = "self loop"
    else:
        adj[j - 1], adj[j] = adj[j], adj[j - 1]
        msg = "sorted"
    with pytest.raises(sg.ScanError) as e:
        sg.GPUScan(off, adj, 0.5, 2)
    assert msg in str(e.value)
    ok = sg.GPUScan(off, g.adjacency().astype(np.int32), 0.5, 2)   # the graph without the fault
    assert ok.shape == (g.n,)


# The generator pins again, in the GPU suite: it runs on the GPU host, whose CPU architecture
# differs from the one the CPU suite runs on, so the bench graph is checked on both.
def test_rmat_generator_same_on_this_host():
    import hashlib
    import json
    from pathlib import Path
    pins = json.loads((Path(__file__).parent / "golden" / "rmat_checksums.json").read_text())
    for scale, want in pins["rmat"].items():
        g = sg.Graph.rmat(int(scale), 16, seed=1)
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(g.offsets(), np.uint64).tobytes())
        h.update(np.ascontiguousarray(g.adjacency(), np.uint32).tobytes())
        assert h.hexdigest() == want["sha256"], f"R-MAT scale {scale} differs on this host"
