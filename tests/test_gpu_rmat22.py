"""The benchmark configuration itself: R-MAT scale 22, edge factor 16, seed 1.

The engine's output at the size the bench measures is compared with the oracle: every
common-neighbour count, and labels, roles and every run counter at eps=0.5, mu=5 (the
headline point, no cores) and eps=0.2, mu=2 (the sweep point with cores, clusters, borders
and hubs), in both predicates.  The reference's own kernels run on the same graph and must
give an output the oracle admits.  The oracle's counts are computed once per module
(about a minute on 16 host cores) and reused for every (eps, mu).
"""
import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

pytestmark = pytest.mark.gpu

EXACT, REF = sg.PRED_EXACT, sg.PRED_REF_F64


@pytest.fixture(scope="module")
def s22():
    g = sg.Graph.rmat(22, 16, seed=1)
    off, adj = g.offsets(), g.adjacency()
    assert g.n == 4194304 and g.num_edges == 64151738 and g.max_degree == 163088
    cn = oracle.common_neighbors(off, adj)          # every edge, reference edge order
    yield g, off, adj, cn
    g.release_device()


def test_rmat22_common_neighbors(s22):
    g, off, adj, cn = s22
    got, st = g.common_neighbors()
    bad = np.flatnonzero(got != cn)
    assert bad.size == 0, f"{bad.size} of {cn.size} counts differ, first at {bad[:5]}"


def compare(res, want):
    label, role, counts = want
    bad = np.flatnonzero(res.label != label)
    assert bad.size == 0, f"{bad.size} labels differ, first at {bad[:5]}"
    assert np.array_equal(res.role, role)
    st = res.stats
    got = {"cores": st["num_cores"], "clusters": st["num_clusters"], "borders": st["num_borders"],
           "hubs": st["num_hubs"], "outliers": st["num_outliers"], "similar_edges": st["num_similar_edges"],
           "disagreements": st["pred_disagreements"], "multi_borders": st["multi_cluster_borders"]}
    assert got == counts


@pytest.mark.parametrize("eps,mu", [("0.5", 5), ("0.2", 2)])
@pytest.mark.parametrize("mode", [REF, EXACT])
def test_rmat22_scan_matches_oracle(s22, eps, mu, mode):
    g, off, adj, cn = s22
    want = oracle.scan_ex(off, adj, eps, mu, mode, cn=cn)
    compare(g.run(eps, mu, mode), want)
    if (eps, mu) == ("0.2", 2):
        assert want[2]["cores"] > 0 and want[2]["clusters"] > 0 and want[2]["hubs"] > 0


def test_rmat22_hash_classes_only(s22, monkeypatch):
    """The same graph with the bitmap path off: hubs are split into id-range chunks, partial
    counts are added atomically and the predicate runs as its own pass."""
    g, off, adj, cn = s22
    monkeypatch.setenv("SCAN_GB300_BITMAP", "off")
    g.release_device()
    try:
        g.upload()
        compare(g.run("0.5", 5, REF), oracle.scan_ex(off, adj, "0.5", 5, REF, cn=cn))
        compare(g.run("0.2", 2, EXACT), oracle.scan_ex(off, adj, "0.2", 2, EXACT, cn=cn))
    finally:
        g.release_device()
        monkeypatch.delenv("SCAN_GB300_BITMAP")
        g.upload()


def test_rmat22_drop_in_matches_oracle(s22):
    """The call the bench's e2e figure times: GPUScan() from host CSR buffers."""
    g, off, adj, cn = s22
    label, _, _ = oracle.scan_ex(off, adj, "0.5", 5, REF, cn=cn)
    out = sg.GPUScan(off.astype(np.uint32), adj.view(np.int32), 0.5, 5)
    assert np.array_equal(out, label)


_prepared = {}


@pytest.mark.parametrize("eps,mu", [("0.5", 5), ("0.2", 2)])
def test_rmat22_reference_kernels_admissible(s22, eps, mu):
    """GPUSCAN++'s kernels on the benchmark graph (its cubin, its launch order): the oracle
    must admit their output, and the engine's answer is admissible in the same sense."""
    if not oracle.reference_kernels_available():
        pytest.skip("reference cubin not built (reference sources absent where build() ran)")
    g, off, adj, cn = s22
    if "s22" not in _prepared:                      # GPUScan()'s host inputs, made once
        _prepared["s22"] = oracle.reference_gpuscan_prepare(off, adj)
    ref, _ = oracle.reference_gpuscan(off, adj, float(eps), mu, prepared=_prepared["s22"])
    viol = oracle.check_admissible(off, adj, eps, mu, REF, ref, cn=cn)
    assert viol == {"core": 0, "border": 0, "membership": 0, "hub_rule": 0}, viol
    res = g.run(eps, mu, REF)
    assert oracle.check_admissible(off, adj, eps, mu, REF, res.label, cn=cn) == viol
