"""Every similarity plan gives the oracle's results.

The plan (the small-pivot intersection strategy and degree cut, the hub threshold, the
largest table chunk) is what the autotuner chooses per graph or batch; each setting must
give identical labels, roles, counters and common-neighbour counts.  Plans are pinned with
scan_graph_set_plan so every strategy runs whatever the tuner would pick.
"""
import itertools

import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

pytestmark = pytest.mark.gpu

PLANS = list(itertools.product((64, 128), (sg.SMALL_SERIAL, sg.SMALL_BATCHED, sg.SMALL_SEARCH), (4096, 6144),
                               (6144, 12288)))


def graphs():
    return {"rmat14": sg.Graph.rmat(14, 16, seed=21),
            "sbm": sg.Graph.sbm(30000, 24, 0.1, 0.001, 64, seed=22),
            "chung_lu": sg.Graph.chung_lu(200000, 2.1, 1500000, 60000, seed=23)}


@pytest.fixture(scope="module")
def cases():
    out = {}
    for name, g in graphs().items():
        off, adj = g.offsets(), g.adjacency()
        out[name] = (g, off, adj, oracle.common_neighbors(off, adj))
    yield out
    for g, *_ in out.values():
        g.release_device()


@pytest.mark.parametrize("name", ["rmat14", "sbm", "chung_lu"])
@pytest.mark.parametrize("small_deg,strategy,hub,chunk", PLANS)
def test_plan_matches_oracle(cases, name, small_deg, strategy, hub, chunk):
    g, off, adj, cn = cases[name]
    g.set_plan(small_deg, strategy, hub, chunk)
    assert g.plan() == {"small_deg": small_deg, "small_strategy": strategy, "hub_min_deg": hub, "chunk_max": chunk}
    for eps, mu, mode in (("0.5", 5, sg.PRED_REF_F64), ("0.3", 2, sg.PRED_EXACT)):
        res = g.run(eps, mu, mode)
        label, role, counts = oracle.scan_ex(off, adj, eps, mu, mode, cn=cn)
        assert np.array_equal(res.label, label) and np.array_equal(res.role, role), (eps, mu, mode)
        assert res.stats["num_similar_edges"] == counts["similar_edges"]
        assert res.stats["pred_disagreements"] == counts["disagreements"]
    got, _ = g.common_neighbors()
    assert np.array_equal(got, cn)


def test_set_plan_rejects_bad_values():
    g = sg.Graph.rmat(8, 16, seed=1)
    for bad in ((0, 0, 6144, 6144), (129, 0, 6144, 6144), (64, 3, 6144, 6144), (64, 0, 32, 6144),
                (64, 0, 6144, 5000)):
        with pytest.raises(sg.ScanError) as e:
            g.set_plan(*bad)
        assert e.value.status == 1


def test_autotune_reports_its_plan():
    g = sg.Graph.sbm(20000, 16, 0.1, 0.001, 64, seed=24)
    info = g.autotune()
    assert info["small_deg"] in (64, 128) and info["small_strategy"] in (0, 1, 2)
    assert info["hub_min_deg"] in (4096, 6144) and info["chunk_max"] in (6144, 12288)
    label, role, _ = oracle.scan(g.offsets(), g.adjacency(), "0.4", 3, 0)
    res = g.run("0.4", 3, sg.PRED_EXACT)
    assert np.array_equal(res.label, label) and np.array_equal(res.role, role)
