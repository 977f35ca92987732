"""Batched SCAN (scan_batch_*): many graphs with their own (eps, mu) in one captured pass.

Each graph's result must equal the oracle's SCAN of that graph at its own (eps, mu), and
scan_run on that graph alone; the second run replays the captured CUDA graph with new
parameters.
"""
import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

pytestmark = pytest.mark.gpu


def small_sbm_batch(k, seed):
    rng = np.random.default_rng(seed)
    graphs = []
    for i in range(k):
        n = int(np.exp(rng.uniform(np.log(100), np.log(5000))))
        blocks = int(rng.integers(2, 17))
        graphs.append(sg.Graph.sbm(n, min(blocks, n), 0.1, 0.001, 64, seed=1000 + i))
    graphs += [sg.Graph.rmat(10, 16, seed=3), sg.Graph.from_edges(5, [(0, 1), (1, 2)])]
    return graphs


def params(k, seed):
    rng = np.random.default_rng(seed)
    return [("0.3", "0.5", "0.7")[i] for i in rng.integers(0, 3, k)], [int(x) for x in rng.integers(2, 9, k)]


@pytest.mark.parametrize("mode", [sg.PRED_EXACT, sg.PRED_REF_F64])
def test_batch_matches_oracle_and_each_graph_alone(mode):
    graphs = small_sbm_batch(30, 1)
    cns = [oracle.common_neighbors(g.offsets(), g.adjacency()) for g in graphs]
    with sg.Batch(graphs, 0, autotune=True) as b:
        for rep in range(2):      # rep 0 captures the CUDA graph, rep 1 replays it
            eps, mus = params(len(graphs), 10 + rep)
            labels, roles, st = b.run(eps, mus, mode)
            assert st["num_graphs"] == len(graphs) and st["graph_kernels"] > 0
            cores = clusters = 0
            for i, (g, lab, rol, e, m) in enumerate(zip(graphs, labels, roles, eps, mus)):
                ol, orole, oc = oracle.scan_ex(g.offsets(), g.adjacency(), e, m, mode, cn=cns[i])
                assert np.array_equal(lab, ol) and np.array_equal(rol, orole), (i, e, m)
                alone = g.run(e, m, mode)
                assert np.array_equal(lab, alone.label) and np.array_equal(rol, alone.role)
                cores += oc["cores"]
                clusters += oc["clusters"]
            assert st["num_cores"] == cores and st["num_clusters"] == clusters


def test_autotuned_graph_matches_oracle():
    g = sg.Graph.rmat(14, 16, seed=8)
    info = g.autotune()
    assert info["long_words"] in (16, 32, 64) and info["similarity_ms"] > 0
    res = g.run("0.4", 3, sg.PRED_EXACT)
    label, role, _ = oracle.scan(g.offsets(), g.adjacency(), "0.4", 3, 0)
    assert np.array_equal(res.label, label) and np.array_equal(res.role, role)
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))
