"""Batched SCAN (scan_batch_*): many graphs with their own (eps, mu) in one captured pass.

Each graph's result must be identical to scan_run on that graph alone; the second run
replays the captured CUDA graph with new parameters.
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
def test_batch_matches_each_graph_alone(mode):
    graphs = small_sbm_batch(30, 1)
    with sg.Batch(graphs, 0, autotune=True) as b:
        for rep in range(2):      # rep 0 captures the CUDA graph, rep 1 replays it
            eps, mus = params(len(graphs), 10 + rep)
            labels, roles, st = b.run(eps, mus, mode)
            assert st["num_graphs"] == len(graphs) and st["graph_kernels"] > 0
            cores = 0
            for g, lab, rol, e, m in zip(graphs, labels, roles, eps, mus):
                alone = g.run(e, m, mode)
                assert np.array_equal(lab, alone.label) and np.array_equal(rol, alone.role)
                cores += alone.stats["num_cores"]
            assert st["num_cores"] == cores


def test_autotuned_graph_matches_oracle():
    g = sg.Graph.rmat(14, 16, seed=8)
    info = g.autotune()
    assert info["long_words"] in (16, 32, 64) and info["similarity_ms"] > 0
    res = g.run("0.4", 3, sg.PRED_EXACT)
    label, role, _ = oracle.scan(g.offsets(), g.adjacency(), "0.4", 3, 0)
    assert np.array_equal(res.label, label) and np.array_equal(res.role, role)
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))
