"""Streamed residency (scan_graph_upload_streamed): the adjacency stays in pinned host memory
read over the host link, the rest on the device under a budget.  Results must be identical."""
import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_streamed_identical_and_smaller_on_device():
    g = sg.Graph.rmat(16, 16, seed=1)
    g.upload(0)
    full = g.device_bytes
    used = g.upload_streamed(0, 128 << 20)
    assert used == g.device_bytes and used <= 128 << 20
    assert full - used >= 4 * g.m            # the adjacency is not on the device
    for mode in (sg.PRED_REF_F64, sg.PRED_EXACT):
        res = g.run("0.5", 5, mode)
        label, role, _ = oracle.scan(g.offsets(), g.adjacency(), "0.5", 5, mode)
        assert np.array_equal(res.label, label) and np.array_equal(res.role, role)
    cn, _ = g.common_neighbors()
    assert np.array_equal(cn, oracle.common_neighbors(g.offsets(), g.adjacency()))


def test_streamed_hub_graph():
    g = sg.Graph.chung_lu(60000, 2.1, 400000, 30000, seed=5)
    g.upload_streamed(0, 0)
    res = g.run("0.3", 3, sg.PRED_EXACT)
    label, _, _ = oracle.scan(g.offsets(), g.adjacency(), "0.3", 3, 0)
    assert np.array_equal(res.label, label)


def test_streamed_budget_enforced():
    g = sg.Graph.rmat(16, 16, seed=2)
    with pytest.raises(sg.ScanError) as e:
        g.upload_streamed(0, 1 << 20)
    assert e.value.status == 5 and "budget" in str(e.value)
