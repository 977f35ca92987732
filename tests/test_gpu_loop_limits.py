"""The bounded device loops give up with an error the caller sees, and the device stays usable.

The union-find's CAS loop (a limited number of attempts per union) and the pointer-jumping
flatten (a fixed number of queued rounds) are shrunk with scan_set_loop_limits until they
cannot finish: every entry point that runs them -- scan_run, a served query, a batch --
must then report SCAN_ERR_DEVICE.  No kernel waits on anything here: the shrunk loops just
stop early.  With the limits restored the same calls equal the oracle again.
"""
import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

pytestmark = pytest.mark.gpu

DEVICE_ERR = 7


def strip(n):
    # every vertex a core at eps 0.3, mu 2; one long cluster: the unions of concurrent
    # threads leave a deep forest that one jumping round cannot flatten
    return sg.Graph.from_edges(n, [(i, i + 1) for i in range(n - 1)] + [(i, i + 2) for i in range(n - 2)])


@pytest.fixture(autouse=True)
def restore_limits():
    yield
    sg.set_loop_limits(-1, -1)


def expect_device_error(fn):
    with pytest.raises(sg.ScanError) as e:
        fn()
    assert e.value.status == DEVICE_ERR, e.value


@pytest.mark.parametrize("n", [5000, 200000])      # one-CTA flatten; chain of rounds
def test_union_find_limit_scan_run(n):
    g = strip(n)
    sg.set_loop_limits(0, -1)                       # no CAS attempt: every core-core union fails
    expect_device_error(lambda: g.run("0.3", 2, sg.PRED_EXACT))
    sg.set_loop_limits(-1, -1)
    res = g.run("0.3", 2, sg.PRED_EXACT)
    label, role, _ = oracle.scan(g.offsets(), g.adjacency(), "0.3", 2, 0)
    assert np.array_equal(res.label, label) and np.array_equal(res.role, role)


def test_flatten_round_limit_scan_run():
    g = strip(200000)
    sg.set_loop_limits(-1, 1)                       # one jumping round for a deep forest
    expect_device_error(lambda: g.run("0.3", 2, sg.PRED_EXACT))
    sg.set_loop_limits(-1, -1)
    assert (g.run("0.3", 2, sg.PRED_EXACT).label == 0).all()


def test_limits_in_served_query():
    g, small = strip(5000), sg.Graph.rmat(10, 16, seed=3)
    with sg.Server(0, 64 << 20, 4) as srv:
        gid, sid = srv.add_graph(g), srv.add_graph(small)
        sg.set_loop_limits(0, -1)
        t = srv.submit(gid, "0.3", 2)
        expect_device_error(lambda: srv.wait(t))
        sg.set_loop_limits(-1, -1)
        label, role, _ = srv.wait(srv.submit(gid, "0.3", 2))
        assert (label == 0).all()
        label, _, _ = srv.wait(srv.submit(sid, "0.5", 3))
        assert np.array_equal(label, oracle.scan(small.offsets(), small.adjacency(), "0.5", 3, 0)[0])
        c = srv.counters()
        assert c["failed"] == 1 and c["completed"] == 3


def test_limits_in_batch():
    graphs = [strip(3000), sg.Graph.rmat(9, 16, seed=2)]
    sg.set_loop_limits(0, -1)
    with sg.Batch(graphs, 0, autotune=False) as b:
        expect_device_error(lambda: b.run(["0.3", "0.5"], [2, 3]))
    sg.set_loop_limits(-1, -1)
    with sg.Batch(graphs, 0, autotune=False) as b:
        labels, _, _ = b.run(["0.3", "0.5"], [2, 3])
        assert (labels[0] == 0).all()
