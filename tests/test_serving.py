"""Serving loop (scan_server_*): cached common-neighbour counts, continuous batching.

Every served result must be identical to scan_run on the same graph and parameters, whether
the query ran alone or mixed with others on the device.
"""
import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg

pytestmark = pytest.mark.gpu


def pool():
    return [sg.Graph.rmat(10, 16, seed=1), sg.Graph.rmat(12, 16, seed=2), sg.Graph.sbm(4000, 8, 0.1, 0.001, 64, seed=3),
            sg.Graph.rmat(14, 16, seed=4), sg.Graph.from_edges(3, [(0, 1)])]


def random_queries(k, ngraphs, seed):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(ngraphs)), f"0.{int(rng.integers(1, 10))}", int(rng.integers(2, 21)),
             int(rng.integers(0, 2))) for _ in range(k)]


def test_mixed_queries_identical_to_alone():
    graphs = pool()
    with sg.Server(0, 256 << 20, 4) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        qs = random_queries(200, len(graphs), 0)
        tickets = [srv.submit(ids[gi], eps, mu, pred) for gi, eps, mu, pred in qs]   # all in flight at once
        for t, (gi, eps, mu, pred) in zip(tickets, qs):
            label, role, info = srv.wait(t)
            alone = graphs[gi].run(eps, mu, pred)
            assert np.array_equal(label, alone.label), (gi, eps, mu, pred)
            assert np.array_equal(role, alone.role)
            assert info["num_cores"] == alone.stats["num_cores"]
            assert info["latency_ms"] >= info["queue_ms"] >= 0
        c = srv.counters()
        assert c["completed"] == c["submitted"] == 200 and c["failed"] == 0 and c["pending"] == 0


def test_budget_for_one_query_at_a_time():
    graphs = pool()[:4]
    with sg.Server(0, 1 << 20, 8) as srv:            # about one scratch block of the scale-14 graph
        ids = [srv.add_graph(g) for g in graphs]
        qs = random_queries(40, len(graphs), 1)
        tickets = [srv.submit(ids[gi], eps, mu, pred) for gi, eps, mu, pred in qs]
        for t, (gi, eps, mu, pred) in zip(tickets, qs):
            label, role, _ = srv.wait(t)
            assert np.array_equal(label, graphs[gi].run(eps, mu, pred).label)


def test_query_above_budget_fails_others_served():
    big, small = sg.Graph.rmat(15, 16, seed=5), sg.Graph.rmat(8, 16, seed=6)
    with sg.Server(0, 1 << 20, 2) as srv:            # 1 MiB: the scale-15 scratch cannot fit
        gb, gs = srv.add_graph(big), srv.add_graph(small)
        t_big = srv.submit(gb, "0.5", 3)
        t_small = srv.submit(gs, "0.5", 3)
        with pytest.raises(sg.ScanError) as e:
            srv.wait(t_big)
        assert e.value.status == 5
        label, _, _ = srv.wait(t_small)
        assert np.array_equal(label, small.run("0.5", 3).label)


def test_replay_trace():
    graphs = pool()[:4]
    with sg.Server(0, 256 << 20, 8) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        qs = random_queries(300, len(graphs), 2)
        arrivals = np.cumsum(np.random.default_rng(3).exponential(1000.0 / 5000, len(qs)))   # 5000 q/s
        lat, st, wall = srv.replay([ids[q[0]] for q in qs], [q[1] for q in qs], [q[2] for q in qs],
                                   [q[3] for q in qs], arrivals)
        assert (st == 0).all() and (lat > 0).all()
        assert wall >= arrivals[-1]


def boundary_graphs():
    ring = [(i, (i + 1) % 20) for i in range(20)] + [(i, (i + 5) % 20) for i in range(20)]
    v, u, a, b = 0, 1, 2, 3
    prune = [(v, u), (v, a), (v, b), (u, a), (u, b)] + [(v, 4 + i) for i in range(12)]
    twin = [(0, 1)] + [(0, 2 + i) for i in range(46339)] + [(1, 2 + i) for i in range(46339)]
    return [sg.Graph.from_edges(20, ring), sg.Graph.from_edges(16, prune), sg.Graph.from_edges(46341, twin),
            sg.Graph.sbm(16000, 8, 0.2, 0.002, 512, seed=7), sg.Graph.rmat(13, 16, seed=8)]


def test_served_queries_at_predicate_boundaries():
    """Served queries visit only the edges ranked similar at their eps (the ranking groups
    edges by similarity threshold); at eps values on and around the exact and reference
    boundaries every result must still equal scan_run."""
    graphs = boundary_graphs()
    eps_values = ["0", "0.1", "0.15", "0.2", "0.22", "0.4", "0.4999999", "0.5", "0.5000001", "0.7071", "0.99", "1",
                  "1.5"]
    with sg.Server(0, 512 << 20, 8) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        qs = [(gi, e, mu, pred) for gi in range(len(graphs)) for e in eps_values for mu in (1, 2, 5)
              for pred in (sg.PRED_EXACT, sg.PRED_REF_F64)]
        tickets = [srv.submit(ids[gi], e, mu, pred) for gi, e, mu, pred in qs]
        for t, (gi, e, mu, pred) in zip(tickets, qs):
            label, role, info = srv.wait(t)
            alone = graphs[gi].run(e, mu, pred)
            assert np.array_equal(label, alone.label), (gi, e, mu, pred)
            assert np.array_equal(role, alone.role), (gi, e, mu, pred)
            assert info["num_similar_edges"] == alone.stats["num_similar_edges"], (gi, e, mu, pred)
            assert info["num_clusters"] == alone.stats["num_clusters"], (gi, e, mu, pred)
