"""Serving loop (scan_server_*): cached common-neighbour counts, continuous batching.

Every served result must equal the oracle's SCAN of that graph at the query's (eps, mu) and
predicate, and equal scan_run on the same graph alone, whether the query ran alone or mixed
with others on the device.  The oracle's counts are computed once per graph (reference edge
order) and reused for every query on it.
"""
import threading

import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from oracle import oracle

pytestmark = pytest.mark.gpu


class OracleOf:
    """The oracle's answers for one graph, its common-neighbour counts computed once."""

    def __init__(self, g):
        self.off, self.adj = g.offsets(), g.adjacency()
        self.cn = oracle.common_neighbors(self.off, self.adj)

    def scan(self, eps, mu, pred):
        return oracle.scan_ex(self.off, self.adj, eps, mu, pred, cn=self.cn)


def check_served(label, role, info, want, where):
    ol, orole, oc = want
    assert np.array_equal(label, ol), where
    assert np.array_equal(role, orole), where
    assert info["num_cores"] == oc["cores"], where
    assert info["num_clusters"] == oc["clusters"], where
    assert info["num_similar_edges"] == oc["similar_edges"], where


def pool():
    return [sg.Graph.rmat(10, 16, seed=1), sg.Graph.rmat(12, 16, seed=2), sg.Graph.sbm(4000, 8, 0.1, 0.001, 64, seed=3),
            sg.Graph.rmat(14, 16, seed=4), sg.Graph.from_edges(3, [(0, 1)])]


def random_queries(k, ngraphs, seed):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(ngraphs)), f"0.{int(rng.integers(1, 10))}", int(rng.integers(2, 21)),
             int(rng.integers(0, 2))) for _ in range(k)]


def test_mixed_queries_identical_to_alone_and_oracle():
    graphs = pool()
    ref = [OracleOf(g) for g in graphs]
    with sg.Server(0, 256 << 20, 4) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        qs = random_queries(200, len(graphs), 0)
        tickets = [srv.submit(ids[gi], eps, mu, pred) for gi, eps, mu, pred in qs]   # all in flight at once
        for t, (gi, eps, mu, pred) in zip(tickets, qs):
            label, role, info = srv.wait(t)
            check_served(label, role, info, ref[gi].scan(eps, mu, pred), (gi, eps, mu, pred))
            alone = graphs[gi].run(eps, mu, pred)
            assert np.array_equal(label, alone.label), (gi, eps, mu, pred)
            assert np.array_equal(role, alone.role)
            assert info["latency_ms"] >= info["queue_ms"] >= 0
        c = srv.counters()
        assert c["completed"] == c["submitted"] == 200 and c["failed"] == 0 and c["pending"] == 0


def test_budget_for_one_query_at_a_time():
    graphs = pool()[:4]
    ref = [OracleOf(g) for g in graphs]
    with sg.Server(0, 1 << 20, 8) as srv:            # about one scratch block of the scale-14 graph
        ids = [srv.add_graph(g) for g in graphs]
        qs = random_queries(40, len(graphs), 1)
        tickets = [srv.submit(ids[gi], eps, mu, pred) for gi, eps, mu, pred in qs]
        for t, (gi, eps, mu, pred) in zip(tickets, qs):
            label, role, info = srv.wait(t)
            check_served(label, role, info, ref[gi].scan(eps, mu, pred), (gi, eps, mu, pred))


def test_query_above_budget_fails_others_served():
    big, small = sg.Graph.rmat(15, 16, seed=5), sg.Graph.rmat(8, 16, seed=6)
    with sg.Server(0, 1 << 20, 2) as srv:            # 1 MiB: the scale-15 scratch cannot fit
        gb, gs = srv.add_graph(big), srv.add_graph(small)
        t_big = srv.submit(gb, "0.5", 3)
        t_small = srv.submit(gs, "0.5", 3)
        with pytest.raises(sg.ScanError) as e:
            srv.wait(t_big)
        assert e.value.status == 5
        label, role, info = srv.wait(t_small)
        check_served(label, role, info, OracleOf(small).scan("0.5", 3, sg.PRED_EXACT), "small")


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
    """Served queries decide each edge from its cached similarity threshold with one compare,
    and test the edges whose threshold lies within a relative 1e-6 of eps^2 with the
    predicate itself.  At eps values on and around the exact and reference boundaries
    (degree-4 ring at eps 0.4, the degree-prune boundary at 0.5, the int-square wrap of the
    twin hubs) every result must equal the oracle and scan_run."""
    graphs = boundary_graphs()
    ref = [OracleOf(g) for g in graphs]
    eps_values = ["0", "0.1", "0.15", "0.2", "0.22", "0.4", "0.4999999", "0.5", "0.5000001", "0.7071", "0.99", "1",
                  "1.5"]
    with sg.Server(0, 512 << 20, 8) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        qs = [(gi, e, mu, pred) for gi in range(len(graphs)) for e in eps_values for mu in (1, 2, 5)
              for pred in (sg.PRED_EXACT, sg.PRED_REF_F64)]
        tickets = [srv.submit(ids[gi], e, mu, pred) for gi, e, mu, pred in qs]
        for t, (gi, e, mu, pred) in zip(tickets, qs):
            label, role, info = srv.wait(t)
            check_served(label, role, info, ref[gi].scan(e, mu, pred), (gi, e, mu, pred))
            alone = graphs[gi].run(e, mu, pred)
            assert np.array_equal(label, alone.label), (gi, e, mu, pred)
            assert info["num_similar_edges"] == alone.stats["num_similar_edges"], (gi, e, mu, pred)


def test_concurrent_add_graph_while_serving():
    """Two threads add graphs of increasing size (each larger one grows the pinned result
    staging) while a third keeps queries on an existing graph in flight; every result must
    still equal the oracle's."""
    base = sg.Graph.rmat(10, 16, seed=21)
    base_ref = OracleOf(base)
    adds = [[sg.Graph.rmat(s, 8, seed=30 + s) for s in (11, 13, 15)],
            [sg.Graph.rmat(s, 8, seed=40 + s) for s in (12, 14, 16)]]
    errors, added = [], []
    with sg.Server(0, 256 << 20, 4) as srv:
        gid = srv.add_graph(base)
        stop = threading.Event()

        def adder(gs):
            try:
                for g in gs:
                    added.append((srv.add_graph(g), g))
            except Exception as e:   # reported below
                errors.append(e)

        def querier():
            rng = np.random.default_rng(5)
            try:
                while not stop.is_set():
                    eps, mu, pred = f"0.{int(rng.integers(1, 10))}", int(rng.integers(2, 8)), int(rng.integers(0, 2))
                    label, role, info = srv.wait(srv.submit(gid, eps, mu, pred))
                    check_served(label, role, info, base_ref.scan(eps, mu, pred), (eps, mu, pred))
            except Exception as e:
                errors.append(e)

        qt = threading.Thread(target=querier)
        qt.start()
        ts = [threading.Thread(target=adder, args=(gs,)) for gs in adds]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        stop.set()
        qt.join()
        assert not errors, errors
        assert len(added) == 6
        for i, g in added:                      # every added graph is served correctly
            label, role, info = srv.wait(srv.submit(i, "0.3", 3, sg.PRED_REF_F64))
            check_served(label, role, info, OracleOf(g).scan("0.3", 3, sg.PRED_REF_F64), i)
