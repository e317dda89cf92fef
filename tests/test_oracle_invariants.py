"""The oracle on the reference's angular invariants (tests/rustalgos/test_centrality.py:677-869):
simplest-path closeness and betweenness differ from shortest-path ones on the mock dual (same
density when nothing is cut off), and betweenness does not depend on node insertion order, also
with a non-live node interleaved."""
import networkx as nx
import numpy as np

import oracle
from cityseer_gb300 import common
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph

SPEED = 1.33333


def _thr(dists):
    return common.pair_distances_betas_time(SPEED, distances=dists)


def _both(ns, dists, closeness, betweenness):
    d, b, s = _thr(dists)
    og = oracle.OracleGraph(ns)
    short, _ = oracle.centrality_shortest(og, d, b, s, ns=ns, closeness=closeness, betweenness=betweenness)
    simp, _ = oracle.centrality_simplest(og, d, b, s, ns=ns, closeness=closeness, betweenness=betweenness)
    return short, simp


def test_simplest_differs_from_shortest_on_the_mock_dual():
    _, _, ns = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))
    short, simp = _both(ns, [5000], True, False)
    np.testing.assert_allclose(short[0, 0], simp[0, 0], atol=0.01)  # density: nothing cut off
    assert not np.allclose(short[1, 0], simp[1, 0], atol=0.01)  # farness
    assert not np.allclose(short[3, 0], simp[2, 0], atol=0.01)  # harmonic
    short, simp = _both(ns, [500, 2000], False, True)
    for k in range(2):
        assert short[5, k].sum() > 0 and simp[3, k].sum() > 0
        assert not np.allclose(short[5, k], simp[3, k], atol=0.01)


def _graph(coords, edges, ordering, live=None):
    lab = {a: str(i) for i, a in enumerate(ordering)}
    g = nx.MultiGraph()
    for a in ordering:
        nd = {"x": coords[a][0], "y": coords[a][1]}
        if live is not None:
            nd["live"] = live[a]
        g.add_node(lab[a], **nd)
    for a, b in edges:
        g.add_edge(lab[a], lab[b])
    return graphs.nx_simple_geoms(g), {v: k for k, v in lab.items()}


def _dual_betweenness_by_edge(g, unlab, dist):
    nodes, _, ns = io.network_structure_from_nx(graphs.nx_to_dual(g))
    d, b, s = _thr([dist])
    out, _ = oracle.centrality_simplest(oracle.OracleGraph(ns), d, b, s, ns=ns, closeness=False)
    res = {}
    for key, a, bb, idx in zip(nodes["index"], nodes["primal_edge_node_a"], nodes["primal_edge_node_b"],
                               nodes["ns_node_idx"]):
        res[tuple(sorted((unlab[a], unlab[bb])))] = out[3, 0, idx]
    return res


def test_simplest_betweenness_invariant_to_node_order():
    coords = {"A": (500000.0, 0.0), "B": (500000.0, 100.0), "C": (500100.0, 100.0), "D": (500050.0, 170.0)}
    edges = [("A", "B"), ("B", "C"), ("B", "D")]
    runs = [_dual_betweenness_by_edge(*_graph(coords, edges, o), 500)
            for o in (["A", "B", "C", "D"], ["D", "C", "B", "A"], ["C", "A", "D", "B"])]
    for e in [("A", "B"), ("B", "C"), ("B", "D")]:
        vals = [r[e] for r in runs]
        assert max(vals) - min(vals) < 0.01, (e, vals)


def test_betweenness_with_a_non_live_node_invariant_to_node_order():
    coords = {"A": (500000.0, 0.0), "B": (500000.0, 100.0), "C": (500000.0, 200.0), "D": (500000.0, 300.0)}
    edges = [("A", "B"), ("B", "C"), ("C", "D")]
    live = {"A": True, "B": True, "C": True, "D": False}
    short_runs, simp_runs = [], []
    for o in (["A", "B", "C", "D"], ["D", "A", "B", "C"], ["B", "D", "A", "C"]):
        g, unlab = _graph(coords, edges, o, live)
        nodes, _, ns = io.network_structure_from_nx(g)
        d, b, s = _thr([1000])
        out, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, ns=ns, closeness=False)
        short_runs.append({unlab[k]: out[5, 0, i] for k, i in zip(nodes["index"], nodes["ns_node_idx"])})
        simp_runs.append(_dual_betweenness_by_edge(g, unlab, 1000))
    for a in "ABCD":
        vals = [r[a] for r in short_runs]
        assert max(vals) - min(vals) < 0.01, (a, vals)
    for e in [("A", "B"), ("B", "C"), ("C", "D")]:
        vals = [r[e] for r in simp_runs]
        assert max(vals) - min(vals) < 0.01, (e, vals)


def test_segment_closeness_invariant_under_decomposition():
    """tests/rustalgos/test_centrality.py:622-649: segment closeness measures to the cut endpoints of
    each threshold, so decomposing every edge into 20 m pieces leaves the sums over the original
    nodes unchanged."""
    g = mock_graph()
    gd = graphs.nx_decompose(g, 20)
    assert gd.number_of_nodes() > g.number_of_nodes()
    assert all(graphs._length(graphs.coords_of(dd["geom"])) <= 20.0 + 1e-6 for _, _, dd in gd.edges(data=True))
    _, _, ns = io.network_structure_from_nx(g)
    _, _, nsd = io.network_structure_from_nx(gd)
    d, b, s = _thr([200, 400, 800, 5000])
    seg = oracle.segment_centrality(oracle.OracleGraph(ns), d, b, s, ns=ns)
    segd = oracle.segment_centrality(oracle.OracleGraph(nsd), d, b, s, ns=nsd)
    n = ns.node_count()
    k = list(d).index(400)
    for m in (0, 1, 2):  # density, harmonic, beta
        assert np.isclose(seg[m, k].sum(), segd[m, k][:n].sum()), m
