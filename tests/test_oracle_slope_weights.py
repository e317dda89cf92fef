"""The oracle on the reference's slope and node-weight checks (tests/rustalgos/test_centrality.py:
343-389 node weights scale closeness but not cycles; :392-448 directional slope penalties, flat cost
when an endpoint has no z, angular routing unaffected on the dual)."""
import networkx as nx
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph

SPEED = 1.33333


def _line(zs):
    g = nx.MultiGraph()
    for i, z in enumerate(zs):
        nd = {"x": 100.0 * i, "y": 0.0}
        if z is not None:
            nd["z"] = z
        g.add_node(str(i), **nd)
    for i in range(len(zs) - 1):
        g.add_edge(str(i), str(i + 1))
    return graphs.nx_simple_geoms(g)


def _idx(ns, key):
    return ns.node_keys_py().index(key)


def test_node_weights_scale_closeness_not_cycles():
    d, b, s = common.pair_distances_betas_time(SPEED, distances=[400, 1600])
    _, _, ns = io.network_structure_from_nx(mock_graph())
    base, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, ns=ns, betweenness=False)
    for wt in (0.5, 2.0):
        g = mock_graph()
        for n in g:
            g.nodes[n]["weight"] = wt
        _, _, nsw = io.network_structure_from_nx(g)
        got, _ = oracle.centrality_shortest(oracle.OracleGraph(nsw), d, b, s, ns=nsw, betweenness=False)
        for m in (0, 1, 3, 4):  # density, farness, harmonic, beta
            np.testing.assert_allclose(got[m], base[m] * wt, rtol=1e-6, atol=1e-9)
        np.testing.assert_array_equal(got[2], base[2])  # cycles


def test_directional_slope_penalty():
    flat = 100.0 / SPEED
    _, _, ns = io.network_structure_from_nx(_line([0.0, 5.0]))
    og = oracle.OracleGraph(ns)
    i0, i1 = _idx(ns, "0"), _idx(ns, "1")
    # the search runs over reversed edges: a tree from 0 times the walk 1 -> 0 (downhill)
    down = oracle.tree_shortest(og, i0, 1000, SPEED)[1]["agg_seconds"][i1]
    up = oracle.tree_shortest(og, i1, 1000, SPEED)[1]["agg_seconds"][i0]
    assert down < flat < up
    with pytest.raises(ValueError, match="dual graph"):
        ns.dijkstra_tree_simplest(i0, 1000, SPEED)
    # missing z on an endpoint: flat cost both ways
    _, _, nsp = io.network_structure_from_nx(_line([0.0, None]))
    ogp = oracle.OracleGraph(nsp)
    j0, j1 = _idx(nsp, "0"), _idx(nsp, "1")
    assert np.isclose(oracle.tree_shortest(ogp, j0, 1000, SPEED)[1]["agg_seconds"][j1], flat, atol=0.01)
    assert np.isclose(oracle.tree_shortest(ogp, j1, 1000, SPEED)[1]["agg_seconds"][j0], flat, atol=0.01)


def test_dual_slope_keeps_angular_routes():
    flat = 100.0 / SPEED
    dual = graphs.nx_to_dual(_line([0.0, 5.0, 10.0]))
    assert dual.nodes["0_1_k0"]["z"] == pytest.approx(2.5) and dual.nodes["1_2_k0"]["z"] == pytest.approx(7.5)
    _, _, nsd = io.network_structure_from_nx(dual)
    og = oracle.OracleGraph(nsd)
    a, b = _idx(nsd, "0_1_k0"), _idx(nsd, "1_2_k0")
    ta = oracle.tree_simplest(og, a, 1000, SPEED)[1]
    tb = oracle.tree_simplest(og, b, 1000, SPEED)[1]
    ab, ba = ta["agg_seconds"][b], tb["agg_seconds"][a]
    assert not np.isclose(ab, ba, atol=0.01)
    assert min(ab, ba) < flat < max(ab, ba)
    assert np.isclose(ta["simpl_dist"][b], 0.0, atol=0.01) and np.isclose(tb["simpl_dist"][a], 0.0, atol=0.01)
