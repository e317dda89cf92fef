"""The oracle (oracle/cs_oracle.c) pinned against the reference's own tests.

Golden vectors: tests/rustalgos/test_centrality.py:472-598 (diamond graph), networkx known answers
on the reference's mock graph (test_centrality.py:247-341, 652-674), the expected simplest/shortest
routes on its dual (test_centrality.py:139-234), the plateau ratio (:872-890) and the tolerance
drift expectations (:893-930).  All graphs come from tests/golden/reference_fixtures.json, which
tests/golden/make_fixtures.py extracts from the reference sources.
"""
import networkx as nx
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common
from cityseer_gb300.tools import graphs, io
from helpers import FIX, diamond_graph, mock_graph, nx_from_spec

SPEED = 1.33333


def _thr(dists):
    return common.pair_distances_betas_time(SPEED, distances=dists)


def _dual_of(g):
    return io.network_structure_from_nx(graphs.nx_to_dual(g))


def test_diamond_golden_vectors():
    g = diamond_graph()
    _, _, ns = io.network_structure_from_nx(g)
    _, _, nsd = _dual_of(g)
    dists = [50, 150, 250]
    d, b, s = _thr(dists)
    short, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, ns=ns, betweenness=False)
    simp, _ = oracle.centrality_simplest(oracle.OracleGraph(nsd), d, b, s, ns=nsd, betweenness=False)
    seg = oracle.segment_centrality(oracle.OracleGraph(ns), d, b, s, ns=ns)
    rows = {
        "node_result_short": (short, ["node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta"]),
        "node_result_simplest": (simp, ["node_density", "node_farness", "node_harmonic", "node_betweenness"]),
        "segment_result": (seg, ["segment_density", "segment_harmonic", "segment_beta", "segment_betweenness"]),
    }
    gold = FIX["centrality"]["local_centrality_all"]
    assert len(gold) == 30
    for gd in gold:
        arr, names = rows[gd["result"]]
        got = arr[names.index(gd["attr"]), dists.index(gd["distance"])]
        # the reference test's own tolerances (config.ATOL / config.RTOL)
        assert np.allclose(got, gd["values"], atol=0.01, rtol=1e-4), (gd, got)


@pytest.fixture(scope="module")
def mock():
    g = mock_graph()
    _, _, ns = io.network_structure_from_nx(g)
    gr = nx.Graph()
    gr.add_nodes_from(g.nodes)
    for u, v, k, data in g.edges(keys=True, data=True):
        gr.add_edge(u, v, length=graphs._length(data["geom"]))
    return g, ns, gr


def test_mock_betweenness_and_harmonic_vs_networkx(mock):
    g, ns, gr = mock
    d, b, s = _thr([5000])
    out, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, ns=ns)
    keys = ns.node_keys_py()
    bc = nx.betweenness_centrality(gr, normalized=False, weight="length")
    hc = nx.harmonic_centrality(gr, distance="length")
    for i, k in enumerate(keys):
        assert abs(out[5, 0, i] - bc[k]) < 0.01
        assert abs(out[3, 0, i] - hc[k]) < 0.01
    assert set(np.unique(out[0, 0]).tolist()) <= {49.0, 3.0, 1.0, 0.0}


def test_mock_closeness_recomputed_from_networkx(mock):
    """test_centrality.py:247-341: closeness terms and circuit ranks rebuilt from nx distances."""
    g, ns, gr = mock
    betas = [0.02, 0.01, 0.005, 0.0008]
    dists = common.distances_from_betas(betas)
    d, b, s = _thr(dists)
    out, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, ns=ns, betweenness=False)
    keys = ns.node_keys_py()
    n = len(keys)
    dens = np.zeros((len(d), n))
    far = np.zeros((len(d), n))
    harm = np.zeros((len(d), n))
    grav = np.zeros((len(d), n))
    cyc = np.zeros((len(d), n))
    for si, sk in enumerate(keys):
        dist = nx.single_source_dijkstra_path_length(gr, sk, weight="length")
        score = np.zeros(len(d))
        for di, cut in enumerate(d):
            inside = {k for k, v in dist.items() if v <= cut}
            edges = {tuple(sorted((u, v))) + (kk,) for u, v, kk in g.edges(keys=True)
                     if u != v and u in inside and v in inside}
            if inside:
                score[di] = max(0, len(edges) - len(inside) + 1)
        for tk, dv in dist.items():
            if tk == sk:
                continue
            ti = keys.index(tk)
            for di, cut in enumerate(d):
                if dv <= cut:
                    dens[di, si] += 1
                    far[di, si] += dv
                    harm[di, si] += 1 / dv
                    grav[di, si] += np.exp(-betas[di] * dv)
                    cyc[di, ti] += score[di]
    for di in range(len(d)):
        for arr, m in ((dens, 0), (far, 1), (cyc, 2), (harm, 3), (grav, 4)):
            assert np.allclose(out[m, di], arr[di], atol=0.01, rtol=1e-4), (m, di)


def test_mock_dual_routes():
    """Simplest routes keep to the periphery; shortest cut through; no sidesteps
    (test_centrality.py:166-234)."""
    g = mock_graph()
    nodes, _, nsd = _dual_of(g)
    keys = nodes["index"]
    og = oracle.OracleGraph(nsd)
    paths = FIX["centrality"]["dual_paths"]

    def route(tree, src, tgt):
        out = [tgt]
        while out[-1] != src:
            out.append(int(tree["pred"][out[-1]]))
        return [keys[i] for i in reversed(out)]

    maxs = int(5000 / SPEED)
    src, tgt = keys.index("11_6_k0"), keys.index("39_40_k0")
    _, t_simpl = oracle.tree_simplest(og, src, maxs, SPEED)
    assert route(t_simpl, src, tgt) == paths[0]["path"]
    _, t_short = oracle.tree_shortest(og, src, maxs, SPEED)
    assert route(t_short, src, tgt) == paths[1]["path"]
    src2, tgt2 = keys.index("10_43_k0"), keys.index("10_5_k0")
    _, t2 = oracle.tree_simplest(og, src2, maxs, SPEED)
    assert route(t2, src2, tgt2) == paths[2]["path"]


def test_mock_trees_vs_networkx(mock):
    g, ns, gr = mock
    og = oracle.OracleGraph(ns)
    keys = ns.node_keys_py()
    for max_dist in (0, 500, 2000, 5000):
        for si, sk in enumerate(keys):
            _, tree = oracle.tree_shortest(og, si, int(max_dist / SPEED), SPEED)
            nd = nx.single_source_dijkstra_path_length(gr, sk, weight="length", cutoff=max_dist)
            for tk, dv in nd.items():
                ti = keys.index(tk)
                assert abs(tree["short_dist"][ti] - dv) < 0.01


def test_plateau_ratio():
    g = nx_from_spec(FIX["helpers"]["make_angular_plateau_graph"])
    nodes, _, nsd = _dual_of(g)
    d, b, s = _thr([1000])
    out, _ = oracle.centrality_simplest(oracle.OracleGraph(nsd), d, b, s, ns=nsd, closeness=False)
    betw = dict(zip(nodes["index"], out[3, 0]))
    assert np.isclose(betw["B_C_k0"] / betw["C_D_k0"], 1.8, atol=1e-6)


def test_tolerance_drift_clears_stale_predecessors():
    from cityseer_gb300.centrality import prepare_source_sampling, validate_tolerance

    g = nx_from_spec(FIX["helpers"]["make_tolerance_drift_graph"])
    nodes, _, ns = io.network_structure_from_nx(g)
    idx = {k: i for i, k in enumerate(nodes["index"])}
    d, b, s = _thr([20])
    og = oracle.OracleGraph(ns)
    sp = prepare_source_sampling(ns, None, None, None, [idx["S"]])
    plan = oracle.plan_from(sp, ns.node_bound())
    exact, _ = oracle.centrality_shortest(og, d, b, s, tol=validate_tolerance(0.0), closeness=False, plan=plan)
    tol, _ = oracle.centrality_shortest(og, d, b, s, tol=validate_tolerance(10.0), closeness=False, plan=plan)
    e = {k: exact[5, 0, i] for k, i in idx.items()}
    t = {k: tol[5, 0, i] for k, i in idx.items()}
    assert np.isclose(e["A"], 0.0, atol=0.01) and np.isclose(e["B"], 0.0, atol=0.01) and e["C"] > 0
    assert np.isclose(t["A"], 0.0, atol=0.01) and t["B"] > 0 and t["C"] > 0
