"""The host paths above the C-ABI (query building, threshold groups of 16, source plans, post-scale,
result objects, the sharded form's default share, OD rows) run on the CPU with the C-ABI calls
answered by the oracle.  The stand-in library is test infrastructure: it reads the query the host
built (sources, weights, eligibility, thresholds) from the pointers passed, runs the oracle on exactly
that, and writes the rows where the host asked.  The GPU parity tests cover the kernels themselves."""
import numpy as np
import pytest

import oracle
import standin
from cityseer_gb300 import synth
from cityseer_gb300.centrality import OdMatrix, prepare_source_sampling, validate_tolerance
from cityseer_gb300.common import pair_distances_betas_time
from cityseer_gb300.replicas import sharded_centrality_shortest
from cityseer_gb300.tools import io
from helpers import mock_graph


@pytest.fixture
def stand_in(monkeypatch):
    return standin.install(monkeypatch)


def _want(ns, dists, p=None, w=None, seed=None, src=None, closeness=True, betweenness=True, tol=None):
    sp = prepare_source_sampling(ns, p, w, seed, src)
    d, b, s = pair_distances_betas_time(1.33333, distances=dists)
    out, reach = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, tol=validate_tolerance(tol),
                                            closeness=closeness, betweenness=betweenness,
                                            plan=oracle.plan_from(sp, ns.node_bound()))
    return out, reach, sp


def test_shortest_host_path(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    lib = stand_in(ns)
    for kw in (dict(), dict(p=0.5, seed=4), dict(src=[1, 2, 3, 5, 8, 13]), dict(closeness=False),
               dict(betweenness=False, tol=5.0)):
        dists = [200, 800, 5000]
        want, reach, sp = _want(ns, dists, **kw)
        res = ns.centrality_shortest(distances=dists, sample_probability=kw.get("p"), random_seed=kw.get("seed"),
                                     source_indices=kw.get("src"), compute_closeness=kw.get("closeness", True),
                                     compute_betweenness=kw.get("betweenness", True), tolerance=kw.get("tol"))
        np.testing.assert_array_equal(res._data, want)
        if kw.get("p") or kw.get("src"):
            assert res.reachability_totals == [int(x) for x in reach]
            assert res.sampled_source_count == sp.sampled_count
    assert lib.calls == 5


def test_more_than_sixteen_thresholds_run_in_groups(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    lib = stand_in(ns)
    dists = list(range(100, 2100, 100))  # 20 thresholds: groups of 16 and 4
    res = ns.centrality_shortest(distances=dists)
    want, _, _ = _want(ns, dists)
    np.testing.assert_array_equal(res._data, want)
    assert lib.calls == 2


def test_sharded_default_share_equals_the_plain_call(stand_in):
    p, dists = synth.lattice_config("c1", side=12)
    ns = synth.primal_structure(p)
    stand_in(ns)
    plain = ns.centrality_shortest(distances=dists, source_indices=list(range(0, 144, 3)))
    shard = sharded_centrality_shortest(ns, distances=dists, source_indices=list(range(0, 144, 3)))
    np.testing.assert_array_equal(shard._data, plain._data)
    assert shard.reachability_totals == plain.reachability_totals


def test_sharded_simplest_default_share_equals_the_plain_call(stand_in):
    from cityseer_gb300.replicas import sharded_centrality_simplest
    from cityseer_gb300.tools import graphs

    ns = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    stand_in(ns)
    subset = ns.node_indices()[::4]
    plain = ns.centrality_simplest(distances=list(range(100, 2000, 100)), source_indices=subset)
    shard = sharded_centrality_simplest(ns, distances=list(range(100, 2000, 100)), source_indices=subset)
    np.testing.assert_array_equal(shard._data, plain._data)
    assert shard.reachability_totals == plain.reachability_totals


def test_sharded_segment_default_share_equals_the_plain_call(stand_in):
    from cityseer_gb300.replicas import sharded_segment_centrality

    ns = io.network_structure_from_nx(mock_graph())[2]
    stand_in(ns)
    dists = list(range(50, 1000, 50))
    np.testing.assert_array_equal(sharded_segment_centrality(ns, distances=dists)._data,
                                  ns.segment_centrality(distances=dists)._data)


def test_od_host_path(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    stand_in(ns)
    rng = np.random.default_rng(2)
    idx = np.asarray(ns.node_indices())
    od = OdMatrix(rng.choice(idx, 300).tolist(), rng.choice(idx, 300).tolist(), rng.uniform(0, 3, 300).tolist())
    res = ns.betweenness_od_shortest(od, distances=[300, 1200])
    d, b, s = pair_distances_betas_time(1.33333, distances=[300, 1200])
    want = oracle.betweenness_od(oracle.OracleGraph(ns), d, b, s, od.rows(ns.node_bound()), ns=ns)
    np.testing.assert_array_equal(res._data, want)


def test_simplest_host_path(stand_in):
    from cityseer_gb300.tools import graphs

    ns = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    lib = stand_in(ns)
    cases = (dict(), dict(p=0.5, seed=8), dict(src=[0, 4, 9, 16, 25, 36]), dict(asu=90.0, fso=2.0, closeness=True),
             dict(dists=list(range(100, 2000, 100))))
    for kw in cases:
        dists = kw.get("dists", [300, 1200])
        sp = prepare_source_sampling(ns, kw.get("p"), None, kw.get("seed"), kw.get("src"))
        d, b, s = pair_distances_betas_time(1.33333, distances=dists)
        want, reach = oracle.centrality_simplest(oracle.OracleGraph(ns), d, b, s, tol=validate_tolerance(None),
                                                 plan=oracle.plan_from(sp, ns.node_bound()),
                                                 asu=kw.get("asu", 180.0), fso=kw.get("fso", 1.0))
        res = ns.centrality_simplest(distances=dists, sample_probability=kw.get("p"), random_seed=kw.get("seed"),
                                     source_indices=kw.get("src"), angular_scaling_unit=kw.get("asu"),
                                     farness_scaling_offset=kw.get("fso"))
        np.testing.assert_array_equal(res._data, want)
        if kw.get("p") or kw.get("src"):
            assert res.reachability_totals == [int(x) for x in reach]
    assert lib.calls == 6  # 19 thresholds: two groups


def test_segment_host_path(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    ns.set_node_live(ns.node_indices()[3], False)
    lib = stand_in(ns)
    for dists in ([200, 600], list(range(50, 1000, 50))):
        res = ns.segment_centrality(distances=dists)
        d, b, s = pair_distances_betas_time(1.33333, distances=dists)
        np.testing.assert_array_equal(res._data, oracle.segment_centrality(oracle.OracleGraph(ns), d, b, s, ns=ns))
    assert lib.calls == 3


def test_od_host_path_more_than_sixteen_thresholds(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    lib = stand_in(ns)
    rng = np.random.default_rng(5)
    idx = np.asarray(ns.node_indices())
    od = OdMatrix(rng.choice(idx, 200).tolist(), rng.choice(idx, 200).tolist(), rng.uniform(0, 3, 200).tolist())
    dists = list(range(100, 2000, 100))
    res = ns.betweenness_od_shortest(od, distances=dists)
    d, b, s = pair_distances_betas_time(1.33333, distances=dists)
    want = oracle.betweenness_od(oracle.OracleGraph(ns), d, b, s, od.rows(ns.node_bound()), ns=ns)
    np.testing.assert_array_equal(res._data, want)
    assert lib.calls == 2


def test_tree_host_bookkeeping(stand_in):
    """dijkstra_tree_shortest / dijkstra_tree_segment host decoding and edge bookkeeping (visited
    edges, last and origin segments) from the kernel's rows, against the oracle for every source,
    including equal-distance ties (the stand-in's rows follow the oracle's settle order)."""
    import networkx as nx

    from cityseer_gb300.tools import graphs

    grid = nx.MultiGraph()  # a perfect 6 x 6 grid: equal edge lengths, many equal distances
    for i in range(6):
        for j in range(6):
            grid.add_node(f"{i}-{j}", x=100.0 * i, y=100.0 * j)
            if i:
                grid.add_edge(f"{i - 1}-{j}", f"{i}-{j}")
            if j:
                grid.add_edge(f"{i}-{j - 1}", f"{i}-{j}")
    for g in (mock_graph(), graphs.nx_simple_geoms(grid)):
        ns = io.network_structure_from_nx(g)[2]
        ns.remove_street_node(ns.node_indices()[7])
        stand_in(ns)
        og = oracle.OracleGraph(ns)
        for src in ns.node_indices():
            for max_seconds in (0, 200, 1500):
                vis, tree = ns.dijkstra_tree_shortest(src, max_seconds, 1.33333)
                vis_ref, t_ref = oracle.tree_shortest(og, src, max_seconds, 1.33333)
                assert vis == vis_ref.tolist()
                vis, vedges, tree, emap = ns.dijkstra_tree_segment(src, max_seconds, 1.33333)
                vis_ref, ve_ref, t_ref = oracle.tree_segment(og, src, max_seconds, 1.33333)
                assert vis == vis_ref.tolist() and vedges == ve_ref.tolist()
                for v in vis_ref:
                    assert np.float32(tree[v].agg_seconds) == t_ref["agg_seconds"][v]
                    assert (tree[v].pred if tree[v].pred is not None else -1) == t_ref["pred"][v]
                    assert (tree[v].last_seg if tree[v].last_seg is not None else -1) == t_ref["last_seg"][v]
                    assert (tree[v].origin_seg if tree[v].origin_seg is not None else -1) == t_ref["origin_seg"][v]
                for e in ve_ref:
                    assert emap[e].visited


@pytest.mark.parametrize("seed", range(6))
def test_randomised_host_calls(stand_in, seed):
    """Seeded random graphs, removals, liveness, thresholds (up to 20), flags, sampling and subsets:
    the public calls equal the oracle on the same plan."""
    rng = np.random.default_rng(100 + seed)
    p, _ = synth.lattice_config("c1", side=int(rng.integers(6, 12)))
    ns = synth.primal_structure(p)
    nb = ns.node_bound()
    for v in rng.choice(nb, 3, replace=False):
        ns.remove_street_node(int(v))
    idx = ns.node_indices()
    for v in rng.choice(idx, 4, replace=False):
        ns.set_node_live(int(v), False)
    stand_in(ns)
    k = int(rng.integers(1, 21))
    dists = sorted(int(x) for x in rng.choice(np.arange(100, 3000, 50), k, replace=False))
    closeness, betweenness = [(True, True), (True, False), (False, True)][seed % 3]
    kw = {}
    if seed % 2:
        kw = dict(sample_probability=float(rng.uniform(0.2, 0.9)), random_seed=int(rng.integers(0, 1 << 31)))
    elif seed % 3 == 0:
        kw = dict(source_indices=sorted(int(x) for x in rng.choice(idx, 15, replace=False)))
    res = ns.centrality_shortest(distances=dists, compute_closeness=closeness, compute_betweenness=betweenness, **kw)
    want, reach, sp = _want(ns, dists, p=kw.get("sample_probability"), seed=kw.get("random_seed"),
                            src=kw.get("source_indices"), closeness=closeness, betweenness=betweenness)
    np.testing.assert_array_equal(res._data, want)
    seg = ns.segment_centrality(distances=dists, compute_closeness=closeness, compute_betweenness=betweenness)
    d, b, s = pair_distances_betas_time(1.33333, distances=dists)
    np.testing.assert_array_equal(seg._data, oracle.segment_centrality(oracle.OracleGraph(ns), d, b, s,
                                                                       closeness=closeness,
                                                                       betweenness=betweenness, ns=ns))
