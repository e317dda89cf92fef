"""OD-weighted betweenness (rust/src/centrality.rs:2419-2540): the origin-destination matrix on the
host, and the oracle's restatement pinned two ways -- against its own shortest-path betweenness
(pinned to networkx on the reference's mock graph) and against networkx shortest paths directly."""
import networkx as nx
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common
from cityseer_gb300.centrality import OdMatrix
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph

SPEED = 1.33333


def test_od_matrix_construction():
    # tests/test_sampling.py:668-675
    od = OdMatrix([0, 0, 1], [1, 2, 2], [1.0, 2.0, 3.0])
    assert od.len() == 3
    assert od.n_origins() == 2


def test_od_matrix_last_weight_wins_and_rows():
    od = OdMatrix([3, 1, 3, 1, 9], [2, 0, 2, 4, 1], [1.0, 2.0, 7.5, 0.25, 1.0])
    assert od.len() == 4 and od.n_origins() == 3
    ptr, dst, w = od.rows(5)  # origin 9 lies beyond the node bound: no row
    assert ptr.tolist() == [0, 0, 2, 2, 3, 3]
    assert dst.tolist() == [0, 4, 2]
    assert w.tolist() == [2.0, 0.25, 7.5]
    with pytest.raises(ValueError, match="must have equal length"):
        OdMatrix([0, 1], [1], [1.0, 1.0])


@pytest.fixture(scope="module")
def mock():
    g = mock_graph()
    _, _, ns = io.network_structure_from_nx(g)
    gr = nx.Graph()
    gr.add_nodes_from(g.nodes)
    for u, v, k, data in g.edges(keys=True, data=True):
        gr.add_edge(u, v, length=graphs._length(data["geom"]))
    return g, ns, gr


def _all_pairs(ns, w=1.0):
    idx = ns.node_indices()
    o = [a for a in idx for b in idx if a != b]
    d = [b for a in idx for b in idx if a != b]
    return OdMatrix(o, d, [w] * len(o))


def test_oracle_all_pairs_is_twice_pair_counted_betweenness(mock):
    """Every ordered pair with weight 1 seeds each target with 1.0 where centrality_shortest seeds
    0.5 (all nodes eligible), so the OD rows are exactly twice the shortest-path betweenness rows."""
    _, ns, _ = mock
    og = oracle.OracleGraph(ns)
    d, b, s = common.pair_distances_betas_time(SPEED, distances=[200, 800, 5000])
    short, _ = oracle.centrality_shortest(og, d, b, s, ns=ns, closeness=False)
    od = oracle.betweenness_od(og, d, b, s, _all_pairs(ns).rows(ns.node_bound()), ns=ns)
    np.testing.assert_array_equal(od[0], 2.0 * short[5])
    np.testing.assert_array_equal(od[1], 2.0 * short[6])
    assert od[0, 2].max() > 0


def test_oracle_single_pairs_vs_networkx(mock):
    """One pair (o, t) of weight w credits w to every node strictly inside the o -> t shortest path
    (and w exp(-beta d) in the beta row), when the path is unique and within the threshold."""
    _, ns, gr = mock
    og = oracle.OracleGraph(ns)
    keys = ns.node_keys_py()
    rng = np.random.default_rng(5)
    d, b, s = common.pair_distances_betas_time(SPEED, distances=[5000])
    checked = 0
    for _ in range(40):
        oi, ti = rng.choice(len(keys), 2, replace=False)
        if not nx.has_path(gr, keys[oi], keys[ti]):
            continue
        paths = list(nx.all_shortest_paths(gr, keys[oi], keys[ti], weight="length"))
        if len(paths) != 1:
            continue
        w = float(rng.uniform(0.5, 4.0))
        od = OdMatrix([oi], [ti], [w])
        out = oracle.betweenness_od(og, d, b, s, od.rows(ns.node_bound()), ns=ns)
        want = np.zeros(len(keys))
        inner = [keys.index(k) for k in paths[0][1:-1]]
        want[inner] = np.float32(w)
        np.testing.assert_allclose(out[0, 0], want, rtol=1e-12, atol=0)
        dist = nx.shortest_path_length(gr, keys[oi], keys[ti], weight="length")
        wantb = np.zeros(len(keys))
        wantb[inner] = np.float32(w) * np.exp(-b[0] * dist)
        np.testing.assert_allclose(out[1, 0], wantb, rtol=1e-5, atol=0)
        checked += 1
    assert checked >= 20


def test_oracle_zero_weights(mock):
    # tests/test_sampling.py:708-724
    _, ns, _ = mock
    og = oracle.OracleGraph(ns)
    idx = ns.node_indices()
    d, b, s = common.pair_distances_betas_time(SPEED, distances=[500])
    od = OdMatrix([idx[0], idx[1]], [idx[1], idx[2]], [0.0, 0.0])
    out = oracle.betweenness_od(og, d, b, s, od.rows(ns.node_bound()), ns=ns)
    assert np.all(out == 0.0)
