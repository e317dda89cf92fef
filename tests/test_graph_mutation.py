"""Graph store robustness after removals (the reference's tests/test_graph_mutation.py): removed nodes
and edges are rejected with the reference's ValueError messages, before any GPU work."""
import pytest

from cityseer_gb300.tools import io
from helpers import mock_graph


@pytest.fixture
def ns():
    return io.network_structure_from_nx(mock_graph())[2]


def test_removed_node_is_rejected_by_setters_and_getters(ns):
    v = ns.street_node_indices()[0]
    ns.remove_street_node(v)
    with pytest.raises(ValueError, match="does not exist"):
        ns.set_node_live(v, True)
    for get in (ns.get_node_payload_py, ns.get_node_weight, ns.is_node_live):
        with pytest.raises(ValueError, match="node_idx .* does not exist"):
            get(v)


@pytest.mark.parametrize("closeness,betweenness", [(True, False), (False, True)])
def test_removed_source_index_is_rejected(ns, closeness, betweenness):
    v = ns.street_node_indices()[0]
    ns.remove_street_node(v)
    with pytest.raises(ValueError, match="does not exist"):
        ns.centrality_shortest(compute_closeness=closeness, compute_betweenness=betweenness, distances=[500],
                               source_indices=[v], sample_probability=1.0, pbar_disabled=True)


def test_add_edge_to_a_removed_endpoint_is_rejected(ns):
    a, b = ns.street_node_indices()[:2]
    pa, pb = ns.get_node_payload_py(a), ns.get_node_payload_py(b)
    wkt = f"LINESTRING({pa.coord[0]} {pa.coord[1]}, {pb.coord[0]} {pb.coord[1]})"
    ns.remove_street_node(b)
    with pytest.raises(ValueError, match="end_nd_idx .* does not exist"):
        ns.add_street_edge(a, b, 999999, pa.node_key, pb.node_key, wkt)


def test_removed_edge_getters(ns):
    s, e, k = ns.edge_references()[0]
    pl = ns.get_edge_payload_py(s, e, k)
    assert pl.edge_idx == k and pl.length > 0 and pl.imp_factor == 1.0 and not pl.is_transport
    ns.remove_street_edge(s, e, k)
    for get in (ns.get_edge_payload_py, ns.get_edge_length, ns.get_edge_impedance):
        with pytest.raises(ValueError, match="Edge not found"):
            get(s, e, k)


def test_remove_edge_with_a_removed_endpoint(ns):
    s, e, k = ns.edge_references()[0]
    ns.remove_street_node(s)
    with pytest.raises(ValueError, match="start_nd_idx .* does not exist"):
        ns.remove_street_edge(s, e, k)


def test_simplest_wrappers_require_a_dual_graph(ns):
    """tests/metrics/test_networks.py:247-261 (raised before any GPU work)."""
    from cityseer_gb300.metrics import networks

    for fn in (networks.closeness_simplest, networks.betweenness_simplest, networks.node_centrality_simplest):
        with pytest.raises(ValueError, match="dual graph"):
            fn(ns, {}, distances=[200, 400])


def test_remaining_getters_and_compatibility_methods():
    """street_node_lives, node_zs, node_xyzs (rust/src/graph.rs:660-696); barriers and the edge
    R-tree are accepted and do not change centrality inputs."""
    import networkx as nx

    from cityseer_gb300.tools import graphs

    g = nx.MultiGraph()
    g.add_node("a", x=0.0, y=0.0, z=3.0)
    g.add_node("b", x=100.0, y=0.0)
    g.add_edge("a", "b")
    ns = io.network_structure_from_nx(graphs.nx_simple_geoms(g))[2]
    assert ns.node_zs == [3.0, None]
    assert ns.node_xyzs == [(0.0, 0.0, 3.0), (100.0, 0.0, None)]
    assert ns.street_node_lives == [True, True]
    import numpy as np

    before = {k: np.copy(v) for k, v in ns.arrays().items()}
    ns.build_edge_rtree()
    ns.set_barriers(["LINESTRING (50 -10, 50 10)"])
    ns.unset_barriers()
    for k, v in ns.arrays().items():
        np.testing.assert_array_equal(v, before[k], err_msg=k)  # NaN z compares equal here
