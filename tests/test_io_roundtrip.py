"""The circular workflow of the reference (pysrc/cityseer/tools/io.py:1213-1321): the frames that
network_structure_from_nx returns rebuild the same NetworkStructure, primal and dual."""
import networkx as nx
import numpy as np
import pytest

from cityseer_gb300.tools import graphs, io
from helpers import diamond_graph


def _grid():
    g = nx.MultiGraph()
    for i in range(5):
        for j in range(4):
            g.add_node(f"{i}_{j}", x=100.0 * i + 3.0 * j, y=80.0 * j, live=(i + j) % 5 != 0, weight=1.0 + 0.1 * i)
            if i:
                g.add_edge(f"{i - 1}_{j}", f"{i}_{j}", imp_factor=1.0 + 0.05 * j)
            if j:
                g.add_edge(f"{i}_{j - 1}", f"{i}_{j}")
    return graphs.nx_simple_geoms(g)


@pytest.mark.parametrize("dual", [False, True])
def test_frames_rebuild_the_same_structure(dual):
    for g in (_grid(), diamond_graph()):
        if dual:
            g = graphs.nx_to_dual(g)
        nodes, edges, ns = io.network_structure_from_nx(g)
        ns2 = io.network_structure_from_gpd(nodes, edges)
        ns2.set_is_dual(ns.is_dual)
        a, b = ns.arrays(), ns2.arrays()
        for k in a:
            np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]), err_msg=k)
        assert ns2.node_keys_py() == ns.node_keys_py()


def test_missing_columns_are_reported():
    nodes, edges, _ = io.network_structure_from_nx(_grid())
    with pytest.raises(ValueError, match="nodes GDF: weight"):
        io.network_structure_from_gpd({k: v for k, v in nodes.items() if k != "weight"}, edges)
    with pytest.raises(ValueError, match="edges GDF: imp_factor"):
        io.network_structure_from_gpd(nodes, {k: v for k, v in edges.items() if k != "imp_factor"})


def test_frames_back_to_networkx_with_metrics():
    """network_structure_from_nx -> frames (+ a cc_* column) -> nx_from_cityseer_geopandas -> the same
    graph, and the ingest of that graph gives the same store."""
    g = _grid()
    nodes, edges, ns = io.network_structure_from_nx(g)
    nodes["cc_density_400"] = np.arange(len(nodes["index"]), dtype=float)
    g2 = io.nx_from_cityseer_geopandas(nodes, edges)
    assert sorted(g2.nodes) == sorted(g.nodes) and g2.number_of_edges() == g.number_of_edges()
    for i, key in enumerate(nodes["index"]):
        assert g2.nodes[key]["cc_density_400"] == i
        assert g2.nodes[key]["live"] == g.nodes[key]["live"]
    ns2 = io.network_structure_from_nx(g2)[2]
    for k, v in ns.arrays().items():
        np.testing.assert_array_equal(np.asarray(v), np.asarray(ns2.arrays()[k]), err_msg=k)
