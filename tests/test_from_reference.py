"""NetworkStructure.from_reference: import of a reference NetworkStructure through its public getters.

The reference cannot be imported here, so a stand-in exposes the same getters (node_indices,
get_node_payload_py, edge_references, get_edge_payload_py with the edge's WKT, is_dual) over a graph
ingested from networkx; the import must reproduce the graph store exactly, including the dual
endpoint slots recovered from the geometries, and the oracle's centralities on it."""
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common
from cityseer_gb300.graph import NetworkStructure
from cityseer_gb300.tools import graphs, io
from cityseer_gb300.tools.graphs import align_linestring_coords, coords_of
from helpers import mock_graph


class _Stand_in:
    def __init__(self, g, ns):
        self.g, self.ns = g, ns

    @property
    def is_dual(self):
        return self.ns.is_dual

    def node_indices(self):
        return self.ns.node_indices()

    def get_node_payload_py(self, i):
        return self.ns.get_node_payload_py(i)

    def edge_references(self):
        return self.ns.edge_references()

    def get_edge_payload_py(self, s, e, k):
        pl = self.ns.get_edge_payload_py(s, e, k)
        a, b = pl.start_nd_key_py, pl.end_nd_key_py
        xy = (self.g.nodes[a]["x"], self.g.nodes[a]["y"])
        c = align_linestring_coords(coords_of(self.g[a][b][k]["geom"]), xy)
        pl.geom_wkt = "LINESTRING (" + ", ".join(f"{p[0]!r} {p[1]!r}" for p in c) + ")"
        return pl


def _same_store(a, b):
    x, y = a.arrays(), b.arrays()
    assert set(x) == set(y)
    for k in x:
        np.testing.assert_array_equal(np.asarray(x[k]), np.asarray(y[k]), err_msg=k)
    assert a.node_keys_py() == b.node_keys_py() and a.node_indices() == b.node_indices()


def test_primal_import_is_exact():
    g = mock_graph()
    _, _, ns = io.network_structure_from_nx(g)
    imp = NetworkStructure.from_reference(_Stand_in(g, ns))
    _same_store(ns, imp)
    d, b, s = common.pair_distances_betas_time(1.33333, distances=[500, 2000])
    r0, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, ns=ns)
    r1, _ = oracle.centrality_shortest(oracle.OracleGraph(imp), d, b, s, ns=imp)
    np.testing.assert_array_equal(r0, r1)


def test_dual_import_recovers_endpoint_slots():
    g = graphs.nx_to_dual(mock_graph())
    _, _, ns = io.network_structure_from_nx(g)
    imp = NetworkStructure.from_reference(_Stand_in(g, ns))
    assert imp.is_dual
    _same_store(ns, imp)  # e_shared: the same equality classes, numbered in the same order
    og0, og1 = oracle.OracleGraph(ns), oracle.OracleGraph(imp)
    assert og1.slots_ok
    np.testing.assert_array_equal(og0.slots(), og1.slots())
    d, b, s = common.pair_distances_betas_time(1.33333, distances=[400, 1200])
    r0, _ = oracle.centrality_simplest(og0, d, b, s, ns=ns)
    r1, _ = oracle.centrality_simplest(og1, d, b, s, ns=imp)
    np.testing.assert_array_equal(r0, r1)


def test_gaps_keep_indices():
    g = mock_graph()
    _, _, ns = io.network_structure_from_nx(g)
    for v in (3, 17, 18):
        ns.remove_street_node(v)
    imp = NetworkStructure.from_reference(_Stand_in(g, ns))
    assert imp.node_indices() == ns.node_indices() and imp.node_bound() == ns.node_bound()
    d, b, s = common.pair_distances_betas_time(1.33333, distances=[800])
    r0, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, ns=ns)
    r1, _ = oracle.centrality_shortest(oracle.OracleGraph(imp), d, b, s, ns=imp)
    np.testing.assert_array_equal(r0, r1)


def test_dual_without_geometry_is_refused():
    g = graphs.nx_to_dual(mock_graph())
    _, _, ns = io.network_structure_from_nx(g)
    with pytest.raises(ValueError, match="geom_wkt"):
        NetworkStructure.from_reference(ns)  # this store keeps no geometry
