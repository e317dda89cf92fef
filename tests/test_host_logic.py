"""Host logic of the drop-in (no GPU): sampling plan, tolerance, graph store, CSR builder."""
import numpy as np
import pytest

from cityseer_gb300 import NetworkStructure, device, synth
from cityseer_gb300.centrality import prepare_source_sampling, validate_tolerance


def small():
    p, _ = synth.lattice_config("c1", side=6)
    return synth.primal_structure(p)


def test_validate_tolerance():
    assert validate_tolerance(None) == pytest.approx(1e-4)
    assert validate_tolerance(0.0) == pytest.approx(1e-4)
    assert validate_tolerance(10.0) == pytest.approx(0.1)
    with pytest.raises(ValueError, match="between 0 and 100"):
        validate_tolerance(101.0)
    with pytest.raises(ValueError, match="between 0 and 100"):
        validate_tolerance(-1.0)


def test_sampling_plan_semantics():
    ns = small()
    n = ns.node_count()
    sp = prepare_source_sampling(ns, None, None, None, None)
    assert len(sp.process) == n and sp.eligible.all() and not sp.is_source_indexed
    sp = prepare_source_sampling(ns, 0.5, None, None, [0, 3, 5])
    assert sp.process.tolist() == [0, 3, 5] and sp.sampled_count == 3
    assert np.all(sp.src_wt[[0, 3, 5]] == np.float32(2.0)) and sp.eligible.sum() == 3
    sp = prepare_source_sampling(ns, 0.5, None, 7, None)
    assert 0 < sp.sampled_count < n and np.all(sp.src_wt[sp.process] == np.float32(2.0))
    sp = prepare_source_sampling(ns, 1.0, np.zeros(n, np.float32), 7, None)
    assert sp.sampled_count == 0
    with pytest.raises(ValueError, match="mutually exclusive"):
        prepare_source_sampling(ns, None, np.ones(n), None, [0])
    with pytest.raises(ValueError, match=r"\(0.0, 1.0\]"):
        prepare_source_sampling(ns, 1.5, None, None, None)
    with pytest.raises(ValueError, match="out of range"):
        prepare_source_sampling(ns, 0.5, np.full(n, 2.0), None, None)
    with pytest.raises(ValueError, match="must match node_count"):
        prepare_source_sampling(ns, 0.5, np.ones(n + 3), None, None)
    with pytest.raises(ValueError, match="does not exist"):
        prepare_source_sampling(ns, None, None, None, [n + 10])


def test_non_live_nodes_are_not_sources():
    ns = small()
    ns.set_node_live(2, False)
    sp = prepare_source_sampling(ns, None, None, None, None)
    assert 2 not in sp.process.tolist() and sp.eligible[2] == 0 and sp.n_live == ns.node_count() - 1


def test_graph_builder_and_mutation():
    ns = NetworkStructure()
    a = ns.add_street_node("a", 0.0, 0.0, True, 1.0)
    b = ns.add_street_node("b", 100.0, 0.0, True, 1.0)
    c = ns.add_street_node("c", 100.0, 100.0, True, 1.0)
    ns.add_street_edge(a, b, 0, "a", "b", "LINESTRING (0 0, 100 0)")
    ns.add_street_edge(b, a, 0, "b", "a", "LINESTRING (100 0, 0 0)")
    ns.add_street_edge(b, c, 0, "b", "c", "LINESTRING (100 0, 100 50, 100 100)")
    assert ns.get_edge_length(a, b, 0) == pytest.approx(100.0)
    assert ns.edge_count == 3 and ns.node_bound() == 3
    with pytest.raises(ValueError, match="does not exist"):
        ns.add_street_edge(a, 9, 0, "a", "x", "LINESTRING (0 0, 1 1)")
    with pytest.raises(ValueError, match="Invalid street node payload"):
        ns.add_street_node("d", 0, 0, True, -1.0)
    with pytest.raises(ValueError, match="Impedance"):
        ns.add_street_edge(a, b, 1, "a", "b", "LINESTRING (0 0, 100 0)", imp_factor=0.0)
    ns.remove_street_node(b)
    assert ns.node_indices() == [0, 2] and ns.node_count() == 2 and ns.node_bound() == 3
    assert ns.edge_count == 0
    with pytest.raises(ValueError, match="does not exist"):
        ns.remove_street_node(b)
    with pytest.raises(ValueError, match="dual graph"):
        ns.validate_dual_for_angular("centrality_simplest")


def test_angle_sum_and_length_from_geometry():
    ns = NetworkStructure()
    a = ns.add_street_node(0, 0.0, 0.0, True, 1.0)
    b = ns.add_street_node(1, 20.0, 0.0, True, 1.0)
    ns.add_street_edge(a, b, 0, 0, 1, "LINESTRING (0 0, 10 0, 10 10, 20 10, 20 0)")
    arr = ns.arrays()
    assert arr["e_ang"][0] == np.float32(270.0)
    assert arr["e_len"][0] == np.float32(40.0)


def test_csr_builder_orders_and_flags():
    ns = small()
    h = device.PrimalHost(ns)
    a = ns.arrays()
    n = ns.node_bound()
    in_ptr, in_nb = h.h["in_ptr"], h.h["in_nb"]
    # in-CSR: per node, edges v->u newest first (petgraph Incoming order)
    for u in range(n):
        slots = [e for e in range(len(a["e_src"])) if a["e_dst"][e] == u]
        assert in_nb[in_ptr[u]:in_ptr[u + 1]].tolist() == [int(a["e_src"][e]) for e in reversed(slots)]
    # circuit-rank flags: exactly one directed edge per undirected street
    assert int(h.h["out_cnt"].sum()) == len(a["e_src"]) // 2
    assert not h.has_missing_reverse
    assert np.allclose(h.h["in_seglen"], a["e_len"][h.in_order])


def test_synthetic_lattices_are_connected():
    import networkx as nx

    for name, side in (("c1", 20), ("c2", 20), ("c3", 12)):
        p, _ = synth.lattice_config(name, side=side)
        g = nx.Graph()
        g.add_nodes_from(range(len(p.x)))
        g.add_edges_from(zip(p.u.tolist(), p.v.tolist()))
        assert nx.is_connected(g), name
    p, _ = synth.lattice_config("c3", side=12)
    nsd = synth.dual_structure(p)
    assert nsd.is_dual and nsd.node_count() == len(p.u)
    assert all(k is not None for k in nsd._e_shared)


def test_dual_endpoint_slots_match_oracle():
    import oracle
    from cityseer_gb300 import dual

    p, _ = synth.lattice_config("c3", side=10)
    ns = synth.dual_structure(p)
    a = ns.arrays()
    ex = np.nonzero(a["e_exists"])[0]
    src, dst, key = (a["e_src"][ex].astype(np.int64), a["e_dst"][ex].astype(np.int64),
                     a["e_shared"][ex].astype(np.int64))
    es, en = dual.endpoint_slots(src, dst, key, ns.node_bound())
    slots = oracle.OracleGraph(ns).slots()
    for e in range(len(ex)):
        assert slots[src[e], es[e]] == key[e]
        assert slots[dst[e], en[e]] == key[e]


def test_sampling_probability_schedule():
    from cityseer_gb300 import sampling

    assert sampling.compute_distance_p(1000) == 1.0
    assert sampling.compute_distance_p(0) == 1.0
    p5 = sampling.compute_distance_p(5000)
    p20 = sampling.compute_distance_p(20000)
    # pysrc/cityseer/metrics/networks.py:17-23 table, eps = 0.06: 58.7% at 5 km, 4.6% at 20 km
    assert round(p5 * 100, 1) == 58.7 and round(p20 * 100, 1) == 4.6
    assert sampling.compute_hoeffding_p(float("nan")) == 1.0
