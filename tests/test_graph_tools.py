"""Graph tools against the reference's own checks (tests/tools/test_graphs.py:548-700): the dual of
the diamond graph (5 dual nodes, 8 dual edges, degrees, 100 m welded geometries, bearings and shared
primal nodes per pair) and nx_decompose (lengths preserved, pieces no longer than the maximum)."""
import math

import networkx as nx
import numpy as np
import pytest

from cityseer_gb300.tools import graphs
from helpers import diamond_graph, mock_graph

# (dual edge from -> to): (in bearing, out bearing, shared primal node), tests/tools/test_graphs.py:660-700
EXPECTED = {
    ("0_1_k0", "0_2_k0"): (-60, 60, "0"),
    ("0_1_k0", "1_2_k0"): (120, 0, "1"),
    ("0_1_k0", "1_3_k0"): (120, 60, "1"),
    ("0_2_k0", "1_2_k0"): (60, 180, "2"),
    ("0_2_k0", "2_3_k0"): (60, 120, "2"),
    ("1_2_k0", "1_3_k0"): (180, 60, "1"),
    ("1_2_k0", "2_3_k0"): (0, 120, "2"),
    ("1_3_k0", "2_3_k0"): (60, -60, "3"),
}


def test_diamond_dual():
    g = diamond_graph()
    gd = graphs.nx_to_dual(g)
    assert gd.number_of_nodes() == 5 and gd.number_of_edges() == 8
    for n, d in gd.nodes(data=True):
        assert nx.degree(gd, n) == (4 if n == "1_2_k0" else 3)
        pg = graphs.coords_of(g[d["primal_edge_node_a"]][d["primal_edge_node_b"]][d["primal_edge_idx"]]["geom"])
        assert [tuple(c) for c in graphs.coords_of(d["primal_edge"])] == [tuple(c) for c in pg]
    for (a, b), (inb, outb, shared) in EXPECTED.items():
        (d,) = gd[a][b].values()
        c = graphs.coords_of(d["geom"])
        assert round(graphs._length(c)) == 100
        if (gd.nodes[a]["x"], gd.nodes[a]["y"]) != tuple(c[0][:2]):
            c = c[::-1]
        (sx, sy), (mx, my), (ex, ey) = c[0][:2], c[1][:2], c[-1][:2]
        got = (round(math.degrees(math.atan2(my - sy, mx - sx))), round(math.degrees(math.atan2(ey - my, ex - mx))))
        assert got == (inb, outb), (a, b, got)
        assert d["primal_node_id"] == shared
        assert shared in (gd.nodes[b]["primal_edge_node_a"], gd.nodes[b]["primal_edge_node_b"])


def test_dual_requires_geometries():
    g = diamond_graph()
    del g["0"]["1"][0]["geom"]
    with pytest.raises(KeyError):
        graphs.nx_to_dual(g)


def test_decompose_preserves_length_and_caps_pieces():
    g = mock_graph()
    gd = graphs.nx_decompose(g, 50)
    total = sum(graphs._length(graphs.coords_of(d["geom"])) for _, _, d in g.edges(data=True))
    total_d = sum(graphs._length(graphs.coords_of(d["geom"])) for _, _, d in gd.edges(data=True))
    assert np.isclose(total, total_d, atol=0.01, rtol=1e-4)
    assert all(graphs._length(graphs.coords_of(d["geom"])) <= 50 + 1e-6 for _, _, d in gd.edges(data=True))
    assert gd.number_of_nodes() > g.number_of_nodes()


# edge payloads on the diamond graph (tests/tools/test_io.py:300-520):
# (start, end): (length, angle_sum, imp_factor, in_bearing, out_bearing)
PRIMAL_PAYLOADS = {
    ("0", "1"): (100.0, 0.0, 1.0, 120.0, 120.0), ("0", "2"): (100.0, 0.0, 1.0, 60.0, 60.0),
    ("1", "0"): (100.0, 0.0, 1.0, -60.0, -60.0), ("1", "2"): (100.0, 0.0, 1.0, 0.0, 0.0),
    ("1", "3"): (100.0, 0.0, 1.0, 60.0, 60.0), ("2", "0"): (100.0, 0.0, 1.0, -120.0, -120.0),
    ("2", "1"): (100.0, 0.0, 1.0, 180.0, 180.0), ("2", "3"): (100.0, 0.0, 1.0, 120.0, 120.0),
    ("3", "1"): (100.0, 0.0, 1.0, -120.0, -120.0), ("3", "2"): (100.0, 0.0, 1.0, -60.0, -60.0),
}
DUAL_PAYLOADS = {
    ("0_1_k0", "0_2_k0"): (100.0, 120.0, 1.0, -60.0, 60.0), ("0_1_k0", "1_2_k0"): (100.0, 120.0, 1.0, 120.0, 0.0),
    ("0_1_k0", "1_3_k0"): (100.0, 60.0, 1.0, 120.0, 60.0), ("0_2_k0", "0_1_k0"): (100.0, 120.0, 1.0, -120.0, 120.0),
    ("0_2_k0", "1_2_k0"): (100.0, 120.0, 1.0, 60.0, 180.0), ("0_2_k0", "2_3_k0"): (100.0, 60.0, 1.0, 60.0, 120.0),
    ("1_2_k0", "0_1_k0"): (100.0, 120.0, 1.0, 180.0, -60.0),
}


@pytest.mark.parametrize("dual", [False, True])
def test_diamond_edge_payloads(dual):
    from cityseer_gb300.tools import io

    g = diamond_graph()
    g.nodes["3"]["live"] = False
    if dual:
        g = graphs.nx_to_dual(g)
    nodes, edges, ns = io.network_structure_from_nx(g)
    assert ns.is_dual is dual and ns.edge_count == 2 * g.number_of_edges() and len(nodes["index"]) == ns.node_count()
    for v in ns.street_node_indices():
        p = ns.get_node_payload_py(v)
        i = nodes["index"].index(p.node_key)
        assert p.coord == (nodes["x"][i], nodes["y"][i]) and p.live == nodes["live"][i]
    want = DUAL_PAYLOADS if dual else PRIMAL_PAYLOADS
    seen = 0
    for s, e, k in ns.edge_references():
        pl = ns.get_edge_payload_py(s, e, k)
        row = edges["index"].index(f"{pl.start_nd_key_py}-{pl.end_nd_key_py}")
        assert (edges["start_ns_node_idx"][row], edges["end_ns_node_idx"][row], edges["edge_idx"][row]) == (s, e, k)
        assert np.isnan(pl.seconds)
        key = (pl.start_nd_key_py, pl.end_nd_key_py)
        if key in want:
            np.testing.assert_allclose((pl.length, pl.angle_sum, pl.imp_factor, pl.in_bearing, pl.out_bearing),
                                       want[key], atol=0.01, rtol=1e-4, err_msg=str(key))
            seen += 1
    assert seen == len(want)


def test_bearing_and_angle_helpers():
    """The geometry helpers behind edge bearings and angle sums, on the reference's known answers
    (tests/tools/test_util.py:14-86)."""
    from cityseer_gb300.graph import _bearing, _coords_angle, cumulative_angle

    for b, want in (((1, 0), 0), ((1, 1), 45), ((0, 1), 90), ((-1, 0), 180), ((-1, -1), -135), ((0, -1), -90),
                    ((1, -1), -45)):
        assert _bearing((0, 0), b) == want
    for coords, want in (([[0, 0], [1, 0], [2, 0]], 0), ([[0, 0], [1, 0], [2, 1]], 45),
                         ([[0, 0], [1, 0], [1, 1]], 90), ([[0, 0], [1, 0], [0, 1]], 135)):
        assert np.isclose(_coords_angle(*coords), want) and np.isclose(_coords_angle(*coords[::-1]), want)
        assert np.isclose(cumulative_angle(coords), want)
    assert np.isclose(cumulative_angle([[0, 0], [1, 0], [1, 1], [2, 1]]), 180)
