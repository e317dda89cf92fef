"""networkx -> NetworkStructure ingest (pysrc/cityseer/tools/io.py:1018-1210), without geopandas.

Returns (nodes, edges, NetworkStructure) where nodes/edges are plain dict-of-lists frames
(column name -> list) indexed like the reference's GeoDataFrames.
"""
from __future__ import annotations

import networkx as nx

from ..graph import NetworkStructure
from .graphs import align_linestring_coords, coords_of


def network_structure_from_nx(g: nx.MultiGraph):
    ns = NetworkStructure()
    ns.set_is_dual(bool(g.graph.get("is_dual", False)))
    node_rows: dict[str, tuple] = {}
    for key, data in g.nodes(data=True):
        if not isinstance(key, str):
            raise TypeError(f"Node key must be of type string but encountered {type(key)}")
        live = bool(data.get("live", True))
        weight = data.get("weight", 1)
        idx = ns.add_street_node(key, data["x"], data["y"], live, weight, z=data.get("z"))
        node_rows[key] = (idx, data["x"], data["y"], data.get("z"), live, weight)
    edge_rows = {}
    for s in g.nodes():
        s_idx, sx, sy = node_rows[s][:3]
        for e in g.neighbors(s):
            e_idx = node_rows[e][0]
            for k, data in g[s][e].items():
                geom = data.get("geom")
                if geom is None:
                    raise ValueError(f"Edge has no geometry: start_node={s}, end_node={e}, edge_idx={k}")
                coords = align_linestring_coords(coords_of(geom), (sx, sy))
                ei = ns.add_street_edge_coords(s_idx, e_idx, int(k), s, e, coords,
                                               float(data.get("imp_factor", 1.0)),
                                               shared_primal_node_key=data.get("primal_node_id"))
                edge_rows[f"{s}-{e}"] = (ei, s_idx, e_idx, k, s, e)
    ns.validate()
    nodes = {"index": list(node_rows), "ns_node_idx": [r[0] for r in node_rows.values()],
             "x": [r[1] for r in node_rows.values()], "y": [r[2] for r in node_rows.values()],
             "live": [r[4] for r in node_rows.values()], "weight": [r[5] for r in node_rows.values()]}
    if g.graph.get("is_dual"):
        for col in ("primal_edge_node_a", "primal_edge_node_b", "primal_edge_idx"):
            nodes[col] = [g.nodes[k].get(col) for k in node_rows]
    edges = {"index": list(edge_rows), "ns_edge_idx": [r[0] for r in edge_rows.values()],
             "start_ns_node_idx": [r[1] for r in edge_rows.values()],
             "end_ns_node_idx": [r[2] for r in edge_rows.values()]}
    return nodes, edges, ns
