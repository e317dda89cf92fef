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
                imp = float(data.get("imp_factor", 1.0))
                shared = data.get("primal_node_id")
                ei = ns.add_street_edge_coords(s_idx, e_idx, int(k), s, e, coords, imp,
                                               shared_primal_node_key=shared)
                # keyed like the reference's frame (io.py:1149): parallel edges share a row, the last wins
                edge_rows[f"{s}-{e}"] = (ei, s_idx, e_idx, k, s, e, imp, coords, shared)
    ns.validate()
    nodes = {"index": list(node_rows), "ns_node_idx": [r[0] for r in node_rows.values()],
             "x": [r[1] for r in node_rows.values()], "y": [r[2] for r in node_rows.values()],
             "live": [r[4] for r in node_rows.values()], "weight": [r[5] for r in node_rows.values()]}
    if g.graph.get("is_dual"):
        for col in ("primal_edge_node_a", "primal_edge_node_b", "primal_edge_idx"):
            nodes[col] = [g.nodes[k].get(col) for k in node_rows]
    rows = list(edge_rows.values())
    edges = {"index": list(edge_rows), "ns_edge_idx": [r[0] for r in rows],
             "start_ns_node_idx": [r[1] for r in rows], "end_ns_node_idx": [r[2] for r in rows],
             "edge_idx": [int(r[3]) for r in rows], "nx_start_node_key": [r[4] for r in rows],
             "nx_end_node_key": [r[5] for r in rows], "imp_factor": [r[6] for r in rows],
             "geom": [r[7] for r in rows], "primal_node_id": [r[8] for r in rows]}
    nodes["z"] = [r[3] for r in node_rows.values()]
    return nodes, edges, ns


def _records(frame):
    """Rows of a (Geo)DataFrame or of a dict of equal-length columns, as dicts (index under "index")."""
    if hasattr(frame, "iterrows"):
        for key, row in frame.iterrows():
            rec = dict(row)
            rec["index"] = key
            if hasattr(frame, "geometry"):
                rec["geom"] = row[frame.geometry.name]
            yield rec
        return
    cols = list(frame)
    n = len(frame[cols[0]]) if cols else 0
    for i in range(n):
        yield {c: frame[c][i] for c in cols}


def network_structure_from_gpd(nodes_gdf, edges_gdf) -> NetworkStructure:
    """Rebuilds a NetworkStructure from the node and edge frames network_structure_from_nx returns
    (pysrc/cityseer/tools/io.py:1213-1321): GeoDataFrames, or the plain dicts of columns this package
    returns where geopandas is absent.  Edges whose end nodes are missing are skipped."""
    node_cols = ("x", "y", "live", "weight")
    edge_cols = ("start_ns_node_idx", "end_ns_node_idx", "edge_idx", "nx_start_node_key", "nx_end_node_key",
                 "imp_factor")
    have_n = set(nodes_gdf.columns) if hasattr(nodes_gdf, "columns") else set(nodes_gdf)
    have_e = set(edges_gdf.columns) if hasattr(edges_gdf, "columns") else set(edges_gdf)
    for c in node_cols:
        if c not in have_n:
            raise ValueError(f"Missing expected column in nodes GDF: {c}")
    for c in edge_cols:
        if c not in have_e:
            raise ValueError(f"Missing expected column in edges GDF: {c}")
    ns = NetworkStructure()
    mapping, xy = {}, {}
    for rec in _records(nodes_gdf):
        z = rec.get("z")
        if z is not None and isinstance(z, float) and z != z:
            z = None
        key = rec["index"]
        mapping[key] = ns.add_street_node(str(key), float(rec["x"]), float(rec["y"]), bool(rec["live"]),
                                          float(rec["weight"]), z=None if z is None else float(z))
        xy[key] = (float(rec["x"]), float(rec["y"]))
    for rec in _records(edges_gdf):
        a, b = rec["nx_start_node_key"], rec["nx_end_node_key"]
        if a not in mapping or b not in mapping:
            continue
        coords = align_linestring_coords(coords_of(rec["geom"]), xy[a])
        shared = rec.get("primal_node_id")
        if shared is not None and isinstance(shared, float) and shared != shared:
            shared = None
        ns.add_street_edge_coords(mapping[a], mapping[b], int(rec["edge_idx"]), a, b, coords,
                                  float(rec["imp_factor"]), shared_primal_node_key=None if shared is None else str(shared))
    ns.validate()
    ns.build_edge_rtree()
    return ns


def nx_from_cityseer_geopandas(nodes_gdf, edges_gdf) -> nx.MultiGraph:
    """The inverse of network_structure_from_nx's frames (pysrc/cityseer/tools/io.py:1431-1501): nodes
    with x, y, live, weight (and z), edges keyed by (start, end, edge_idx) with their impedance and
    geometry, and every cc_* metric column copied onto the nodes.  Accepts GeoDataFrames or the dicts
    of columns this package returns."""
    g = nx.MultiGraph()
    recs = list(_records(nodes_gdf))
    for rec in recs:
        kw = {"x": rec["x"], "y": rec["y"], "live": rec.get("live", True), "weight": rec.get("weight", 1)}
        z = rec.get("z")
        if z is not None and not (isinstance(z, float) and z != z):
            kw["z"] = z
        g.add_node(str(rec["index"]), **kw)
    for rec in _records(edges_gdf):
        a, b, k = str(rec["nx_start_node_key"]), str(rec["nx_end_node_key"]), rec["edge_idx"]
        if not g.has_edge(a, b, k):
            extra = {"total_bearing": rec["total_bearing"]} if "total_bearing" in rec else {}
            g.add_edge(a, b, k, imp_factor=rec["imp_factor"], geom=rec["geom"], **extra)
    cols = [c for c in (nodes_gdf.columns if hasattr(nodes_gdf, "columns") else nodes_gdf) if str(c).startswith("cc_")]
    for c in cols:
        for rec in recs:
            g.nodes[str(rec["index"])][c] = rec[c]
    return g
