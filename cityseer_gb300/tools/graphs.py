"""networkx graph helpers restated without shapely.

Edge geometries are sequences of coordinate tuples (anything with a ``.coords`` attribute, such as
a shapely LineString, is accepted as well).
  nx_simple_geoms  pysrc/cityseer/tools/graphs.py:58-107
  nx_decompose     pysrc/cityseer/tools/graphs.py:1829-1962
  nx_to_dual       pysrc/cityseer/tools/graphs.py:1965-2149 (half geometries split at the
                   normalised midpoint, welded at the shared primal node; util.py:264-312 for the
                   coordinate alignment)
"""
from __future__ import annotations

import math

import networkx as nx


def coords_of(geom) -> list[tuple[float, ...]]:
    return [tuple(float(v) for v in c) for c in getattr(geom, "coords", geom)]


def _seg_len(a, b) -> float:
    return math.hypot(b[0] - a[0], b[1] - a[1])


def _length(coords) -> float:
    return sum(_seg_len(coords[i], coords[i + 1]) for i in range(len(coords) - 1))


def _interpolate(coords, dist):
    """Point at `dist` along the polyline (clamped to its ends)."""
    if dist <= 0:
        return tuple(coords[0][:2])
    acc = 0.0
    for i in range(len(coords) - 1):
        s = _seg_len(coords[i], coords[i + 1])
        if acc + s >= dist and s > 0:
            f = (dist - acc) / s
            a, b = coords[i], coords[i + 1]
            return (a[0] + (b[0] - a[0]) * f, a[1] + (b[1] - a[1]) * f)
        acc += s
    return tuple(coords[-1][:2])


def _interpolate_z(coords, dist):
    """z at `dist` (2D length) along a 3D polyline, linear within the segment, as GEOS interpolates
    a 3D LineString; None for a 2D polyline."""
    if not coords or len(coords[0]) < 3 or any(len(c) < 3 for c in coords):
        return None
    if dist <= 0:
        return float(coords[0][2])
    acc = 0.0
    for i in range(len(coords) - 1):
        s = _seg_len(coords[i], coords[i + 1])
        if acc + s >= dist and s > 0:
            f = (dist - acc) / s
            return float(coords[i][2] + (coords[i + 1][2] - coords[i][2]) * f)
        acc += s
    return float(coords[-1][2])


def substring(coords, start_dist, end_dist):
    """Part of the polyline between two distances from its start (start < end)."""
    sp = _interpolate(coords, start_dist)
    ep = _interpolate(coords, end_dist)
    out = [sp]
    cur = 0.0
    for i in range(len(coords) - 1):
        if start_dist < cur < end_dist:
            out.append(tuple(coords[i][:2]))
        elif cur >= end_dist:
            break
        cur += _seg_len(coords[i], coords[i + 1])
    out.append(ep)
    return out


def align_linestring_coords(coords, xy, reverse=False, tolerance=0.5):
    """util.align_linestring_coords (pysrc/cityseer/tools/util.py:264-312)."""
    coords = list(coords)
    a = math.hypot(coords[0][0] - xy[0], coords[0][1] - xy[1])
    b = math.hypot(coords[-1][0] - xy[0], coords[-1][1] - xy[1])
    if not reverse:
        if a > b:
            coords = coords[::-1]
        tol = math.hypot(coords[0][0] - xy[0], coords[0][1] - xy[1])
    else:
        if a < b:
            coords = coords[::-1]
        tol = math.hypot(coords[-1][0] - xy[0], coords[-1][1] - xy[1])
    if tol > tolerance:
        raise ValueError(f"Closest side of edge geom {coords} is {tol} from node {xy}, exceeding tolerance of "
                         f"{tolerance}.")
    return coords


def nx_simple_geoms(g: nx.MultiGraph) -> nx.MultiGraph:
    """Straight geometries between node coordinates; zero-length edges are removed."""
    g = g.copy()
    remove = []
    for s, e, k in g.edges(keys=True):
        sd, ed = g.nodes[s], g.nodes[e]
        if sd.get("z") is not None and ed.get("z") is not None:
            geom = [(sd["x"], sd["y"], sd["z"]), (ed["x"], ed["y"], ed["z"])]
        else:
            geom = [(sd["x"], sd["y"]), (ed["x"], ed["y"])]
        if _length(geom) == 0:
            remove.append((s, e, k))
        else:
            g[s][e][k]["geom"] = geom
    for s, e, k in remove:
        g.remove_edge(s, e, key=k)
    return g


def _sub_name(parts) -> str:
    """util.add_node's name for a node made from others (pysrc/cityseer/tools/util.py:529-541)."""
    names = []
    for n in parts:
        n = str(n)
        names.append(f"{n[:5]}|{n[-5:]}" if len(n) > 10 else n)
    return "±".join(names)


def nx_decompose(g: nx.MultiGraph, decompose_max: float) -> nx.MultiGraph:
    """Splits every edge into ceil(length / decompose_max) pieces of equal length
    (pysrc/cityseer/tools/graphs.py:1829-1962).  New nodes are named from the edge's end nodes and
    a counter; a new node is live unless both parent nodes are non-live (when both carry `live`)."""
    if decompose_max <= 0:
        raise ValueError("decompose_max must be positive")
    out = g.copy()
    for s, e, data in g.edges(data=True):
        sxy = (g.nodes[s]["x"], g.nodes[s]["y"])
        line = align_linestring_coords(coords_of(data["geom"]), sxy)
        L = _length(line)
        cuts = max(1, int(math.ceil(L / decompose_max)))
        step_size = L / cuts
        out.remove_edge(s, e)
        rest = {k: v for k, v in data.items() if k != "geom"}
        prior, step = s, 0.0
        for i in range(cuts - 1):
            seg = substring(line, step, step + step_size)
            x, y = seg[-1][0], seg[-1][1]
            name = _sub_name([s, i, e])
            if name in out:
                raise ValueError(f"Attempted to add a duplicate node at x: {x}, y:{y}. "
                                 f"Check for existence of duplicate edges in the vicinity of {s}-{e}.")
            out.add_node(name, x=x, y=y)
            if "live" in g.nodes[s] and "live" in g.nodes[e]:
                out.nodes[name]["live"] = bool(g.nodes[s]["live"]) or bool(g.nodes[e]["live"])
            out.add_edge(prior, name, geom=seg, **rest)
            prior = name
            step += step_size
        out.add_edge(prior, e, geom=substring(line, step, L), **rest)
    return out


def _dual_key(a, b, k) -> str:
    s = sorted([str(a), str(b)])
    return f"{s[0]}_{s[1]}_k{k}"


def _half_geoms(g, a, b, k):
    line = align_linestring_coords(coords_of(g[a][b][k]["geom"]), (g.nodes[a]["x"], g.nodes[a]["y"]))
    L = _length(line)
    ah = substring(line, 0.0, 0.5 * L)
    bh = substring(line, 0.5 * L, L)
    axy = (g.nodes[a]["x"], g.nodes[a]["y"])
    bxy = (g.nodes[b]["x"], g.nodes[b]["y"])
    ah[0] = axy
    mid = ah[-1]
    bh[0] = mid
    bh[-1] = bxy
    return ah, bh


def nx_to_dual(g: nx.MultiGraph) -> nx.MultiGraph:
    if g.graph.get("is_dual"):
        raise ValueError("Graph is already a dual graph.")
    d = nx.MultiGraph()
    d.graph["is_dual"] = True
    if "crs" in g.graph:
        d.graph["crs"] = g.graph["crs"]
    for s, e, k, data in g.edges(data=True, keys=True):
        line = coords_of(data["geom"])
        mid = _interpolate(line, 0.5 * _length(line))
        key = _dual_key(s, e, k)
        d.add_node(key, x=mid[0], y=mid[1], primal_edge=line, primal_edge_node_a=s, primal_edge_node_b=e,
                   primal_edge_idx=k)
        mz = _interpolate_z(line, 0.5 * _length(line))
        if mz is not None:  # the midpoint of a 3D primal edge keeps its z (graphs.py:2099-2100)
            d.nodes[key]["z"] = mz
        if "live" in g.nodes[s] and "live" in g.nodes[e]:
            d.nodes[key]["live"] = bool(g.nodes[s]["live"]) or bool(g.nodes[e]["live"])
    for s, e, k in g.edges(keys=True):
        hub = _dual_key(s, e, k)
        s_half, e_half = _half_geoms(g, s, e, k)
        for n_side, m_side, half in ((s, e, s_half), (e, s, e_half)):
            for nb in nx.neighbors(g, n_side):
                if nb == m_side:
                    continue
                for k2 in g[n_side][nb]:
                    spoke = _dual_key(n_side, nb, k2)
                    if d.has_edge(hub, spoke):
                        continue
                    spoke_half, _ = _half_geoms(g, n_side, nb, k2)
                    # welded at n_side: hub midpoint -> n_side -> spoke midpoint
                    to_node = half[::-1] if n_side == s else half
                    merged = list(to_node) + list(spoke_half[1:])
                    d.add_edge(hub, spoke, primal_node_id=n_side, geom=merged)
    return d
