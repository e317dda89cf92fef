"""Data layers on the street network: data entries, their assignment to street nodes, and the
per-source aggregation and accessibility sums (the reference's rustalgos.data, rust/src/data.rs).

`DataMap` mirrors the reference's class: `insert`, `entry_keys`, `get_entry`, `count`,
`node_data_map`, `assign_data_to_network`, `aggregate_to_src_idx` and `accessibility`, with the same
argument names, defaults, keys (`py_key_to_composite`, rust/src/common.rs:91-96) and result types.

* Assignment (`find_assignments_for_entry`, rust/src/graph.rs:1346-1486) restated for point data
  over the structure's street segments (straight between node coordinates unless the edge was added
  with a polyline): the nearest street edges within `max_assignment_dist` (up to
  `n_nearest_candidates`), each giving its start and end node when the straight line from the point
  to the node crosses no street; a point stops at the first edge that gave a node.  Barriers are not
  checked (`set_barriers` stores them without an index): a structure with barriers is refused.
* `accessibility` runs on the GPU: one search per live source to the largest threshold (the
  per-warp kernel's label-correcting search, so the distances equal dijkstra_tree_shortest's), then
  per reached node its assigned entries, deduplicated per dedupe key to the nearest (data.rs:562-595)
  and summed per land-use class and threshold (data.rs:688-731).  Angular accessibility
  (`angular=True`, on a dual graph) aggregates the GPU's simplest-path trees on the host.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass

import numpy as np

from . import common, config

_POINT = re.compile(r"^\s*POINT\s*Z?\s*\(\s*([-+0-9.eE]+)\s+([-+0-9.eE]+)(?:\s+[-+0-9.eE]+)?\s*\)\s*$", re.I)


def composite_key(obj) -> str:
    """py_key_to_composite (rust/src/common.rs:91-96): '<type name>:<str(value)>'."""
    return f"{type(obj).__name__}:{obj}"


def _parse_point(key: str, wkt: str) -> tuple[float, float]:
    m = _POINT.match(wkt)
    if not m:
        raise ValueError(f"Failed to parse WKT for key '{key}': only POINT geometries are supported here")
    return float(m.group(1)), float(m.group(2))


@dataclass
class DataEntry:
    """DataEntry (rust/src/data.rs:306-378)."""

    data_key_py: object
    data_key: str
    dedupe_key_py: object
    dedupe_key: str
    geom_wkt: str
    x: float
    y: float

    @classmethod
    def new(cls, data_key_py, geom_wkt: str, dedupe_key_py=None) -> "DataEntry":
        data_key = composite_key(data_key_py)
        if dedupe_key_py is None:
            dedupe_key_py, dedupe_key = data_key_py, data_key
        else:
            dedupe_key = composite_key(dedupe_key_py)
        x, y = _parse_point(data_key, geom_wkt)
        return cls(data_key_py, data_key, dedupe_key_py, dedupe_key, geom_wkt, x, y)


class LanduseAccess:
    """Per land-use key: weighted, unweighted and nearest-distance rows (rust/src/data.rs:21-45),
    each a {distance: f64[node_count]} dict compacted to the structure's node indices."""

    def __init__(self, distances, node_indices, weighted, unweighted, nearest, max_dist):
        self._d = list(distances)
        self._idx = np.asarray(node_indices, np.int64)
        self._w, self._u, self._n = weighted, unweighted, nearest
        self._max = max_dist

    @property
    def weighted(self) -> dict[int, np.ndarray]:
        return {d: self._w[i][self._idx].copy() for i, d in enumerate(self._d)}

    @property
    def unweighted(self) -> dict[int, np.ndarray]:
        return {d: self._u[i][self._idx].copy() for i, d in enumerate(self._d)}

    @property
    def distance(self) -> dict[int, np.ndarray]:
        return {self._max: self._n[self._idx].copy()}


class AccessibilityResult:
    """AccessibilityResult (rust/src/data.rs:47-101)."""

    def __init__(self, distances, node_keys_py, node_indices, result: dict[str, LanduseAccess]):
        self.distances = list(distances)
        self.node_keys_py = node_keys_py
        self.node_indices = list(node_indices)
        self._result = result

    @property
    def result(self) -> dict[str, LanduseAccess]:
        return dict(self._result)


def _street_segments(ns):
    """Unique street segments (start node, end node, ax, ay, bx, by), one per undirected edge
    geometry (build_edge_rtree, rust/src/graph.rs:1064-1131), as arrays."""
    a = ns.arrays()
    ex = np.nonzero(a["e_exists"])[0]
    src = a["e_src"][ex].astype(np.int64)
    dst = a["e_dst"][ex].astype(np.int64)
    trans = ns._e_transport.view()[ex].astype(bool) if hasattr(ns, "_e_transport") else np.zeros(len(ex), bool)
    xs, ys = ns._x.view(), ns._y.view()
    seen = set()
    starts, ends, edge_of = [], [], []
    polys = getattr(ns, "_edge_coords", {})
    segs = []
    for j, e in enumerate(ex):
        if trans[j]:
            continue
        u, v = int(src[j]), int(dst[j])
        pts = polys.get(int(e))
        if pts is None:
            pts = ((xs[u], ys[u]), (xs[v], ys[v]))
        key = (min(u, v), max(u, v), tuple(pts) if u < v else tuple(reversed(pts)))
        if key in seen:
            continue
        seen.add(key)
        item = len(starts)
        starts.append(u)
        ends.append(v)
        for p, q in zip(pts[:-1], pts[1:]):
            segs.append((item, p[0], p[1], q[0], q[1]))
    s = np.asarray(segs, np.float64).reshape(-1, 5)
    return np.asarray(starts, np.int64), np.asarray(ends, np.int64), s


def _point_segment_dist(px, py, ax, ay, bx, by):
    dx, dy = bx - ax, by - ay
    ll = dx * dx + dy * dy
    t = np.where(ll > 0, ((px - ax) * dx + (py - ay) * dy) / np.where(ll > 0, ll, 1.0), 0.0)
    t = np.clip(t, 0.0, 1.0)
    return np.hypot(px - (ax + t * dx), py - (ay + t * dy))


def _proper_crossing(x1, y1, x2, y2, s):
    """Whether segment (x1, y1)-(x2, y2) crosses any of the segments s (rows ax, ay, bx, by) at a
    point interior to both (line_intersects_streets, rust/src/graph.rs:1488-1514)."""
    if len(s) == 0:
        return False
    lo_x, hi_x, lo_y, hi_y = min(x1, x2), max(x1, x2), min(y1, y2), max(y1, y2)
    m = ((np.minimum(s[:, 0], s[:, 2]) <= hi_x) & (np.maximum(s[:, 0], s[:, 2]) >= lo_x)
         & (np.minimum(s[:, 1], s[:, 3]) <= hi_y) & (np.maximum(s[:, 1], s[:, 3]) >= lo_y))
    if not m.any():
        return False
    c = s[m]

    def orient(ax, ay, bx, by, cx, cy):
        return np.sign((bx - ax) * (cy - ay) - (by - ay) * (cx - ax))

    o1 = orient(x1, y1, x2, y2, c[:, 0], c[:, 1])
    o2 = orient(x1, y1, x2, y2, c[:, 2], c[:, 3])
    o3 = orient(c[:, 0], c[:, 1], c[:, 2], c[:, 3], x1, y1)
    o4 = orient(c[:, 0], c[:, 1], c[:, 2], c[:, 3], x2, y2)
    return bool(np.any((o1 * o2 < 0) & (o3 * o4 < 0)))


class DataMap:
    """DataMap (rust/src/data.rs:380-740): data entries keyed by composite key, and their
    assignment to street nodes (node_data_map: node -> [(data_key, distance to the node)])."""

    def __init__(self):
        self.entries: dict[str, DataEntry] = {}
        self.node_data_map: dict[int, list[tuple[str, float]]] = {}
        self._progress = 0

    # -- container (data.rs:400-443)
    def progress_init(self) -> None:
        self._progress = 0

    def progress(self) -> int:
        return self._progress

    def insert(self, data_key_py, geom_wkt: str, dedupe_key_py=None) -> None:
        e = DataEntry.new(data_key_py, geom_wkt, dedupe_key_py)
        self.entries[e.data_key] = e

    def entry_keys(self) -> list[str]:
        return list(self.entries.keys())

    def get_entry(self, data_key: str) -> DataEntry | None:
        return self.entries.get(data_key)

    def count(self) -> int:
        return len(self.entries)

    def is_empty(self) -> bool:
        return not self.entries

    # -- assignment (data.rs:447-510, graph.rs:1346-1486)
    def assign_data_to_network(self, network_structure, max_assignment_dist: float, n_nearest_candidates: int) -> None:
        ns = network_structure
        if getattr(ns, "_barriers", None):
            raise NotImplementedError("data assignment with barriers is not supported")
        starts, ends, segs = _street_segments(ns)
        xs, ys = ns._x.view(), ns._y.view()
        self.node_data_map = {}
        if len(starts) == 0:
            return
        for key, ent in self.entries.items():
            px, py = ent.x, ent.y
            d_seg = _point_segment_dist(px, py, segs[:, 1], segs[:, 2], segs[:, 3], segs[:, 4])
            d_item = np.full(len(starts), np.inf)
            np.minimum.at(d_item, segs[:, 0].astype(np.int64), d_seg)
            take = min(int(n_nearest_candidates), len(d_item))
            if take <= 0:
                continue
            near = np.argpartition(d_item, take - 1)[:take] if take < len(d_item) else np.arange(len(d_item))
            near = near[np.argsort(d_item[near], kind="stable")]
            cand = [int(i) for i in near if d_item[i] <= max_assignment_dist]
            checked: dict[int, tuple[int, float] | None] = {}
            added: set[int] = set()
            found = 0

            def valid(node: int):
                nd = math.hypot(xs[node] - px, ys[node] - py)
                if nd < 1e-6:
                    return node, 0.0
                if _proper_crossing(px, py, float(xs[node]), float(ys[node]), segs[:, 1:]):
                    return None
                return node, nd

            for item in cand:
                produced = False
                for node in (int(starts[item]), int(ends[item])):
                    if node not in checked:
                        checked[node] = valid(node)
                    res = checked[node]
                    if res is not None and res[0] not in added:
                        added.add(res[0])
                        self.node_data_map.setdefault(res[0], []).append((key, res[1]))
                        produced = True
                if produced:  # point geometries stop at the first edge that gave a node
                    break
                found += 1
                if found >= n_nearest_candidates:
                    break

    # -- device-side tables
    def _tables(self, ns, classes: dict[str, int] | None = None):
        """node_data_map and the entries as arrays: per node its assignments (CSR), per entry its
        dedupe group and class, per group its assignments (CSR)."""
        keys = list(self.entries.keys())
        pos = {k: i for i, k in enumerate(keys)}
        groups: dict[str, int] = {}
        entry_group = np.zeros(len(keys), np.int64)
        for i, k in enumerate(keys):
            entry_group[i] = groups.setdefault(self.entries[k].dedupe_key, len(groups))
        nb = ns.node_bound()
        cnt = np.zeros(nb + 1, np.int64)
        for node, lst in self.node_data_map.items():
            cnt[node + 1] = len(lst)
        ptr = np.cumsum(cnt)
        n_assign = int(ptr[-1])
        a_entry = np.zeros(n_assign, np.int64)
        a_dist = np.zeros(n_assign, np.float64)
        a_node = np.zeros(n_assign, np.int64)
        a_rank = np.zeros(n_assign, np.int64)
        for node, lst in self.node_data_map.items():
            o = int(ptr[node])
            for r, (k, dd) in enumerate(lst):
                a_entry[o + r] = pos[k]
                a_dist[o + r] = dd
                a_node[o + r] = node
                a_rank[o + r] = r
        a_group = entry_group[a_entry] if n_assign else np.zeros(0, np.int64)
        order = np.argsort(a_group, kind="stable")
        gcnt = np.bincount(a_group, minlength=len(groups)) if n_assign else np.zeros(len(groups), np.int64)
        gptr = np.zeros(len(groups) + 1, np.int64)
        gptr[1:] = np.cumsum(gcnt)
        entry_class = np.full(len(keys), -1, np.int64)
        if classes is not None:
            for i, k in enumerate(keys):
                entry_class[i] = classes.get(k, -1)
        return dict(keys=keys, entry_group=entry_group, n_groups=len(groups), ptr=ptr, a_entry=a_entry,
                    a_dist=a_dist, a_node=a_node, a_rank=a_rank, g_ptr=gptr, g_assign=order.astype(np.int64),
                    entry_class=entry_class)

    # -- aggregation (data.rs:513-602)
    def aggregate_to_src_idx(self, netw_src_idx: int, network_structure, max_walk_seconds: int, speed_m_s: float,
                             angular: bool | None = None) -> dict[str, float]:
        """Reachable data entries of one source: data_key -> network distance + assignment
        distance (f32), each dedupe key at its nearest entry.  The source's tree is a GPU call."""
        ns = network_structure
        angular = bool(angular)
        if angular:
            ns.validate_dual_for_angular("aggregate_to_src_idx")
        t = self._tables(ns)
        dist = _aggregate_host(ns, t, [int(netw_src_idx)], int(max_walk_seconds), float(speed_m_s), angular)[0]
        return {t["keys"][e]: float(dist[e]) for e in np.nonzero(~np.isnan(dist))[0]}

    # -- accessibility (data.rs:605-740)
    def accessibility(self, network_structure, landuses_map, accessibility_keys, distances=None, betas=None,
                      minutes=None, angular=None, spatial_tolerance=None, min_threshold_wt=None, speed_m_s=None,
                      pbar_disabled=None) -> AccessibilityResult:
        ns = network_structure
        angular = bool(angular)
        if angular:
            ns.validate_dual_for_angular("accessibility")
        speed = float(speed_m_s) if speed_m_s is not None else config.SPEED_M_S
        d, b, s = common.pair_distances_betas_time(speed, distances=distances, betas=betas, minutes=minutes,
                                                   min_threshold_wt=min_threshold_wt)
        if len(landuses_map) != self.count():
            raise ValueError("The number of landuse encodings must match the number of data points")
        lu = {}
        for k, val in landuses_map.items():
            ck = composite_key(k)
            if ck not in self.entries:
                raise KeyError(f"Data entries key missing: {ck}")
            lu[ck] = str(val)
        keys = list(dict.fromkeys(accessibility_keys))
        mcw = np.asarray(common.clip_wts_curve(d, b, int(spatial_tolerance or 0)), np.float32)
        cls_of = {k: keys.index(v) for k, v in lu.items() if v in keys}
        t = self._tables(ns, cls_of)
        nb = ns.node_bound()
        arr = ns.arrays()
        sources = np.nonzero(arr["live"][:nb].astype(bool))[0]  # existing and live
        if angular:
            u, w, n = _accessibility_host(ns, t, sources, d, b, mcw, max(s), speed, len(keys))
        else:
            from . import access

            u, w, n = access.accessibility_rows(ns, t, sources, d, b, s, mcw, speed, len(keys))
        idx = ns.node_indices()
        res = {key: LanduseAccess(d, idx, w[c], u[c], n[c], max(d)) for c, key in enumerate(keys)}
        self._progress = len(idx)
        return AccessibilityResult(d, ns.node_keys_py(), idx, res)


def _aggregate_host(ns, t, sources, max_seconds: int, speed: float, angular: bool):
    """aggregate_to_src_idx over GPU trees, the aggregation on the host: per source an f32 distance
    per entry (NaN when not reached).  Visit order: the tree's settle order."""
    from . import centrality, dual

    if angular:
        counts, nodes, _simpl, agg, _preds = dual.tree_simplest_raw(ns, list(sources), max_seconds, speed)
        rows = [(nodes[q][: int(counts[q])], agg[q][: int(counts[q])]) for q in range(len(sources))]
    else:
        counts, nodes, agg, _preds = centrality.tree_shortest_raw(ns, list(sources), max_seconds, speed)
        rows = [(nodes[q][: int(counts[q])], agg[q][: int(counts[q])]) for q in range(len(sources))]
    out = np.full((len(sources), len(t["keys"])), np.nan, np.float32)
    max_walk = np.float32(np.float32(max_seconds) * np.float32(speed))
    ptr, a_entry, a_dist, eg = t["ptr"], t["a_entry"], t["a_dist"], t["entry_group"]
    for q, (nodes, agg) in enumerate(rows):
        best = {}
        for v, sec in zip(nodes, agg):
            sec = np.float32(sec)
            if not (sec < np.float32(max_seconds)):
                continue
            net = np.float32(sec * np.float32(speed))
            for a in range(int(ptr[v]), int(ptr[v + 1])):
                tot = np.float32(net + np.float32(a_dist[a]))
                if not (tot <= max_walk):
                    continue
                g = int(eg[a_entry[a]])
                cur = best.get(g)
                if cur is None or tot < cur[0]:
                    best[g] = (tot, int(a_entry[a]))
        for tot, e in best.values():
            out[q, e] = tot
    return out


def _accessibility_host(ns, t, sources, d, b, mcw, max_seconds, speed, n_classes):
    nb = ns.node_bound()
    K = len(d)
    u = np.zeros((n_classes, K, nb))
    w = np.zeros((n_classes, K, nb))
    n = np.full((n_classes, nb), np.nan)
    if len(sources) == 0:
        return u, w, n
    dist = _aggregate_host(ns, t, sources, max_seconds, speed, True)
    cls = t["entry_class"]
    dmax = max(d)
    for q, src in enumerate(sources):
        for e in np.nonzero(~np.isnan(dist[q]))[0]:
            c = int(cls[e])
            if c < 0:
                continue
            dd = np.float32(dist[q, e])
            for i in range(K):
                if not (dd <= np.float32(d[i])):
                    continue
                u[c, i, src] += 1.0
                raw = np.float32(np.exp(np.float32(-np.float32(b[i]) * dd), dtype=np.float32))
                w[c, i, src] += float(np.float32(min(raw, mcw[i]) / mcw[i]))
                if d[i] == dmax and (np.isnan(n[c, src]) or float(dd) < n[c, src]):
                    n[c, src] = float(dd)
    return u, w, n
