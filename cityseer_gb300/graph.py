"""Host-side NetworkStructure: the reference's graph store, restated over numpy columns.

Mirrors ``rustalgos.graph.NetworkStructure`` (rust/src/graph.rs:381-1341): the same builder
methods, getters, validation messages and index semantics (StableGraph indices with gaps after
removals; petgraph reverse-insertion edge order).  The centrality methods hand the graph to the
GPU through ``cityseer_gb300.device`` (a device-resident CSR) and libcsgpu.so.
"""
from __future__ import annotations

import math
import re
from collections.abc import Sequence
from typing import Any

import numpy as np

_LS_RE = re.compile(r"^\s*LINESTRING\s*(Z|M|ZM)?\s*\((.*)\)\s*$", re.IGNORECASE | re.DOTALL)


def parse_linestring_wkt(wkt: str) -> list[tuple[float, ...]]:
    m = _LS_RE.match(wkt)
    if not m:
        raise ValueError(f"Failed to parse WKT: {wkt[:200]}")
    coords = []
    for part in m.group(2).split(","):
        vals = part.split()
        if len(vals) < 2:
            raise ValueError(f"Failed to parse WKT coordinate '{part}'")
        coords.append(tuple(float(v) for v in vals))
    return coords


def _bearing(a, b) -> float:
    """measure_bearing (rust/src/graph.rs:326-332): degrees, 0 for coincident points."""
    if a[0] == b[0] and a[1] == b[1]:
        return 0.0
    return math.degrees(math.atan2(b[1] - a[1], b[0] - a[0]))


def _coords_angle(a, b, c) -> float:
    """measure_coords_angle (rust/src/graph.rs:336-346)."""
    if (a[0] == b[0] and a[1] == b[1]) or (b[0] == c[0] and b[1] == c[1]):
        return 0.0
    a1 = _bearing(b, a)
    a2 = _bearing(c, b)
    diff = a2 - a1
    r = math.fmod(diff + 180.0, 360.0)
    if r < 0.0:
        r += 360.0
    return abs(r - 180.0)


def cumulative_angle(coords: Sequence[Sequence[float]]) -> float:
    """measure_cumulative_angle (rust/src/graph.rs:367-379), f64."""
    if len(coords) < 3:
        return 0.0
    s = 0.0
    for i in range(1, len(coords) - 1):
        s += _coords_angle(coords[i - 1], coords[i], coords[i + 1])
    return s


def linestring_length(coords: Sequence[Sequence[float]]) -> float:
    """Euclidean length of the 2D polyline in f64 (geo Euclidean.length, rust/src/graph.rs:774)."""
    s = 0.0
    for i in range(len(coords) - 1):
        s += float(np.hypot(coords[i + 1][0] - coords[i][0], coords[i + 1][1] - coords[i][1]))
    return s


class _Col:
    """Growable numpy column with amortised appends."""

    __slots__ = ("a", "n")

    def __init__(self, dtype, data=None):
        if data is None:
            self.a = np.zeros(16, dtype=dtype)
            self.n = 0
        else:
            self.a = np.ascontiguousarray(data, dtype=dtype)
            self.n = len(self.a)

    def append(self, v):
        if self.n == len(self.a):
            b = np.zeros(max(16, 2 * len(self.a)), dtype=self.a.dtype)
            b[: self.n] = self.a[: self.n]
            self.a = b
        self.a[self.n] = v
        self.n += 1

    def view(self) -> np.ndarray:
        return self.a[: self.n]


class NodeVisit:
    """Per-node traversal state (rust/src/graph.rs:251-288)."""

    __slots__ = ("visited", "discovered", "pred", "short_dist", "simpl_dist", "origin_seg", "last_seg", "agg_seconds")

    def __init__(self):
        self.visited = False
        self.discovered = False
        self.pred = None
        self.short_dist = math.inf
        self.simpl_dist = math.inf
        self.origin_seg = None
        self.last_seg = None
        self.agg_seconds = math.inf

    def __repr__(self):
        return (
            f"NodeVisit(visited={self.visited}, pred={self.pred}, short_dist={self.short_dist}, "
            f"simpl_dist={self.simpl_dist}, agg_seconds={self.agg_seconds})"
        )


class EdgeVisit:
    """Per-edge traversal state (rust/src/graph.rs:290-315)."""

    __slots__ = ("visited", "start_nd_idx", "end_nd_idx", "edge_idx")

    def __init__(self):
        self.visited = False
        self.start_nd_idx = None
        self.end_nd_idx = None
        self.edge_idx = None


class NodePayload:
    """Node payload as rustalgos.graph.NodePayload exposes it (rust/src/graph.rs:24-88)."""

    __slots__ = ("node_key", "x", "y", "z", "live", "weight", "is_transport")

    def __init__(self, node_key, x, y, z, live, weight, is_transport):
        self.node_key, self.x, self.y, self.z = node_key, x, y, z
        self.live, self.weight, self.is_transport = live, weight, is_transport

    @property
    def coord(self) -> tuple[float, float]:
        return (self.x, self.y)

    @property
    def coord_z(self) -> tuple[float, float, float | None]:
        return (self.x, self.y, self.z)


class EdgePayload:
    """Edge payload as rustalgos.graph.EdgePayload exposes it (rust/src/graph.rs:90-115).  This
    store keeps no geometry, so geom_wkt is None."""

    __slots__ = ("start_nd_key_py", "end_nd_key_py", "edge_idx", "length", "angle_sum", "imp_factor",
                 "in_bearing", "out_bearing", "seconds", "geom_wkt", "is_transport")

    def __init__(self, **kw):
        for k in self.__slots__:
            setattr(self, k, kw.get(k))


def _leaving_direction(coords, at_start: bool) -> tuple[float, float] | None:
    """Direction in which a polyline leaves its start (or, reversed, its end): the first vertex
    that differs from the end point, minus the end point."""
    pts = coords if at_start else coords[::-1]
    x0, y0 = pts[0][0], pts[0][1]
    for q in pts[1:]:
        if q[0] != x0 or q[1] != y0:
            return (q[0] - x0, q[1] - y0)
    return None


def _recover_shared_keys(edges, coords_of_edge, node_xy) -> list[str]:
    """Shared primal node of each dual edge, up to naming, from the edge geometries.

    A dual edge runs from one dual node's midpoint through the primal node the two primal edges
    share to the other's midpoint; at a dual node, edges towards the same primal endpoint leave
    along the same half of its primal edge (same direction) and edges towards the other endpoint
    leave the opposite way.  Each (dual node, side) is a port, each edge joins the ports of its two
    ends, and the connected ports are one primal node.  Only equality of the keys matters to the
    endpoint slots (rust/src/centrality.rs:533-566), so the component id serves as the key."""
    n_e = len(edges)
    ref_dir: dict[int, tuple[float, float]] = {}
    port = [[0, 0] for _ in range(n_e)]
    for j, (s, e, _k) in enumerate(edges):
        c = coords_of_edge(j)
        sx, sy = node_xy(s)
        fwd = (c[0][0] - sx) ** 2 + (c[0][1] - sy) ** 2 <= (c[-1][0] - sx) ** 2 + (c[-1][1] - sy) ** 2
        for end, node in enumerate((s, e)):
            at_start = fwd if end == 0 else not fwd
            d = _leaving_direction(c, at_start)
            if d is None:
                raise ValueError(f"dual edge {s} -> {e} has no length: its shared primal node is undefined")
            r = ref_dir.setdefault(node, d)
            port[j][end] = 0 if d[0] * r[0] + d[1] * r[1] > 0.0 else 1
    parent: dict[tuple[int, int], tuple[int, int]] = {}

    def find(a):
        parent.setdefault(a, a)
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for j, (s, e, _k) in enumerate(edges):
        ra, rb = find((s, port[j][0])), find((e, port[j][1]))
        if ra != rb:
            parent[rb] = ra
    ids: dict[tuple[int, int], int] = {}
    out = []
    for j, (s, _e, _k) in enumerate(edges):
        r = find((s, port[j][0]))
        out.append(f"shared-{ids.setdefault(r, len(ids))}")
    return out


class NetworkStructure:
    """Graph store with the reference's builder API; centralities run on the GPU."""

    def __init__(self):
        self._keys: list[Any] | None = []
        self._x = _Col(np.float64)
        self._y = _Col(np.float64)
        self._z = _Col(np.float64)
        self._has_z = _Col(np.uint8)
        self._live = _Col(np.uint8)
        self._weight = _Col(np.float32)
        self._exists = _Col(np.uint8)
        self._transport = _Col(np.uint8)
        self._e_src = _Col(np.int32)
        self._e_dst = _Col(np.int32)
        self._e_idx = _Col(np.int64)
        self._e_len = _Col(np.float32)
        self._e_ang = _Col(np.float32)
        self._e_imp = _Col(np.float32)
        self._e_sec = _Col(np.float32)
        self._e_inb = _Col(np.float32)
        self._e_outb = _Col(np.float32)
        self._e_exists = _Col(np.uint8)
        self._e_transport = _Col(np.uint8)
        self._e_shared: list[str | None] = []
        self._e_keys: list[tuple[Any, Any] | None] | None = []
        self._is_dual = False
        self._barriers: list[str] | None = None
        self._edge_rtree_built = False
        self._progress = 0
        self._version = 0
        self._cache: dict[str, Any] = {}

    # ------------------------------------------------------------------ bulk construction
    @classmethod
    def from_arrays(
        cls,
        x: np.ndarray,
        y: np.ndarray,
        edge_src: np.ndarray,
        edge_dst: np.ndarray,
        edge_length: np.ndarray,
        *,
        edge_idx: np.ndarray | None = None,
        edge_angle_sum: np.ndarray | None = None,
        edge_imp: np.ndarray | None = None,
        edge_shared_key: Sequence[str | None] | np.ndarray | None = None,
        live: np.ndarray | None = None,
        weight: np.ndarray | None = None,
        z: np.ndarray | None = None,
        is_dual: bool = False,
        node_keys: Sequence[Any] | None = None,
    ) -> "NetworkStructure":
        """Builds a structure from columns: nodes 0..n-1, directed edges in insertion order.

        Equivalent to calling add_street_node / add_street_edge in order, with the edge lengths
        and angle sums already computed (f32) as add_street_edge would from the geometry.
        """
        ns = cls()
        n = len(x)
        m = len(edge_src)
        ns._keys = None if node_keys is None else list(node_keys)
        ns._x = _Col(np.float64, x)
        ns._y = _Col(np.float64, y)
        if z is None:
            ns._z = _Col(np.float64, np.full(n, np.nan))
            ns._has_z = _Col(np.uint8, np.zeros(n))
        else:
            z = np.asarray(z, dtype=np.float64)
            ns._z = _Col(np.float64, z)
            ns._has_z = _Col(np.uint8, ~np.isnan(z))
        ns._live = _Col(np.uint8, np.ones(n) if live is None else live)
        w = np.ones(n, np.float32) if weight is None else np.asarray(weight, np.float32)
        if not np.all(np.isfinite(w)) or np.any(w < 0):
            raise ValueError("Invalid street node payload: weight must be finite and non-negative (>= 0.0).")
        ns._weight = _Col(np.float32, w)
        ns._exists = _Col(np.uint8, np.ones(n))
        ns._transport = _Col(np.uint8, np.zeros(n))
        es = np.asarray(edge_src, np.int64)
        ed = np.asarray(edge_dst, np.int64)
        if m and (es.min() < 0 or ed.min() < 0 or es.max() >= n or ed.max() >= n):
            raise ValueError("edge endpoint does not exist in the graph.")
        ns._e_src = _Col(np.int32, es)
        ns._e_dst = _Col(np.int32, ed)
        ns._e_idx = _Col(np.int64, np.zeros(m) if edge_idx is None else edge_idx)
        ns._e_len = _Col(np.float32, edge_length)
        ns._e_ang = _Col(np.float32, np.zeros(m) if edge_angle_sum is None else edge_angle_sum)
        imp = np.ones(m, np.float32) if edge_imp is None else np.asarray(edge_imp, np.float32)
        if np.any(~np.isfinite(imp)) or np.any(imp <= 0):
            raise ValueError("Invalid edge payload : imp_factor must be finite and positive (> 0.0).")
        ns._e_imp = _Col(np.float32, imp)
        ns._e_sec = _Col(np.float32, np.full(m, np.nan))
        ns._e_inb = _Col(np.float32, np.zeros(m))
        ns._e_outb = _Col(np.float32, np.zeros(m))
        ns._e_exists = _Col(np.uint8, np.ones(m))
        ns._e_transport = _Col(np.uint8, np.zeros(m))
        if edge_shared_key is None:
            ns._e_shared = [None] * m
        else:
            ns._e_shared = [None if k is None else str(k) for k in edge_shared_key]
        ns._e_keys = None
        ns._is_dual = bool(is_dual)
        return ns

    # ------------------------------------------------------------------ basic state
    def _touch(self):
        self._version += 1
        self._cache.clear()

    def progress_init(self) -> None:
        self._progress = 0

    def progress(self) -> int:
        """Sources processed by the running centrality call, read live from its workspace on the
        device (rust/src/graph.rs:387-415); after the call, the sources it processed."""
        if getattr(self, "_running", False):
            ws = self._cache.get("wsd" if self._is_dual else "ws")
            if ws is not None:
                import ctypes as C

                from . import _native

                n = C.c_int64(0)
                if _native.load().cs_workspace_progress(ws.ptr, C.byref(n)) == _native.CS_OK:
                    return int(n.value)
        return self._progress

    def _run(self, fn, *args, **kwargs):
        """Runs a centrality call with progress() reading the device counter meanwhile."""
        self._progress = 0
        self._running = True
        try:
            return fn(self, *args, **kwargs)
        finally:
            self._running = False

    @property
    def is_dual(self) -> bool:
        return self._is_dual

    def set_is_dual(self, is_dual: bool) -> None:
        self._is_dual = bool(is_dual)
        self._touch()

    @classmethod
    def from_reference(cls, ref) -> "NetworkStructure":
        """Imports a `cityseer.rustalgos.graph.NetworkStructure` (rust/src/graph.rs:381-1341) through
        its public getters.  Nodes keep their indices (gaps after removals included); edges are added
        in `edge_references()` order with their stored payloads (length, angle sum, impedance,
        bearings, seconds), so nothing is recomputed.  A dual graph's shared primal node per edge is
        not a public field: it is recovered from the edge geometries (`geom_wkt`), see
        `_recover_shared_keys`.  Transport nodes and edges are not imported (transport linking is
        outside this package).  Where edges were removed and others added later, the reference's
        adjacency order can differ from edge-reference order, and so can heap ties."""
        ns = cls()
        dual = ref.is_dual() if callable(getattr(ref, "is_dual", None)) else bool(ref.is_dual)
        ns.set_is_dual(bool(dual))
        present = [int(i) for i in ref.node_indices()]
        nb = (max(present) + 1) if present else 0
        have = set(present)
        gaps = []
        xy: dict[int, tuple[float, float]] = {}
        for i in range(nb):
            if i not in have:
                ns._add_node(None, 0.0, 0.0, None, False, np.float32(0.0), False)
                gaps.append(i)
                continue
            p = ref.get_node_payload_py(i)
            if p.is_transport:
                raise NotImplementedError("transport nodes are not imported")
            x, y, z = p.coord_z
            xy[i] = (float(x), float(y))
            ns._add_node(p.node_key, x, y, z, bool(p.live), np.float32(p.weight), False)
        edges = [tuple(int(v) for v in er) for er in ref.edge_references()]
        pls = [ref.get_edge_payload_py(s, e, k) for s, e, k in edges]
        shared = [None] * len(edges)
        if dual and edges:
            if any(pl.geom_wkt is None for pl in pls):
                raise ValueError("dual edges need geom_wkt to recover their shared primal nodes")
            shared = _recover_shared_keys(edges, lambda j: parse_linestring_wkt(pls[j].geom_wkt), xy.__getitem__)
        for (s, e, k), pl, sh in zip(edges, pls, shared):
            if pl.is_transport:
                raise NotImplementedError("transport edges are not imported")
            ns._add_edge(s, e, k, np.float32(pl.length), np.float32(pl.angle_sum), np.float32(pl.imp_factor),
                         np.float32(np.nan if pl.seconds is None else pl.seconds), np.float32(pl.in_bearing),
                         np.float32(pl.out_bearing), sh, (pl.start_nd_key_py, pl.end_nd_key_py), False)
        for i in gaps:
            ns._exists.view()[i] = 0
        ns._touch()
        ns.validate()
        return ns

    def get_node_payload_py(self, node_idx: int) -> NodePayload:
        self._node_checked(node_idx)
        z = None if not self._has_z.view()[node_idx] else float(self._z.view()[node_idx])
        return NodePayload(self._keys[node_idx] if self._keys is not None else node_idx,
                           float(self._x.view()[node_idx]), float(self._y.view()[node_idx]), z,
                           bool(self._live.view()[node_idx]), float(self._weight.view()[node_idx]),
                           bool(self._transport.view()[node_idx]))

    def get_edge_payload_py(self, start_nd_idx: int, end_nd_idx: int, edge_idx: int) -> EdgePayload:
        self._require_node(start_nd_idx, "start_nd_idx")
        self._require_node(end_nd_idx, "end_nd_idx")
        e = self._find_edge(start_nd_idx, end_nd_idx, edge_idx)
        if e < 0:
            raise ValueError("Edge not found")
        keys = self._e_keys[e] if self._e_keys is not None and self._e_keys[e] is not None else (None, None)
        return EdgePayload(start_nd_key_py=keys[0], end_nd_key_py=keys[1], edge_idx=int(self._e_idx.view()[e]),
                           length=float(self._e_len.view()[e]), angle_sum=float(self._e_ang.view()[e]),
                           imp_factor=float(self._e_imp.view()[e]), in_bearing=float(self._e_inb.view()[e]),
                           out_bearing=float(self._e_outb.view()[e]), seconds=float(self._e_sec.view()[e]),
                           geom_wkt=None, is_transport=bool(self._e_transport.view()[e]))

    # ------------------------------------------------------------------ builders
    def add_street_node(self, node_key: Any, x: float, y: float, live: bool, weight: float, z: float | None = None) -> int:
        """add_street_node (rust/src/graph.rs:426-452)."""
        w = np.float32(weight)
        if not np.isfinite(w) or w < 0:
            raise ValueError(
                f"Invalid street node payload: weight must be finite and non-negative (>= 0.0). Found {weight}. "
                f"Node key: {node_key!r}"
            )
        return self._add_node(node_key, x, y, z, bool(live), w, False)

    def add_transport_node(self, node_key: Any, x: float, y: float, linking_radius: float | None = None,
                           z: float | None = None) -> int:
        """Transport nodes are never live and carry zero weight (rust/src/graph.rs:454-555)."""
        return self._add_node(node_key, x, y, z, False, np.float32(0.0), True)

    def _add_node(self, key, x, y, z, live, w, transport) -> int:
        idx = self._x.n
        if self._keys is None:
            self._keys = list(range(idx))
        self._keys.append(key)
        self._x.append(float(x))
        self._y.append(float(y))
        self._z.append(np.nan if z is None else float(z))
        self._has_z.append(0 if z is None else 1)
        self._live.append(1 if live else 0)
        self._weight.append(w)
        self._exists.append(1)
        self._transport.append(1 if transport else 0)
        self._touch()
        return idx

    def _require_node(self, idx: int, name: str) -> None:
        if idx < 0 or idx >= self._x.n or not self._exists.view()[idx]:
            raise ValueError(f"{name} {idx} does not exist in the graph.")

    def add_street_edge(
        self,
        start_nd_idx: int,
        end_nd_idx: int,
        edge_idx: int,
        start_nd_key_py: Any,
        end_nd_key_py: Any,
        geom_wkt: str,
        imp_factor: float | None = None,
        shared_primal_node_key: str | None = None,
    ) -> int:
        """add_street_edge (rust/src/graph.rs:727-889): length, bearings, angle_sum from WKT."""
        coords = parse_linestring_wkt(geom_wkt)
        if len(coords) < 2:
            raise ValueError(
                f"Street edge geometry (idx {edge_idx}) between nodes {start_nd_idx} and {end_nd_idx} must have "
                f"at least 2 coordinates. Found {len(coords)}."
            )
        return self.add_street_edge_coords(start_nd_idx, end_nd_idx, edge_idx, start_nd_key_py, end_nd_key_py,
                                           coords, imp_factor, shared_primal_node_key)

    def add_street_edge_coords(self, start_nd_idx, end_nd_idx, edge_idx, start_key, end_key, coords,
                               imp_factor=None, shared_primal_node_key=None) -> int:
        """add_street_edge with an already parsed coordinate list."""
        length = np.float32(linestring_length(coords))
        first, last = coords[0], coords[-1]
        inb = 0.0
        for c in coords[1:]:
            if c[0] != first[0] or c[1] != first[1]:
                inb = _bearing(first, c)
                break
        outb = 0.0
        for c in reversed(coords[:-1]):
            if c[0] != last[0] or c[1] != last[1]:
                outb = _bearing(c, last)
                break
        angle_sum = np.float32(cumulative_angle(coords))
        imp = np.float32(1.0 if imp_factor is None else imp_factor)
        if not np.isfinite(imp) or imp <= 0:
            raise ValueError(
                f"Invalid impedance factor ({imp_factor}) for edge (idx {edge_idx}) between nodes {start_nd_idx} "
                f"and {end_nd_idx}.\nImpedance must be finite and positive (> 0.0)."
            )
        self._require_node(start_nd_idx, "start_nd_idx")
        self._require_node(end_nd_idx, "end_nd_idx")
        if not np.isfinite(length):
            raise ValueError("Invalid street edge payload : length must be finite.")
        return self._add_edge(start_nd_idx, end_nd_idx, edge_idx, length, angle_sum, imp, np.float32(np.nan),
                              np.float32(inb), np.float32(outb), shared_primal_node_key, (start_key, end_key), False)

    def add_transport_edge(self, start_nd_idx, end_nd_idx, edge_idx, start_nd_key_py, end_nd_key_py, seconds,
                           imp_factor=None) -> int:
        """add_transport_edge (rust/src/graph.rs:946-985): a travel-time edge without geometry."""
        s = np.float32(seconds)
        if not np.isfinite(s) or s < 0:
            raise ValueError(
                f"Invalid seconds value ({seconds}) for transport edge (idx {edge_idx}) between nodes "
                f"{start_nd_idx} and {end_nd_idx}."
            )
        self._require_node(start_nd_idx, "start_nd_idx")
        self._require_node(end_nd_idx, "end_nd_idx")
        imp = np.float32(1.0 if imp_factor is None else imp_factor)
        return self._add_edge(start_nd_idx, end_nd_idx, edge_idx, np.float32(np.nan), np.float32(np.nan), imp, s,
                              np.float32(np.nan), np.float32(np.nan), None, (start_nd_key_py, end_nd_key_py), True)

    def _add_edge(self, s, d, eidx, length, ang, imp, sec, inb, outb, shared, keys, transport) -> int:
        idx = self._e_src.n
        self._e_src.append(int(s))
        self._e_dst.append(int(d))
        self._e_idx.append(int(eidx))
        self._e_len.append(length)
        self._e_ang.append(ang)
        self._e_imp.append(imp)
        self._e_sec.append(sec)
        self._e_inb.append(inb)
        self._e_outb.append(outb)
        self._e_exists.append(1)
        self._e_transport.append(1 if transport else 0)
        self._e_shared.append(None if shared is None else str(shared))
        if self._e_keys is None:
            self._e_keys = [None] * idx
        self._e_keys.append(keys)
        self._touch()
        return idx

    def remove_street_node(self, node_idx: int) -> None:
        """remove_street_node (rust/src/graph.rs:891-916): removes the node and its edges."""
        if node_idx < 0 or node_idx >= self._x.n or not self._exists.view()[node_idx]:
            raise ValueError(f"Node index {node_idx} does not exist in the graph.")
        if self._transport.view()[node_idx]:
            raise ValueError(
                f"Node index {node_idx} is a transport node and cannot be removed with remove_street_node."
            )
        self._exists.view()[node_idx] = 0
        es, ed, ex = self._e_src.view(), self._e_dst.view(), self._e_exists.view()
        ex[(es == node_idx) | (ed == node_idx)] = 0
        self._touch()

    def remove_street_edge(self, start_nd_idx: int, end_nd_idx: int, edge_idx: int) -> None:
        """remove_street_edge (rust/src/graph.rs:918-944): the newest matching directed edge."""
        self._require_node(start_nd_idx, "start_nd_idx")
        self._require_node(end_nd_idx, "end_nd_idx")
        e = self._find_edge(start_nd_idx, end_nd_idx, edge_idx)
        if e < 0:
            raise ValueError(f"No edge with edge_idx {edge_idx} found from node {start_nd_idx} to node {end_nd_idx}.")
        self._e_exists.view()[e] = 0
        self._touch()

    def _find_edge(self, start, end, edge_idx) -> int:
        es, ed, ei, ex = self._e_src.view(), self._e_dst.view(), self._e_idx.view(), self._e_exists.view()
        hits = np.nonzero((es == start) & (ed == end) & (ei == edge_idx) & (ex == 1))[0]
        return int(hits[-1]) if len(hits) else -1

    # ------------------------------------------------------------------ getters
    def node_count(self) -> int:
        return int(self._exists.view().sum())

    def node_bound(self) -> int:
        ex = self._exists.view()
        nz = np.nonzero(ex)[0]
        return int(nz[-1]) + 1 if len(nz) else 0

    def edge_bound(self) -> int:
        ex = self._e_exists.view()
        nz = np.nonzero(ex)[0]
        return int(nz[-1]) + 1 if len(nz) else 0

    @property
    def edge_count(self) -> int:
        return int(self._e_exists.view().sum())

    def street_node_count(self) -> int:
        return int(((self._exists.view() == 1) & (self._transport.view() == 0)).sum())

    def _node_index_array(self) -> np.ndarray:
        """Indices of the existing nodes as a read-only int64 array, cached until the graph changes."""
        c = self._cache.get("node_idx")
        if c is None:
            c = np.nonzero(self._exists.view())[0].astype(np.int64)
            c.setflags(write=False)
            self._cache["node_idx"] = c
        return c

    def node_indices(self) -> list[int]:
        return self._node_index_array().tolist()

    def street_node_indices(self) -> list[int]:
        return np.nonzero((self._exists.view() == 1) & (self._transport.view() == 0))[0].tolist()

    def node_keys_py(self) -> list[Any]:
        c = self._cache.get("node_keys")
        if c is None:
            idx = self._node_index_array()
            c = idx.tolist() if self._keys is None else [self._keys[i] for i in idx]
            self._cache["node_keys"] = c
        return list(c)

    @property
    def node_xs(self) -> list[float]:
        return self._x.view()[self._exists.view() == 1].tolist()

    @property
    def node_ys(self) -> list[float]:
        return self._y.view()[self._exists.view() == 1].tolist()

    @property
    def node_xys(self) -> list[tuple[float, float]]:
        m = self._exists.view() == 1
        return list(zip(self._x.view()[m].tolist(), self._y.view()[m].tolist()))

    @property
    def node_lives(self) -> list[bool]:
        return [bool(v) for v in self._live.view()[self._exists.view() == 1]]

    @property
    def street_node_lives(self) -> list[bool]:
        m = (self._exists.view() == 1) & (self._transport.view() == 0)
        return [bool(v) for v in self._live.view()[m]]

    @property
    def node_zs(self) -> list[float | None]:
        m = self._exists.view() == 1
        return [float(z) if h else None for z, h in zip(self._z.view()[m], self._has_z.view()[m])]

    @property
    def node_xyzs(self) -> list[tuple[float, float, float | None]]:
        m = self._exists.view() == 1
        return list(zip(self._x.view()[m].tolist(), self._y.view()[m].tolist(), self.node_zs))

    # Spatial indexes and barriers serve data assignment (rust/src/graph.rs:1064-1231), which this
    # package does not restate; centrality never reads them, in the reference as here.
    def build_edge_rtree(self) -> None:
        """Accepted for compatibility: no edge R-tree is kept (centrality does not use one)."""
        self._edge_rtree_built = True

    def set_barriers(self, barriers_wkt: list[str]) -> None:
        """Stores the barrier geometries (WKT); centrality does not use them."""
        self._barriers = list(barriers_wkt)

    def unset_barriers(self) -> None:
        self._barriers = None

    def _node_checked(self, node_idx: int) -> None:
        self._require_node(node_idx, "node_idx")

    def get_node_weight(self, node_idx: int) -> float:
        self._node_checked(node_idx)
        return float(self._weight.view()[node_idx])

    def is_node_live(self, node_idx: int) -> bool:
        self._node_checked(node_idx)
        return bool(self._live.view()[node_idx])

    def set_node_live(self, node_idx: int, live: bool) -> None:
        if node_idx < 0 or node_idx >= self._x.n or not self._exists.view()[node_idx]:
            raise ValueError(f"Node index {node_idx} does not exist in the graph.")
        self._live.view()[node_idx] = 1 if live else 0
        self._touch()

    def edge_references(self) -> list[tuple[int, int, int]]:
        ex = np.nonzero(self._e_exists.view())[0]
        es, ed, ei = self._e_src.view(), self._e_dst.view(), self._e_idx.view()
        return [(int(es[e]), int(ed[e]), int(ei[e])) for e in ex]

    def get_edge_length(self, start_nd_idx: int, end_nd_idx: int, edge_idx: int) -> float:
        self._require_node(start_nd_idx, "start_nd_idx")
        self._require_node(end_nd_idx, "end_nd_idx")
        e = self._find_edge(start_nd_idx, end_nd_idx, edge_idx)
        if e < 0:
            raise ValueError("Edge not found")
        return float(self._e_len.view()[e])

    def get_edge_impedance(self, start_nd_idx: int, end_nd_idx: int, edge_idx: int) -> float:
        self._require_node(start_nd_idx, "start_nd_idx")
        self._require_node(end_nd_idx, "end_nd_idx")
        e = self._find_edge(start_nd_idx, end_nd_idx, edge_idx)
        if e < 0:
            raise ValueError("Edge not found")
        return float(self._e_imp.view()[e])

    def validate(self) -> None:
        """validate (rust/src/graph.rs:1035-1058)."""
        if self.node_count() == 0:
            raise ValueError("NetworkStructure contains no nodes.")
        ex = self._e_exists.view() == 1
        street = ex & (self._e_transport.view() == 0)
        if np.any(~np.isfinite(self._e_len.view()[street])):
            raise ValueError("Invalid street edge payload : length must be finite.")
        if np.any(~np.isfinite(self._e_ang.view()[street])):
            raise ValueError("Invalid street edge payload : angle_sum must be finite.")
        imp = self._e_imp.view()[ex]
        if np.any(~np.isfinite(imp)) or np.any(imp <= 0):
            raise ValueError("Invalid edge payload : imp_factor must be finite and positive (> 0.0).")

    def validate_dual_for_angular(self, context: str) -> None:
        """validate_dual_for_angular (rust/src/graph.rs:1333-1341)."""
        if not self._is_dual:
            raise ValueError(
                f"{context} requires a dual graph for angular analysis. Convert the graph with "
                "cityseer.tools.graphs.nx_to_dual(...) before ingesting it into NetworkStructure."
            )

    # ------------------------------------------------------------------ arrays for the device / oracle
    def arrays(self) -> dict[str, np.ndarray]:
        """Column view of the graph (node slots and edge slots, with existence flags)."""
        c = self._cache.get("arrays")
        if c is not None:
            return c
        nb = self._x.n
        shared = self._e_shared
        uniq: dict[str, int] = {}
        sid = np.full(self._e_src.n, -1, np.int32)
        for i, k in enumerate(shared):
            if k is not None:
                sid[i] = uniq.setdefault(k, len(uniq))
        c = {
            "n_slots": nb,
            "node_exists": self._exists.view().copy(),
            "live": (self._live.view() & self._exists.view()).astype(np.uint8),
            "weight": self._weight.view().copy(),
            "has_z": self._has_z.view().copy(),
            "z": self._z.view().copy(),
            "e_src": self._e_src.view().copy(),
            "e_dst": self._e_dst.view().copy(),
            "e_exists": self._e_exists.view().copy(),
            "e_idx": self._e_idx.view().copy(),
            "e_len": self._e_len.view().copy(),
            "e_ang": self._e_ang.view().copy(),
            "e_imp": self._e_imp.view().copy(),
            "e_sec": self._e_sec.view().copy(),
            "e_shared": sid,
        }
        self._cache["arrays"] = c
        return c

    # ------------------------------------------------------------------ traversals and centrality
    def _validate_src(self, src_idx: int, speed_m_s: float) -> None:
        """validate_dijkstra_inputs (rust/src/centrality.rs:1009-1030)."""
        nb = self.node_bound()
        if src_idx < 0 or src_idx >= nb:
            raise ValueError(f"src_idx {src_idx} out of range for network with node_bound {nb}")
        if not self._exists.view()[src_idx]:
            raise ValueError(f"src_idx {src_idx} does not exist in the graph")
        if not math.isfinite(speed_m_s) or speed_m_s <= 0:
            raise ValueError(f"speed_m_s must be finite and positive, got {speed_m_s}")

    def dijkstra_tree_shortest(self, src_idx: int, max_seconds: int, speed_m_s: float):
        from . import centrality

        self._validate_src(src_idx, speed_m_s)
        return centrality.tree_shortest(self, [src_idx], max_seconds, speed_m_s)[0]

    def dijkstra_tree_shortest_batch(self, src_indices: Sequence[int], max_seconds: int, speed_m_s: float):
        """Many isochrone queries in one launch (one warp per query)."""
        from . import centrality

        for s in src_indices:
            self._validate_src(int(s), speed_m_s)
        return centrality.tree_shortest(self, list(src_indices), max_seconds, speed_m_s)

    def dijkstra_tree_segment(self, src_idx: int, max_seconds: int, speed_m_s: float):
        """(visited_nodes, visited_edges, tree_map, edge_map) as rust/src/centrality.rs:1524-1611."""
        from . import centrality

        self._validate_src(src_idx, speed_m_s)
        return centrality.tree_segment(self, src_idx, max_seconds, speed_m_s)

    def dijkstra_tree_simplest(self, src_idx: int, max_seconds: int, speed_m_s: float):
        from . import centrality

        self.validate_dual_for_angular("dijkstra_tree_simplest")
        self._validate_src(src_idx, speed_m_s)
        return centrality.tree_simplest(self, [src_idx], max_seconds, speed_m_s)[0]

    def centrality_shortest(self, distances=None, betas=None, minutes=None, compute_closeness=None,
                            compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, tolerance=None,
                            sample_probability=None, sampling_weights=None, random_seed=None, source_indices=None,
                            pbar_disabled=None):
        from . import centrality

        return self._run(
            centrality.centrality_shortest, distances=distances, betas=betas, minutes=minutes, compute_closeness=compute_closeness,
            compute_betweenness=compute_betweenness, min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s,
            tolerance=tolerance, sample_probability=sample_probability, sampling_weights=sampling_weights,
            random_seed=random_seed, source_indices=source_indices, pbar_disabled=pbar_disabled)

    def centrality_simplest(self, distances=None, betas=None, minutes=None, compute_closeness=None,
                            compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, tolerance=None,
                            angular_scaling_unit=None, farness_scaling_offset=None, sample_probability=None,
                            sampling_weights=None, random_seed=None, source_indices=None, pbar_disabled=None):
        from . import centrality

        return self._run(
            centrality.centrality_simplest, distances=distances, betas=betas, minutes=minutes, compute_closeness=compute_closeness,
            compute_betweenness=compute_betweenness, min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s,
            tolerance=tolerance, angular_scaling_unit=angular_scaling_unit,
            farness_scaling_offset=farness_scaling_offset, sample_probability=sample_probability,
            sampling_weights=sampling_weights, random_seed=random_seed, source_indices=source_indices,
            pbar_disabled=pbar_disabled)

    def segment_centrality(self, distances=None, betas=None, minutes=None, compute_closeness=None,
                           compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, pbar_disabled=None):
        from . import centrality

        return self._run(
            centrality.segment_centrality, distances=distances, betas=betas, minutes=minutes, compute_closeness=compute_closeness,
            compute_betweenness=compute_betweenness, min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s,
            pbar_disabled=pbar_disabled)

    def betweenness_od_shortest(self, od_matrix, distances=None, betas=None, minutes=None, min_threshold_wt=None,
                                speed_m_s=None, tolerance=None, pbar_disabled=None):
        from . import centrality

        return centrality.betweenness_od_shortest(
            self, od_matrix, distances=distances, betas=betas, minutes=minutes, min_threshold_wt=min_threshold_wt,
            speed_m_s=speed_m_s, tolerance=tolerance, pbar_disabled=pbar_disabled)

    # aliases under the names of earlier cityseer releases
    def local_node_centrality_shortest(self, *args, **kwargs):
        return self.centrality_shortest(*args, **kwargs)

    def local_node_centrality_simplest(self, *args, **kwargs):
        return self.centrality_simplest(*args, **kwargs)

    def local_segment_centrality(self, *args, **kwargs):
        return self.segment_centrality(*args, **kwargs)
