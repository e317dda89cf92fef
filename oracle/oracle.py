"""ctypes wrapper of the CPU oracle (oracle/cs_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline
legs as the checker.  The product (cityseer_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcs_oracle.so"

_P = C.c_void_p


class _Desc(C.Structure):
    _fields_ = [
        ("n_bound", C.c_int32), ("n_edges", C.c_int32),
        ("node_exists", _P), ("live", _P), ("weight", _P), ("has_z", _P), ("z", _P),
        ("e_src", _P), ("e_dst", _P), ("e_exists", _P), ("e_idx", _P), ("e_len", _P), ("e_ang", _P),
        ("e_imp", _P), ("e_sec", _P), ("e_shared", _P), ("is_dual", C.c_int32),
    ]


class _Args(C.Structure):
    _fields_ = [
        ("k", C.c_int32), ("distances", _P), ("betas", _P), ("seconds", _P),
        ("compute_closeness", C.c_int32), ("compute_betweenness", C.c_int32),
        ("speed", C.c_float), ("tolerance", C.c_float),
        ("angular_scaling_unit", C.c_float), ("farness_scaling_offset", C.c_float),
        ("n_sources", C.c_int64), ("sources", _P), ("eligible", _P), ("src_wt", _P), ("src_take", _P),
        ("track_reach", C.c_int32), ("nthreads", C.c_int32),
        ("od_ptr", _P), ("od_dst", _P), ("od_w", _P),
    ]


class _NVisit(C.Structure):
    _fields_ = [
        ("visited", C.c_uint8), ("discovered", C.c_uint8), ("pred", C.c_int64), ("short_dist", C.c_float),
        ("simpl_dist", C.c_float), ("origin_seg", C.c_int64), ("last_seg", C.c_int64), ("agg_seconds", C.c_float),
    ]


class _EVisit(C.Structure):
    _fields_ = [("visited", C.c_uint8), ("start", C.c_int64), ("end", C.c_int64), ("edge_idx", C.c_int64)]


_lib = None


def build() -> Path:
    """Compiles the oracle with its Makefile (gcc, -ffp-contract=off)."""
    src = HERE / "cs_oracle.c"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.og_graph_new.restype = _P
        L.og_graph_new.argtypes = [C.POINTER(_Desc)]
        L.og_graph_free.argtypes = [_P]
        L.og_slots_ok.restype = C.c_int32
        L.og_slots_ok.argtypes = [_P]
        for name in ("og_centrality_shortest", "og_centrality_simplest"):
            getattr(L, name).restype = C.c_int
            getattr(L, name).argtypes = [_P, C.POINTER(_Args), _P, _P]
        L.og_segment_centrality.restype = C.c_int
        L.og_segment_centrality.argtypes = [_P, C.POINTER(_Args), _P]
        L.og_betweenness_od.argtypes = [_P, C.POINTER(_Args), _P]
        L.og_tree_shortest.restype = C.c_int64
        L.og_tree_shortest.argtypes = [_P, C.c_int64, C.c_uint32, C.c_float, _P, _P]
        L.og_tree_simplest.restype = C.c_int64
        L.og_tree_simplest.argtypes = [_P, C.c_int64, C.c_uint32, C.c_float, _P, _P]
        L.og_tree_segment.restype = C.c_int64
        L.og_tree_segment.argtypes = [_P, C.c_int64, C.c_uint32, C.c_float, _P, _P, _P, _P, _P]
        L.og_brandes_debug.restype = C.c_int64
        L.og_brandes_debug.argtypes = [_P, C.c_int32, C.c_int64, C.c_uint32, C.c_float, C.c_float, _P, _P, _P, _P,
                                       C.c_int32, _P, _P, _P, _P]
        L.og_betas_from_distances.restype = C.c_int
        L.og_betas_from_distances.argtypes = [_P, C.c_int32, C.c_float, C.c_int32, _P]
        L.og_distances_from_betas.restype = C.c_int
        L.og_distances_from_betas.argtypes = [_P, C.c_int32, C.c_float, C.c_int32, _P]
        L.og_seconds_from_distances.restype = C.c_int
        L.og_seconds_from_distances.argtypes = [_P, C.c_int32, C.c_float, _P]
        L.og_edge_travel_seconds.restype = C.c_float
        L.og_edge_travel_seconds.argtypes = [_P, C.c_int32, C.c_float, C.c_int32]
        L.og_get_slots.argtypes = [_P, _P]
        for n in ("og_sizeof_nvisit", "og_sizeof_evisit", "og_sizeof_args", "og_sizeof_desc"):
            getattr(L, n).restype = C.c_int32
        assert L.og_sizeof_nvisit() == C.sizeof(_NVisit)
        assert L.og_sizeof_evisit() == C.sizeof(_EVisit)
        assert L.og_sizeof_args() == C.sizeof(_Args)
        assert L.og_sizeof_desc() == C.sizeof(_Desc)
        _lib = L
    return _lib


class OracleGraph:
    """An oracle graph built from a NetworkStructure's columns (arrays kept alive here)."""

    def __init__(self, ns):
        a = ns.arrays()
        self.n = int(a["n_slots"])
        self.m = len(a["e_src"])
        self.keep = {
            "node_exists": np.ascontiguousarray(a["node_exists"], np.uint8),
            "live": np.ascontiguousarray(a["live"], np.uint8),
            "weight": np.ascontiguousarray(a["weight"], np.float32),
            "has_z": np.ascontiguousarray(a["has_z"], np.uint8),
            "z": np.ascontiguousarray(a["z"], np.float64),
            "e_src": np.ascontiguousarray(a["e_src"], np.int32),
            "e_dst": np.ascontiguousarray(a["e_dst"], np.int32),
            "e_exists": np.ascontiguousarray(a["e_exists"], np.uint8),
            "e_idx": np.ascontiguousarray(a["e_idx"], np.int64),
            "e_len": np.ascontiguousarray(a["e_len"], np.float32),
            "e_ang": np.ascontiguousarray(a["e_ang"], np.float32),
            "e_imp": np.ascontiguousarray(a["e_imp"], np.float32),
            "e_sec": np.ascontiguousarray(a["e_sec"], np.float32),
            "e_shared": np.ascontiguousarray(a["e_shared"], np.int32),
        }
        d = _Desc()
        d.n_bound = ns.node_bound()
        self.nb = d.n_bound
        d.n_edges = self.m
        for k, v in self.keep.items():
            setattr(d, k, v.ctypes.data)
        d.is_dual = 1 if ns.is_dual else 0
        self.desc = d
        self.h = lib().og_graph_new(C.byref(d))

    def __del__(self):
        try:
            if self.h:
                lib().og_graph_free(self.h)
        except Exception:
            pass

    @property
    def slots_ok(self) -> bool:
        return bool(lib().og_slots_ok(self.h))

    def slots(self) -> np.ndarray:
        out = np.zeros(2 * max(self.nb, 1), np.int32)
        lib().og_get_slots(self.h, out.ctypes.data)
        return out[: 2 * self.nb].reshape(-1, 2)


def _args(nb, dists, betas, secs, speed, tol, closeness, betweenness, plan, nthreads, asu=180.0, fso=1.0):
    keep = {
        "distances": np.ascontiguousarray(dists, np.uint32),
        "betas": np.ascontiguousarray(betas, np.float32),
        "seconds": np.ascontiguousarray(secs, np.uint32),
        "sources": np.ascontiguousarray(plan["sources"], np.int64),
        "eligible": np.ascontiguousarray(plan["eligible"], np.uint8),
        "src_wt": np.ascontiguousarray(plan["src_wt"], np.float32),
        "src_take": np.ascontiguousarray(plan["src_take"], np.uint8),
    }
    a = _Args()
    a.k = len(dists)
    a.distances = keep["distances"].ctypes.data
    a.betas = keep["betas"].ctypes.data
    a.seconds = keep["seconds"].ctypes.data
    a.compute_closeness = int(bool(closeness))
    a.compute_betweenness = int(bool(betweenness))
    a.speed = speed
    a.tolerance = tol
    a.angular_scaling_unit = asu
    a.farness_scaling_offset = fso
    a.n_sources = len(keep["sources"])
    a.sources = keep["sources"].ctypes.data
    a.eligible = keep["eligible"].ctypes.data
    a.src_wt = keep["src_wt"].ctypes.data
    a.src_take = keep["src_take"].ctypes.data
    a.track_reach = int(bool(plan.get("track_reach", False)))
    a.nthreads = int(nthreads)
    return a, keep


def plan_from(sp, nb: int) -> dict:
    """Oracle source plan from the host layer's resolved SourcePlan (same sources, same weights)."""
    take = np.zeros(nb, np.uint8)
    take[sp.process] = 1
    # betweenness post-scale for a source subset without sampling (rust/src/centrality.rs:1852-1868)
    scale = 1.0
    if sp.is_source_indexed and sp.sample_probability is None and sp.n_sources > 0:
        scale = sp.n_live / sp.n_sources
    return {
        "sources": sp.process.astype(np.int64),
        "eligible": sp.eligible,
        "src_wt": sp.src_wt,
        "src_take": take,
        "track_reach": sp.sample_probability is not None or sp.is_source_indexed,
        "betweenness_scale": scale,
        "node_indices": None,
    }


def all_sources_plan(ns) -> dict:
    """The default plan: every node a source, eligible if live, weight = node weight."""
    a = ns.arrays()
    nb = ns.node_bound()
    idx = np.asarray(ns.node_indices(), np.int64)
    live = a["live"][:nb]
    return {
        "sources": idx,
        "eligible": live.astype(np.uint8),
        "src_wt": a["weight"][:nb].astype(np.float32),
        "src_take": np.ones(nb, np.uint8),
        "track_reach": False,
    }


def centrality_shortest(og: OracleGraph, dists, betas, secs, speed=1.33333, tol=1e-4, closeness=True,
                        betweenness=True, plan=None, nthreads=1, ns=None):
    plan = plan if plan is not None else all_sources_plan(ns)
    k = len(dists)
    out = np.zeros((7, k, og.nb), np.float64)
    reach = np.zeros(k, np.uint32)
    a, keep = _args(og.nb, dists, betas, secs, speed, tol, closeness, betweenness, plan, nthreads)
    rc = lib().og_centrality_shortest(og.h, C.byref(a), out.ctypes.data, reach.ctypes.data)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    _post_scale(og, out, (5, 6), plan, betweenness)
    return out, reach


def betweenness_od(og: OracleGraph, dists, betas, secs, od_rows, speed=1.33333, tol=1e-4, nthreads=1, ns=None):
    """betweenness_od_shortest (rust/src/centrality.rs:2419-2540).  od_rows = (ptr [n_bound + 1],
    dst, w): each origin node's destinations and trip weights, one entry per pair.  Returns
    [2][K][n_bound] (node_betweenness, node_betweenness_beta)."""
    plan = all_sources_plan(ns)
    k = len(dists)
    ptr = np.ascontiguousarray(od_rows[0], np.int64)
    dst = np.ascontiguousarray(od_rows[1], np.int64)
    w = np.ascontiguousarray(od_rows[2], np.float32)
    if len(dst) and (dst.min() < 0 or dst.max() >= og.nb):
        raise ValueError("OD destination is not a node index")
    out = np.zeros((2, k, og.nb), np.float64)
    a, keep = _args(og.nb, dists, betas, secs, speed, tol, False, True, plan, nthreads)
    keep["od"] = (ptr, dst, w)
    a.od_ptr = ptr.ctypes.data
    a.od_dst = dst.ctypes.data if len(dst) else None
    a.od_w = w.ctypes.data if len(w) else None
    if not len(dst):
        return out
    if lib().og_betweenness_od(og.h, C.byref(a), out.ctypes.data) != 0:
        raise ValueError("oracle rejected the arguments")
    return out


def _post_scale(og, out, rows, plan, betweenness):
    sc = plan.get("betweenness_scale", 1.0)
    if betweenness and sc != 1.0:
        idx = np.nonzero(og.keep["node_exists"][: og.nb])[0]
        for r in rows:
            out[r][:, idx] *= sc


def centrality_simplest(og: OracleGraph, dists, betas, secs, speed=1.33333, tol=1e-4, closeness=True,
                        betweenness=True, plan=None, nthreads=1, ns=None, asu=180.0, fso=1.0):
    plan = plan if plan is not None else all_sources_plan(ns)
    k = len(dists)
    out = np.zeros((4, k, og.nb), np.float64)
    reach = np.zeros(k, np.uint32)
    a, keep = _args(og.nb, dists, betas, secs, speed, tol, closeness, betweenness, plan, nthreads, asu, fso)
    rc = lib().og_centrality_simplest(og.h, C.byref(a), out.ctypes.data, reach.ctypes.data)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    _post_scale(og, out, (3,), plan, betweenness)
    return out, reach


def segment_centrality(og: OracleGraph, dists, betas, secs, speed=1.33333, closeness=True, betweenness=True,
                       ns=None, nthreads=1):
    plan = all_sources_plan(ns)
    k = len(dists)
    out = np.zeros((4, k, og.nb), np.float64)
    a, keep = _args(og.nb, dists, betas, secs, speed, 1e-4, closeness, betweenness, plan, nthreads)
    rc = lib().og_segment_centrality(og.h, C.byref(a), out.ctypes.data)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return out


def _tree_arrays(tree, n):
    return {
        "visited": np.array([tree[i].visited for i in range(n)], bool),
        "pred": np.array([tree[i].pred for i in range(n)], np.int64),
        "short_dist": np.array([tree[i].short_dist for i in range(n)], np.float32),
        "simpl_dist": np.array([tree[i].simpl_dist for i in range(n)], np.float32),
        "agg_seconds": np.array([tree[i].agg_seconds for i in range(n)], np.float32),
        "origin_seg": np.array([tree[i].origin_seg for i in range(n)], np.int64),
        "last_seg": np.array([tree[i].last_seg for i in range(n)], np.int64),
    }


def tree_shortest(og: OracleGraph, src: int, max_seconds: int, speed: float):
    visited = np.zeros(max(og.nb, 1), np.int64)
    tree = (_NVisit * max(og.nb, 1))()
    nv = lib().og_tree_shortest(og.h, src, max_seconds, speed, visited.ctypes.data, C.addressof(tree))
    return visited[:nv].copy(), _tree_arrays(tree, og.nb)


def tree_simplest(og: OracleGraph, src: int, max_seconds: int, speed: float):
    visited = np.zeros(max(og.nb, 1), np.int64)
    tree = (_NVisit * max(og.nb, 1))()
    nv = lib().og_tree_simplest(og.h, src, max_seconds, speed, visited.ctypes.data, C.addressof(tree))
    return visited[:nv].copy(), _tree_arrays(tree, og.nb)


def tree_segment(og: OracleGraph, src: int, max_seconds: int, speed: float):
    visited = np.zeros(max(og.nb, 1), np.int64)
    vedges = np.zeros(og.m + 1, np.int64)
    nve = C.c_int64()
    tree = (_NVisit * max(og.nb, 1))()
    emap = (_EVisit * (og.m + 1))()
    nv = lib().og_tree_segment(og.h, src, max_seconds, speed, visited.ctypes.data, C.addressof(tree),
                               vedges.ctypes.data, C.byref(nve), C.addressof(emap))
    return visited[:nv].copy(), vedges[: nve.value].copy(), _tree_arrays(tree, og.nb)


def brandes_debug(og: OracleGraph, src: int, max_seconds: int, speed: float, tol: float = 1e-4,
                  angular: bool = False, pmax: int = 32):
    ns_ = og.nb * (2 if angular else 1)
    agg = np.zeros(ns_, np.float32)
    route = np.zeros(ns_, np.float32)
    npred = np.zeros(ns_, np.int32)
    preds = np.zeros(ns_ * pmax, np.int64)
    sigma = np.zeros(ns_, np.float64)
    order = np.zeros(ns_, np.int64)
    brc = np.zeros(og.nb, np.float32)
    bas = np.zeros(og.nb, np.float32)
    nv = lib().og_brandes_debug(og.h, int(angular), src, max_seconds, speed, tol, agg.ctypes.data, route.ctypes.data,
                                npred.ctypes.data, preds.ctypes.data, pmax, sigma.ctypes.data, order.ctypes.data,
                                brc.ctypes.data, bas.ctypes.data)
    if nv < 0:
        raise ValueError("a state has more predecessors than pmax")
    return {
        "agg_seconds": agg, "route_cost": route, "npred": npred, "preds": preds.reshape(ns_, pmax),
        "sigma": sigma, "order": order[:nv].copy(), "best_route_cost": brc, "best_agg_seconds": bas,
    }


def betas_from_distances(dists, mtw=None):
    d = np.ascontiguousarray(dists, np.uint32)
    out = np.zeros(len(d), np.float32)
    rc = lib().og_betas_from_distances(d.ctypes.data, len(d), C.c_float(mtw or 0.0), int(mtw is not None),
                                       out.ctypes.data)
    if rc != 0:
        raise ValueError("invalid distances")
    return out


def distances_from_betas(betas, mtw=None):
    b = np.ascontiguousarray(betas, np.float32)
    out = np.zeros(len(b), np.uint32)
    rc = lib().og_distances_from_betas(b.ctypes.data, len(b), C.c_float(mtw or 0.0), int(mtw is not None),
                                       out.ctypes.data)
    if rc != 0:
        raise ValueError("invalid betas")
    return out


def seconds_from_distances(dists, speed):
    d = np.ascontiguousarray(dists, np.uint32)
    out = np.zeros(len(d), np.uint32)
    rc = lib().og_seconds_from_distances(d.ctypes.data, len(d), C.c_float(speed), out.ctypes.data)
    if rc != 0:
        raise ValueError("invalid distances")
    return out


def default_threads() -> int:
    return max(1, (os.cpu_count() or 2) - 1)


class _Data(C.Structure):
    _fields_ = [("n_entries", C.c_int64), ("n_groups", C.c_int64), ("nd_ptr", _P), ("nd_entry", _P),
                ("nd_dist", _P), ("entry_group", _P)]


def _data_struct(t):
    keep = {
        "nd_ptr": np.ascontiguousarray(t["ptr"], np.int64),
        "nd_entry": np.ascontiguousarray(t["a_entry"], np.int64),
        "nd_dist": np.ascontiguousarray(t["a_dist"], np.float64),
        "entry_group": np.ascontiguousarray(t["entry_group"], np.int64),
    }
    dd = _Data()
    dd.n_entries = len(t["keys"])
    dd.n_groups = int(t["n_groups"])
    for k, v in keep.items():
        setattr(dd, k, v.ctypes.data if len(v) else None)
    return dd, keep


def aggregate(og: OracleGraph, t: dict, src: int, max_seconds: int, speed: float, angular: bool = False):
    """aggregate_to_src_idx (rust/src/data.rs:513-602) on the tables of DataMap._tables: f32 total
    distance per entry, NaN when not reachable."""
    L = lib()
    L.og_aggregate.restype = C.c_int64
    L.og_aggregate.argtypes = [_P, C.POINTER(_Data), C.c_int64, C.c_uint32, C.c_float, C.c_int32, _P, _P, _P]
    dd, keep = _data_struct(t)
    ne, ng = len(t["keys"]), int(t["n_groups"])
    out = np.zeros(max(ne, 1), np.float32)
    gb = np.zeros(max(ng, 1), np.float32)
    ge = np.zeros(max(ng, 1), np.int64)
    L.og_aggregate(og.h, C.byref(dd), int(src), int(max_seconds), C.c_float(speed), int(bool(angular)),
                   out.ctypes.data, gb.ctypes.data, ge.ctypes.data)
    return out[:ne]


def accessibility(og: OracleGraph, t: dict, n_classes: int, dists, betas, mcw, max_seconds: int, speed: float,
                  angular: bool = False):
    """accessibility (rust/src/data.rs:605-740): unweighted, weighted [C][K][n_bound] and nearest
    [C][n_bound] (NaN when none) for every live node."""
    L = lib()
    L.og_accessibility.restype = C.c_int
    L.og_accessibility.argtypes = [_P, C.POINTER(_Data), _P, C.c_int32, C.c_int32, _P, _P, _P, C.c_uint32, C.c_float,
                                   C.c_int32, _P, _P, _P]
    dd, keep = _data_struct(t)
    k = len(dists)
    cls = np.ascontiguousarray(t["entry_class"], np.int32)
    dist_a = np.ascontiguousarray(dists, np.uint32)
    beta_a = np.ascontiguousarray(betas, np.float32)
    mcw_a = np.ascontiguousarray(mcw, np.float32)
    u = np.zeros((n_classes, k, og.nb))
    w = np.zeros((n_classes, k, og.nb))
    n = np.full((n_classes, og.nb), np.nan)
    L.og_accessibility(og.h, C.byref(dd), cls.ctypes.data, int(n_classes), k, dist_a.ctypes.data, beta_a.ctypes.data,
                       mcw_a.ctypes.data, int(max_seconds), C.c_float(speed), int(bool(angular)), u.ctypes.data,
                       w.ctypes.data, n.ctypes.data)
    return u, w, n
