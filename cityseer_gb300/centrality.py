"""Centrality drivers and result classes (the reference's rust/src/centrality.rs surface).

Host logic mirrored here, kernels in libcsgpu.so:
  validate_tolerance          rust/src/centrality.rs:34-48
  prepare_source_sampling     rust/src/centrality.rs:1032-1104 (random stream: stdrng.StdRng)
  sample_source_weight        rust/src/centrality.rs:1107-1139
  scale_metric_results        rust/src/centrality.rs:875-893 (betweenness post-scale)
  result getters              rust/src/centrality.rs:152-355, MetricResult.load_compact common.rs:37-53
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import _native, device
from .common import WALKING_SPEED, pair_distances_betas_time
from .stdrng import StdRng
from .graph import NodeVisit

TIE_EPSILON = np.float32(1e-4)
TOLERANCE_WARN_PCT = 2.0


def validate_tolerance(tolerance: float | None) -> float:
    """Percent -> decimal, clamped to at least TIE_EPSILON (rust/src/centrality.rs:34-48)."""
    pct = np.float32(0.0 if tolerance is None else tolerance)
    if pct < 0.0 or pct > 100.0:
        raise ValueError(f"Tolerance must be between 0 and 100 (percent), got {tolerance}")
    return float(max(np.float32(pct / np.float32(100.0)), TIE_EPSILON))


# ---------------------------------------------------------------------------------------------
# Results
# ---------------------------------------------------------------------------------------------
class _Result:
    _rows: tuple[str, ...] = ()

    def __init__(self, distances, node_keys_py, node_indices, data: np.ndarray):
        self.distances = list(distances)
        self._keys = node_keys_py
        self._idx = np.asarray(node_indices, dtype=np.int64)
        self._data = data  # [M][K][node_bound] f64
        self._keys_list: list | None = None
        self._idx_list: list[int] | None = None
        self.reachability_totals: list[int] = []
        self.sampled_source_count = 0

    # the key and index lists are built on first access (large graphs: a few ms each)
    @property
    def node_keys_py(self) -> list:
        if self._keys_list is None:
            self._keys_list = list(self._keys)
        return self._keys_list

    @property
    def node_indices(self) -> list[int]:
        if self._idx_list is None:
            self._idx_list = self._idx.tolist()
        return self._idx_list

    def _load_compact(self, m: int) -> dict[int, np.ndarray]:
        return {d: self._data[m, i][self._idx].copy() for i, d in enumerate(self.distances)}

    def __getattr__(self, name):
        rows = type(self)._rows
        if name in rows:
            return self._load_compact(rows.index(name))
        raise AttributeError(name)


class CentralityShortestResult(_Result):
    _rows = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
             "node_betweenness_beta")


class CentralitySimplestResult(_Result):
    _rows = ("node_density", "node_farness", "node_harmonic", "node_betweenness")


class CentralitySegmentResult(_Result):
    _rows = ("segment_density", "segment_harmonic", "segment_beta", "segment_betweenness")


class BetweennessShortestResult(_Result):
    """Result of betweenness_od_shortest (rust/src/centrality.rs:94-150)."""
    _rows = ("node_betweenness", "node_betweenness_beta")


class OdMatrix:
    """Sparse origin-destination trip weights (rust/src/centrality.rs:56-91), from parallel arrays of
    origin node indices, destination node indices and weights (COO).  A repeated (origin,
    destination) pair keeps the weight given last, as the reference's map insert does.  Stored as
    pairs sorted by (origin, destination); weights are f32."""

    def __init__(self, origins, destinations, weights):
        if not (len(origins) == len(destinations) == len(weights)):
            raise ValueError(f"origins ({len(origins)}), destinations ({len(destinations)}), and weights "
                             f"({len(weights)}) must have equal length")
        o = np.asarray(origins, dtype=np.int64).reshape(-1)
        d = np.asarray(destinations, dtype=np.int64).reshape(-1)
        w = np.asarray(weights, dtype=np.float64).reshape(-1).astype(np.float32)
        if (len(o) and o.min() < 0) or (len(d) and d.min() < 0):
            raise OverflowError("can't convert negative int to unsigned")
        order = np.lexsort((np.arange(len(o)), d, o))
        o, d, w = o[order], d[order], w[order]
        last = np.ones(len(o), bool)
        if len(o) > 1:
            last[:-1] = (o[1:] != o[:-1]) | (d[1:] != d[:-1])
        self.origins, self.destinations, self.weights = o[last], d[last], w[last]

    def len(self) -> int:
        return int(len(self.origins))

    def n_origins(self) -> int:
        return int(len(np.unique(self.origins)))

    def rows(self, n_bound: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(ptr [n_bound + 1], destinations, weights): each origin node's row, destinations
        ascending.  Origins at or beyond n_bound have no row (the reference never looks them up)."""
        keep = self.origins < n_bound
        o = self.origins[keep]
        ptr = np.zeros(n_bound + 1, np.int64)
        np.cumsum(np.bincount(o, minlength=n_bound), out=ptr[1:])
        return ptr, self.destinations[keep], self.weights[keep]


# ---------------------------------------------------------------------------------------------
# Source sampling plan
# ---------------------------------------------------------------------------------------------
@dataclass
class SourcePlan:
    process: np.ndarray       # node indices handed to the kernel, in order
    src_wt: np.ndarray        # f32 [node_bound]
    eligible: np.ndarray      # u8 [node_bound]
    is_source_indexed: bool
    sample_probability: float | None
    n_sources: int
    n_live: int
    sampled_count: int


def prepare_source_sampling(ns, sample_probability, sampling_weights, random_seed, source_indices) -> SourcePlan:
    nb = ns.node_bound()
    nc = ns.node_count()
    node_indices = ns._node_index_array()
    a = ns.arrays()
    live = a["live"][:nb].astype(bool)
    weight = a["weight"][:nb]
    sw = None
    if sampling_weights is not None:
        w = np.asarray(sampling_weights, dtype=np.float32)
        if len(w) not in (nb, nc):
            raise ValueError(
                f"sampling_weights length ({len(w)}) must match node_count ({nc}) or node_bound ({nb})")
        bad = np.nonzero((w < 0.0) | (w > 1.0))[0]
        if len(bad):
            raise ValueError(f"sampling_weights[{bad[0]}] = {w[bad[0]]} is out of range [0.0, 1.0]")
        if len(w) == nb:
            sw = w
        else:
            sw = np.zeros(nb, np.float32)
            sw[node_indices] = w
    prob = None
    if sample_probability is not None:
        prob = np.float32(sample_probability)
        if prob <= 0.0 or prob > 1.0:
            raise ValueError("sample_probability must be in (0.0, 1.0]")
    if source_indices is not None and sw is not None:
        raise ValueError("source_indices and sampling_weights are mutually exclusive")
    exists = a["node_exists"]
    if source_indices is not None:
        src = np.asarray(list(source_indices), dtype=np.int64)
        for s in src:
            if s < 0 or s >= nb or not exists[s]:
                raise ValueError(f"node index {int(s)} does not exist in the graph")
    n_live = int(live[node_indices].sum())
    is_indexed = source_indices is not None
    sources = src if is_indexed else node_indices
    eligible = np.zeros(nb, np.uint8)
    if is_indexed:
        eligible[sources] = 1
    else:
        eligible[node_indices[live[node_indices]]] = 1
    randoms = None
    if prob is not None and not is_indexed:
        # one f32 per node index from rand's StdRng (rust/src/centrality.rs:1082-1091): a seeded
        # run samples the same sources as the reference; unseeded, the seed comes from the OS
        rng = StdRng.seed_from_u64(int(random_seed)) if random_seed is not None else StdRng(os.urandom(32))
        randoms = rng.random_f32(nb)
    # sample_source_weight (rust/src/centrality.rs:1107-1139) for every listed source at once, in f32
    src_wt = np.zeros(nb, np.float32)
    take = eligible[sources] == 1
    wt = weight[sources].astype(np.float32)
    count = 0
    if is_indexed:
        if prob is not None:
            wt = (wt / prob).astype(np.float32)
        count = int(take.sum())
    elif prob is not None:
        p = np.full(len(sources), prob, np.float32)
        if sw is not None:
            p = (p * sw[sources]).astype(np.float32)
        take &= (p > 0.0) & (randoms[sources] < p)
        wt = np.where(take, wt / np.where(p > 0.0, p, np.float32(1.0)), wt).astype(np.float32)
        count = int(take.sum())
    src_wt[sources[take]] = wt[take]
    return SourcePlan(
        process=sources[take].astype(np.int32),
        src_wt=src_wt,
        eligible=eligible,
        is_source_indexed=is_indexed,
        sample_probability=None if prob is None else float(prob),
        n_sources=len(sources),
        n_live=n_live,
        sampled_count=count,
    )


# ---------------------------------------------------------------------------------------------
# Device state cache per NetworkStructure
# ---------------------------------------------------------------------------------------------
def _primal_host(ns) -> device.PrimalHost:
    c = ns._cache.get("primal_host")
    if c is None:
        c = device.PrimalHost(ns)
        ns._cache["primal_host"] = c
    return c


def _primal_csr(ns) -> device.PrimalCSR:
    """Device CSR of the graph, uploaded on first use and kept resident until the graph changes
    (or drop_device_state() is called)."""
    c = ns._cache.get("primal_csr")
    if c is None:
        c = device.PrimalCSR(_primal_host(ns))
        ns._cache["primal_csr"] = c
    return c


def drop_device_state(ns, keep_workspace: bool = True) -> None:
    """Forgets the device-resident CSR (and optionally the workspaces) of a graph."""
    for k in list(ns._cache):
        if k == "primal_csr" or k == "dual_csr" or (not keep_workspace and k in ("ws", "wsd")):
            del ns._cache[k]


def estimate_reach(ns, csr, speed: float, max_seconds: int, n_samples: int = 48) -> int:
    """Largest reach (nodes settled) over an even sample of sources, from the tree kernel run with
    one-wide rows (it then reports only the count)."""
    key = ("reach", float(np.float32(speed)), int(max_seconds))
    hit = ns._cache.get(key)
    if hit is not None:
        return hit
    idx = ns._node_index_array()
    if len(idx) == 0:
        return 1
    pick = idx[np.linspace(0, len(idx) - 1, min(n_samples, len(idx))).astype(np.int64)]
    lib = _native.load()
    plan = device.plan_primal(csr, 2, 1, speed, cap=csr.n_bound, max_slots=len(pick))
    ws = device.Workspace(plan, csr.n_bound, csr.device)
    dev = csr.device
    src_t = torch.from_numpy(pick.astype(np.int32)).to(dev)
    count = torch.zeros(len(pick), dtype=torch.int32, device=dev)
    scratch = torch.zeros(len(pick), dtype=torch.int32, device=dev)
    aggs = torch.zeros(len(pick), dtype=torch.float32, device=dev)
    rc = lib.cs_tree_shortest(C.byref(csr.struct(speed)), len(pick), src_t.data_ptr(), int(max_seconds),
                              C.c_float(speed), C.byref(plan), ws.ptr, ws.nbytes, 1, count.data_ptr(),
                              scratch.data_ptr(), aggs.data_ptr(), scratch.data_ptr(), _stream_ptr())
    _native.check(rc, "reach estimate")
    r = int(np.abs(count.cpu().numpy()).max())
    del ws
    ns._cache[key] = r
    return r


def _mem_budget(device_: torch.device) -> int:
    free, total = torch.cuda.mem_get_info(device_)
    return int(min(free * 0.6, 96 << 30))


def _lanes_for(mode: int, k: int) -> int:
    return 2 * k if mode == 0 else (k if mode == 1 else 1)


def _workspace(ns, csr, mode: int, k: int, speed: float, max_seconds: int | None = None) -> device.Workspace:
    """The graph's workspace, grown (never shrunk) to the lanes and reach capacity this call needs,
    so calls that vary thresholds or modes reuse one allocation."""
    cap = 0
    if max_seconds is not None and mode != 2:
        r = estimate_reach(ns, csr, speed, max_seconds)
        cap = int(min(csr.n_bound, max(1024, -(-int(r * 1.3) // 256) * 256)))
    need_l = _lanes_for(mode, k)
    ws = ns._cache.get("ws")
    if ws is not None and ws.plan.lanes >= need_l and ws.plan.cap >= cap:
        return ws
    if ws is not None:
        need_l = max(need_l, int(ws.plan.lanes))
        cap = max(cap, int(ws.plan.cap))
        del ns._cache["ws"]
        del ws
    torch.cuda.empty_cache()
    plan = device.plan_primal(csr, 0, (need_l + 1) // 2, speed, cap=cap, mem_budget=_mem_budget(csr.device))
    ws = device.Workspace(plan, csr.n_bound, csr.device)
    ns._cache["ws"] = ws
    return ws


def _groups(k: int):
    """Threshold groups of at most CS_MAX_THRESHOLDS (each group is one launch)."""
    step = _native.MAX_K
    return [(i, min(k, i + step)) for i in range(0, k, step)]


def _cutoff_groups(k: int):
    """Launch groups for the modes whose results at a threshold depend on the search cutoff, which
    the reference sets to the largest threshold for all of them: simplest paths (the cutoff prunes
    by metric seconds while routes are ordered by angle) and segment betweenness (a target beyond a
    threshold still credits it when its first and last segments are long).  Each group is
    (lo, hi, sel): thresholds lo..hi-1 are returned, sel lists the thresholds launched, and a group
    that does not end at the largest threshold carries it as a hidden last lane."""
    if k <= _native.MAX_K:
        return [(0, k, list(range(k)))]
    step = _native.MAX_K - 1
    out = []
    for lo in range(0, k, step):
        hi = min(k, lo + step)
        out.append((lo, hi, list(range(lo, hi)) + ([k - 1] if hi < k else [])))
    return out


def _make_query(dists, betas, secs, speed, tol, closeness, betweenness, track_reach, proc_t, wt_t, el_t,
                asu=180.0, fso=1.0) -> _native.Query:
    q = _native.Query()
    q.k = len(dists)
    for i, (d, b, s) in enumerate(zip(dists, betas, secs)):
        q.distances[i] = int(d)
        q.betas[i] = float(b)
        q.seconds[i] = int(s)
    q.speed_m_s = float(speed)
    q.tolerance = float(tol)
    q.angular_scaling_unit = float(asu)
    q.farness_scaling_offset = float(fso)
    q.compute_closeness = 1 if closeness else 0
    q.compute_betweenness = 1 if betweenness else 0
    q.track_reach = 1 if track_reach else 0
    q.n_sources = int(proc_t.numel())
    q.sources = proc_t.data_ptr() if proc_t.numel() else None
    q.src_wt = wt_t.data_ptr()
    q.eligible = el_t.data_ptr()
    q._keep = (proc_t, wt_t, el_t)  # the device arrays must outlive every launch using q
    return q


def _stream_ptr():
    return torch.cuda.current_stream().cuda_stream


# ---------------------------------------------------------------------------------------------
# centrality_shortest (rust/src/centrality.rs:1624-1874)
# ---------------------------------------------------------------------------------------------
def centrality_shortest(ns, distances=None, betas=None, minutes=None, compute_closeness=None,
                        compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, tolerance=None,
                        sample_probability=None, sampling_weights=None, random_seed=None, source_indices=None,
                        pbar_disabled=None) -> CentralityShortestResult:
    closeness = True if compute_closeness is None else bool(compute_closeness)
    betweenness = True if compute_betweenness is None else bool(compute_betweenness)
    if not closeness and not betweenness:
        raise ValueError(
            "Either or both closeness and betweenness flags is required, but both parameters are False.")
    speed = WALKING_SPEED if speed_m_s is None else float(speed_m_s)
    tol = validate_tolerance(tolerance)
    dists, bets, secs = pair_distances_betas_time(speed, distances, betas, minutes, min_threshold_wt)
    sp = prepare_source_sampling(ns, sample_probability, sampling_weights, random_seed, source_indices)
    track = sp.sample_probability is not None or sp.is_source_indexed
    rows, reach = shortest_rows(ns, sp, sp.process, dists, bets, secs, speed, tol, closeness, betweenness, track)
    return finish_shortest(ns, dists, sp, rows.cpu().numpy(), reach.cpu().numpy(), betweenness, track)


def finish_shortest(ns, dists, sp: SourcePlan, data: np.ndarray, reach_tot: np.ndarray, betweenness: bool,
                    track: bool) -> CentralityShortestResult:
    """Post-scale of betweenness for source subsets (rust/src/centrality.rs:1852-1868) and the
    result object of centrality_shortest."""
    node_indices = ns._node_index_array()
    if betweenness and sp.is_source_indexed and sp.sample_probability is None and sp.n_sources > 0:
        scale = sp.n_live / sp.n_sources
        if scale != 1.0:
            data[5][:, node_indices] *= scale
            data[6][:, node_indices] *= scale
    ns._progress = sp.n_sources
    res = CentralityShortestResult(dists, ns.node_keys_py(), node_indices, data)
    if track:
        res.sampled_source_count = sp.sampled_count
        res.reachability_totals = [int(x) for x in reach_tot]
    return res


def shortest_rows(ns, sp: SourcePlan, process: np.ndarray, dists, bets, secs, speed: float, tol: float,
                  closeness: bool, betweenness: bool, track: bool):
    """The device rows of centrality_shortest for the sources `process` under the plan `sp` (its
    eligibility and source weights): ([7][K][N] f64, [K] i64 reach counts) on the graph's device,
    before any post-scale.  The sharded multi-GPU form runs one slice of a plan's sources per rank
    through it."""
    nb = ns.node_bound()
    K = len(dists)
    csr = _primal_csr(ns)
    dev = csr.device
    proc_t = torch.from_numpy(np.ascontiguousarray(process, np.int32)).to(dev)
    wt_t = torch.from_numpy(sp.src_wt).to(dev)
    el_t = torch.from_numpy(sp.eligible).to(dev)
    g = csr.struct(speed)
    lib = _native.load()
    groups = _groups(K)
    rows = torch.zeros((7, K, nb), dtype=torch.float64, device=dev) if len(groups) > 1 else None
    reach_all = torch.zeros(K, dtype=torch.int64, device=dev)
    for lo, hi in groups:
        k = hi - lo
        ws = _workspace(ns, csr, 0, k, speed, max(secs[lo:hi]))
        out = torch.zeros((7, k, nb), dtype=torch.float64, device=dev)
        reach = torch.zeros(k, dtype=torch.int32, device=dev)
        q = _make_query(dists[lo:hi], bets[lo:hi], secs[lo:hi], speed, tol, closeness, betweenness, track,
                        proc_t, wt_t, el_t)
        o = _native.Outputs(out.data_ptr(), reach.data_ptr())
        rc = lib.cs_centrality_shortest(C.byref(g), C.byref(q), C.byref(ws.plan), ws.ptr, ws.nbytes, o,
                                        _stream_ptr())
        if rc != _native.CS_OK:
            ws.init(_stream_ptr())
        _native.check(rc, "cs_centrality_shortest")
        if rows is None:
            rows = out
        else:
            rows[:, lo:hi] = out
        reach_all[lo:hi] = reach.to(torch.int64)
    return rows, reach_all


# ---------------------------------------------------------------------------------------------
# betweenness_od_shortest (rust/src/centrality.rs:2419-2540)
# ---------------------------------------------------------------------------------------------
def betweenness_od_shortest(ns, od_matrix: OdMatrix, distances=None, betas=None, minutes=None,
                            min_threshold_wt=None, speed_m_s=None, tolerance=None,
                            pbar_disabled=None) -> BetweennessShortestResult:
    """Shortest-path betweenness weighted by origin-destination trips: a search from every live
    origin with a row; each reached destination within a threshold seeds the backward sweep with
    its trip weight (and the weight times exp(-beta d) for the beta row)."""
    speed = WALKING_SPEED if speed_m_s is None else float(speed_m_s)
    dists, bets, secs = pair_distances_betas_time(speed, distances, betas, minutes, min_threshold_wt)
    tol = validate_tolerance(tolerance)
    nb = ns.node_bound()
    node_indices = ns._node_index_array()
    K = len(dists)
    ptr, dst, w = od_matrix.rows(nb)
    idx = node_indices
    live = ns.arrays()["live"][:nb]
    has_row = ptr[1:] > ptr[:-1]
    proc = idx[(live[idx] == 1) & has_row[idx]].astype(np.int32)
    if len(proc):
        # a destination beyond the node bound in a processed row is an index error in the reference
        processed = np.zeros(nb, bool)
        processed[proc] = True
        used = dst[np.repeat(processed, np.diff(ptr))]
        if len(used) and used.max() >= nb:
            raise ValueError(f"OD destination {int(used.max())} is not a node index (node_bound {nb})")
    data = np.zeros((2, K, nb), np.float64)
    ns._progress = len(node_indices)
    res = BetweennessShortestResult(dists, ns.node_keys_py(), node_indices, data)
    if not len(proc):
        return res
    csr = _primal_csr(ns)
    dev = csr.device
    ptr_t = torch.from_numpy(ptr.astype(np.int32)).to(dev)
    dst_t = torch.from_numpy(np.clip(dst, 0, nb).astype(np.int32)).to(dev)
    w_t = torch.from_numpy(w).to(dev)
    proc_t = torch.from_numpy(proc).to(dev)
    dummy_w = torch.zeros(1, dtype=torch.float32, device=dev)
    dummy_e = torch.zeros(1, dtype=torch.uint8, device=dev)
    g = csr.struct(speed)
    lib = _native.load()
    for lo, hi in _groups(K):
        k = hi - lo
        ws = _workspace(ns, csr, 0, k, speed, max(secs[lo:hi]))
        out = torch.zeros((2, k, nb), dtype=torch.float64, device=dev)
        q = _make_query(dists[lo:hi], bets[lo:hi], secs[lo:hi], speed, tol, False, True, False, proc_t, dummy_w,
                        dummy_e)
        o = _native.Outputs(out.data_ptr(), 0)
        rc = lib.cs_betweenness_od_shortest(C.byref(g), C.byref(q), ptr_t.data_ptr(), dst_t.data_ptr(),
                                            w_t.data_ptr(), C.byref(ws.plan), ws.ptr, ws.nbytes, o, _stream_ptr())
        if rc != _native.CS_OK:
            ws.init(_stream_ptr())
        _native.check(rc, "cs_betweenness_od_shortest")
        data[:, lo:hi] = out.cpu().numpy()
    return res


# ---------------------------------------------------------------------------------------------
# centrality_simplest (rust/src/centrality.rs:1880-2132)
# ---------------------------------------------------------------------------------------------
def centrality_simplest(ns, distances=None, betas=None, minutes=None, compute_closeness=None,
                        compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, tolerance=None,
                        angular_scaling_unit=None, farness_scaling_offset=None, sample_probability=None,
                        sampling_weights=None, random_seed=None, source_indices=None,
                        pbar_disabled=None) -> CentralitySimplestResult:
    from . import dual

    ns.validate_dual_for_angular("centrality_simplest")
    closeness = True if compute_closeness is None else bool(compute_closeness)
    betweenness = True if compute_betweenness is None else bool(compute_betweenness)
    tol = validate_tolerance(tolerance)
    if not closeness and not betweenness:
        raise ValueError(
            "Either or both closeness and betweenness flags is required, but both parameters are False.")
    speed = WALKING_SPEED if speed_m_s is None else float(speed_m_s)
    asu = 180.0 if angular_scaling_unit is None else float(angular_scaling_unit)
    fso = 1.0 if farness_scaling_offset is None else float(farness_scaling_offset)
    dists, bets, secs = pair_distances_betas_time(speed, distances, betas, minutes, min_threshold_wt)
    sp = prepare_source_sampling(ns, sample_probability, sampling_weights, random_seed, source_indices)
    return dual.run_simplest(ns, dists, bets, secs, speed, tol, asu, fso, closeness, betweenness, sp)


# ---------------------------------------------------------------------------------------------
# segment_centrality (rust/src/centrality.rs:2134-2407)
# ---------------------------------------------------------------------------------------------
def segment_centrality(ns, distances=None, betas=None, minutes=None, compute_closeness=None,
                       compute_betweenness=None, min_threshold_wt=None, speed_m_s=None,
                       pbar_disabled=None) -> CentralitySegmentResult:
    speed = WALKING_SPEED if speed_m_s is None else float(speed_m_s)
    dists, bets, secs = pair_distances_betas_time(speed, distances, betas, minutes, min_threshold_wt)
    closeness = True if compute_closeness is None else bool(compute_closeness)
    betweenness = True if compute_betweenness is None else bool(compute_betweenness)
    if not closeness and not betweenness:
        raise ValueError(
            "Either or both closeness and betweenness flags is required, but both parameters are False.")
    rows = segment_rows(ns, segment_sources(ns), dists, bets, secs, speed, closeness, betweenness)
    return finish_segment(ns, dists, rows.cpu().numpy())


def segment_sources(ns) -> np.ndarray:
    """The live nodes, in node-index order: segment centrality's sources (rust/src/centrality.rs:2190)."""
    idx = ns._node_index_array()
    return idx[ns.arrays()["live"][idx] == 1].astype(np.int32)


def segment_rows(ns, process, dists, bets, secs, speed: float, closeness: bool, betweenness: bool):
    """The device rows of segment_centrality ([4][K][N] f64) for the sources `process`.  Every launch
    searches to the largest threshold (segment betweenness depends on the cutoff)."""
    nb = ns.node_bound()
    K = len(dists)
    csr = _primal_csr(ns)
    if csr.has_missing_reverse:
        raise ValueError("Edge not found")
    dev = csr.device
    proc_t = torch.from_numpy(np.ascontiguousarray(process, np.int32)).to(dev)
    wt_t = torch.zeros(max(nb, 1), dtype=torch.float32, device=dev)
    el_t = torch.zeros(max(nb, 1), dtype=torch.uint8, device=dev)
    g = csr.struct(speed)
    lib = _native.load()
    groups = _cutoff_groups(K)
    rows = torch.zeros((4, K, nb), dtype=torch.float64, device=dev) if len(groups) > 1 else None
    for lo, hi, sel in groups:
        k = len(sel)
        gd, gb, gs = [dists[i] for i in sel], [bets[i] for i in sel], [secs[i] for i in sel]
        ws = _workspace(ns, csr, 1, k, speed, max(gs))
        out = torch.zeros((4, k, nb), dtype=torch.float64, device=dev)
        q = _make_query(gd, gb, gs, speed, float(TIE_EPSILON), closeness, betweenness, False, proc_t, wt_t, el_t)
        o = _native.Outputs(out.data_ptr(), None)
        rc = lib.cs_segment_centrality(C.byref(g), C.byref(q), C.byref(ws.plan), ws.ptr, ws.nbytes, o,
                                       _stream_ptr())
        if rc != _native.CS_OK:
            ws.init(_stream_ptr())
        _native.check(rc, "cs_segment_centrality")
        if rows is None:
            rows = out
        else:
            rows[:, lo:hi] = out[:, : hi - lo]
    return rows


def finish_segment(ns, dists, data: np.ndarray) -> CentralitySegmentResult:
    node_indices = ns._node_index_array()
    ns._progress = len(node_indices)
    return CentralitySegmentResult(dists, ns.node_keys_py(), node_indices, data)


# ---------------------------------------------------------------------------------------------
# Trees (isochrones): dijkstra_tree_shortest (rust/src/centrality.rs:1141-1200, 1500-1508)
# ---------------------------------------------------------------------------------------------
def tree_shortest_raw(ns, sources: list[int], max_seconds: int, speed: float, row_cap: int | None = None):
    """Batched trees on the GPU: returns (counts, nodes, agg_seconds, preds) numpy arrays, rows in
    settle order, row_cap wide."""
    csr = _primal_csr(ns)
    dev = csr.device
    nb = csr.n_bound
    nq = len(sources)
    if row_cap is None:
        row_cap = nb
    lib = _native.load()
    g = csr.struct(speed)
    ws = _workspace(ns, csr, 2, 1, speed)
    src_t = torch.tensor(sources, dtype=torch.int32, device=dev)
    count = torch.zeros(nq, dtype=torch.int32, device=dev)
    node = torch.empty((nq, row_cap), dtype=torch.int32, device=dev)
    agg = torch.empty((nq, row_cap), dtype=torch.float32, device=dev)
    pred = torch.empty((nq, row_cap), dtype=torch.int32, device=dev)
    rc = lib.cs_tree_shortest(C.byref(g), nq, src_t.data_ptr(), int(max_seconds), C.c_float(speed),
                              C.byref(ws.plan), ws.ptr, ws.nbytes, row_cap, count.data_ptr(), node.data_ptr(),
                              agg.data_ptr(), pred.data_ptr(), _stream_ptr())
    if rc != _native.CS_OK:
        ws.init(_stream_ptr())
    _native.check(rc, "cs_tree_shortest")
    return count.cpu().numpy(), node.cpu().numpy(), agg.cpu().numpy(), pred.cpu().numpy()


def tree_shortest(ns, sources: list[int], max_seconds: int, speed: float):
    """Per source: (visited_nodes, list[NodeVisit]) exactly as dijkstra_tree_shortest returns."""
    counts, nodes, agg, preds = tree_shortest_raw(ns, sources, max_seconds, speed)
    nb = ns.node_bound()
    sp32 = np.float32(speed)
    out = []
    for q in range(len(sources)):
        n = int(counts[q])
        tree = [NodeVisit() for _ in range(nb)]
        visited = nodes[q, :n].tolist()
        for i in range(n):
            v = int(nodes[q, i])
            t = tree[v]
            t.visited = True
            t.discovered = True
            t.agg_seconds = float(agg[q, i])
            t.short_dist = float(np.float32(agg[q, i]) * sp32)
            p = int(preds[q, i])
            t.pred = None if p < 0 else p
        out.append((visited, tree))
    return out


def tree_segment(ns, src: int, max_seconds: int, speed: float):
    """dijkstra_tree_segment (rust/src/centrality.rs:1524-1611): (visited_nodes, visited_edges,
    list[NodeVisit], list[EdgeVisit]).  The search (settle order, agg_seconds, strict-< first
    predecessor) runs on the GPU tree kernel; the edge bookkeeping follows from it on the host: a
    settled node lists its incoming edges from nodes not yet settled (self loops too), and a node's
    last segment is the cheapest edge to its predecessor (first in that node's incoming order on ties).
    """
    from .graph import EdgeVisit, NodeVisit

    counts, nodes, agg, preds = tree_shortest_raw(ns, [src], max_seconds, speed)
    n = int(counts[0])
    host = _primal_host(ns)
    nb = ns.node_bound()
    a = ns.arrays()
    order = nodes[0, :n].astype(np.int64)
    pos = np.full(nb, -1, np.int64)
    pos[order] = np.arange(n)
    in_ptr = host.h["in_ptr"].astype(np.int64)
    in_nb = host.h["in_nb"].astype(np.int64)
    in_slot = host.ex[host.in_order]
    win = host.weights(speed)[0]
    # visited edges, in settle order then incoming order
    cnt = in_ptr[order + 1] - in_ptr[order]
    rows = np.repeat(np.arange(n), cnt)
    offs = np.arange(int(cnt.sum())) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    ei = in_ptr[order][rows] + offs
    u = order[rows]
    v = in_nb[ei]
    keep = (v == u) | (pos[v] < 0) | (pos[v] > rows)
    visited_edges = in_slot[ei[keep]].tolist()
    edge_map = [EdgeVisit() for _ in range(len(a["e_src"]))]
    for e, uu, vv in zip(in_slot[ei[keep]].tolist(), u[keep].tolist(), v[keep].tolist()):
        ev = edge_map[e]
        ev.visited = True
        ev.start_nd_idx = uu
        ev.end_nd_idx = vv
        ev.edge_idx = int(a["e_idx"][e])
    tree = [NodeVisit() for _ in range(nb)]
    sp32 = np.float32(speed)
    for i in range(n):
        x = int(order[i])
        t = tree[x]
        t.visited = True
        t.discovered = True
        t.agg_seconds = float(agg[0, i])
        t.short_dist = float(np.float32(agg[0, i]) * sp32)
        p = int(preds[0, i])
        if p < 0:
            continue
        t.pred = p
        # cheapest edge x -> p among the predecessor's incoming edges (first on ties)
        lo, hi = int(in_ptr[p]), int(in_ptr[p + 1])
        cand = [j for j in range(lo, hi) if in_nb[j] == x]
        best = min(cand, key=lambda j: (win[j], j - lo))
        t.last_seg = int(in_slot[best])
        t.origin_seg = t.last_seg if p == src else tree[p].origin_seg
    return order.tolist(), visited_edges, tree, edge_map


def tree_simplest(ns, sources: list[int], max_seconds: int, speed: float):
    from . import dual

    return dual.tree_simplest(ns, sources, max_seconds, speed)


def last_counters() -> tuple[int, int, int, int]:
    """(sources, edges relaxed, nodes settled, kernel launches) of the last native call on this
    thread."""
    lib = _native.load()
    a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    lib.cs_last_counters(C.byref(a), C.byref(b), C.byref(c), C.byref(d))
    return a.value, b.value, c.value, d.value


_ = math
