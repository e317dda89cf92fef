"""Device-resident CSR for the GPU kernels, built from a NetworkStructure's columns.

Layout in HBM (all int32 / float32 / uint8, one array per field, contiguous):
  in-CSR   per node u: edges v->u, petgraph Incoming order (newest edge first)
           in_ptr[N+1], in_nb[E], in_w[E], in_seglen[E], in_segimp[E]
  out-CSR  per node v: edges v->u sorted by (u, newest first)
           out_ptr[N+1], out_to[E], out_w[E], out_cnt[E], out_seglen[E]
  node_w[N]
Travel seconds depend on the call's speed, so in_w/out_w are (re)computed per speed by
libcsgpu.so's host code (cs_edge_travel_seconds) and cached per speed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native


def _require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("cityseer_gb300 requires a CUDA device (GB300, sm_103a); none is available")
    _native.load()
    return torch.device("cuda", torch.cuda.current_device())


def reverse_lookup(src, dst, eidx, slot):
    """For every directed edge (s->d, edge_idx) the newest edge d->s with the same edge_idx, which
    is what get_edge_length_unchecked(d, s, edge_idx) finds (rust/src/graph.rs:1278-1314).
    Returns indices into the input arrays (-1 where no such edge exists)."""
    m = len(src)
    if m == 0:
        return np.zeros(0, np.int64)
    rec = np.zeros(m, dtype=[("a", np.int64), ("b", np.int64), ("c", np.int64), ("s", np.int64)])
    rec["a"], rec["b"], rec["c"], rec["s"] = src, dst, eidx, slot
    order = np.argsort(rec, order=("a", "b", "c", "s"), kind="stable")
    keys = rec[order][["a", "b", "c"]]
    q = np.zeros(m, dtype=[("a", np.int64), ("b", np.int64), ("c", np.int64)])
    q["a"], q["b"], q["c"] = dst, src, eidx
    # newest (largest slot) of a group is its last element: search the right end
    pos = np.searchsorted(keys, q, side="right") - 1
    ok = pos >= 0
    posc = np.clip(pos, 0, m - 1)
    hit = keys[posc]
    ok &= (hit["a"] == q["a"]) & (hit["b"] == q["b"]) & (hit["c"] == q["c"])
    res = np.where(ok, order[posc], -1)
    return res.astype(np.int64)


def circuit_count_flags(src, dst, eidx, slot):
    """1 for the first directed edge of every undirected key (min, max, edge_idx), self-loops 0:
    counting those once reproduces the HashSet dedupe of circuit_ranks_from_traversal
    (rust/src/centrality.rs:486-515)."""
    m = len(src)
    flags = np.zeros(m, np.uint8)
    if m == 0:
        return flags
    lo = np.minimum(src, dst)
    hi = np.maximum(src, dst)
    rec = np.zeros(m, dtype=[("a", np.int64), ("b", np.int64), ("c", np.int64)])
    rec["a"], rec["b"], rec["c"] = lo, hi, eidx
    order = np.lexsort((slot, rec["c"], rec["b"], rec["a"]))
    r = rec[order]
    first = np.ones(m, bool)
    first[1:] = (r["a"][1:] != r["a"][:-1]) | (r["b"][1:] != r["b"][:-1]) | (r["c"][1:] != r["c"][:-1])
    flags[order[first]] = 1
    flags[src == dst] = 0
    return flags


def edge_seconds(arr: dict, speed: float, use_impedance: bool) -> np.ndarray:
    lib = _native.load()
    m = len(arr["e_src"])
    out = np.zeros(m, np.float32)
    src = np.ascontiguousarray(arr["e_src"], np.int32)
    dst = np.ascontiguousarray(arr["e_dst"], np.int32)
    ln = np.ascontiguousarray(arr["e_len"], np.float32)
    imp = np.ascontiguousarray(arr["e_imp"], np.float32)
    sec = np.ascontiguousarray(arr["e_sec"], np.float32)
    hz = np.ascontiguousarray(arr["has_z"], np.uint8)
    z = np.ascontiguousarray(np.nan_to_num(arr["z"]), np.float64)
    rc = lib.cs_edge_travel_seconds(m, src.ctypes.data, dst.ctypes.data, ln.ctypes.data, imp.ctypes.data,
                                    sec.ctypes.data, hz.ctypes.data, z.ctypes.data, C.c_float(speed),
                                    1 if use_impedance else 0, out.ctypes.data)
    _native.check(rc)
    return out


class PrimalHost:
    """Host-side CSR index arrays of a primal graph (built once per graph version)."""

    def __init__(self, ns):
        a = ns.arrays()
        self.arr = a
        self.n_bound = ns.node_bound()
        n = self.n_bound
        ex = np.nonzero(a["e_exists"])[0]
        src = a["e_src"][ex].astype(np.int64)
        dst = a["e_dst"][ex].astype(np.int64)
        eidx = a["e_idx"][ex].astype(np.int64)
        self.ex = ex
        self.m = len(ex)
        self.in_order = np.lexsort((-ex, dst)) if self.m else np.zeros(0, np.int64)
        self.out_order = np.lexsort((-ex, dst, src)) if self.m else np.zeros(0, np.int64)
        in_cnt = np.bincount(dst, minlength=n) if self.m else np.zeros(n, np.int64)
        out_cnt = np.bincount(src, minlength=n) if self.m else np.zeros(n, np.int64)
        in_ptr = np.zeros(n + 1, np.int64)
        out_ptr = np.zeros(n + 1, np.int64)
        in_ptr[1:] = np.cumsum(in_cnt)
        out_ptr[1:] = np.cumsum(out_cnt)
        self.max_out_degree = int(out_cnt.max()) if n else 0
        rev = reverse_lookup(src, dst, eidx, ex)
        self.has_missing_reverse = bool(np.any(rev < 0))
        lens = a["e_len"][ex]
        imps = a["e_imp"][ex]
        seglen = np.where(rev >= 0, lens[np.clip(rev, 0, None)], np.float32(np.nan)).astype(np.float32)
        segimp = np.where(rev >= 0, imps[np.clip(rev, 0, None)], np.float32(np.nan)).astype(np.float32)
        cnt = circuit_count_flags(src, dst, eidx, ex)
        c = np.ascontiguousarray
        self.h = {
            "in_ptr": c(in_ptr.astype(np.int32)),
            "in_nb": c(src[self.in_order].astype(np.int32)),
            "in_seglen": c(seglen[self.in_order]),
            "in_segimp": c(segimp[self.in_order]),
            "out_ptr": c(out_ptr.astype(np.int32)),
            "out_to": c(dst[self.out_order].astype(np.int32)),
            "out_cnt": c(cnt[self.out_order].astype(np.uint8)),
            "out_seglen": c(seglen[self.out_order]),
            "node_w": c(a["weight"][:n].astype(np.float32)),
        }
        self._w: dict[float, tuple[np.ndarray, np.ndarray, float]] = {}

    def weights(self, speed: float):
        key = float(np.float32(speed))
        hit = self._w.get(key)
        if hit is None:
            w = edge_seconds(self.arr, speed, True)[self.ex]
            med = float(np.median(w)) if len(w) else 1.0
            hit = (np.ascontiguousarray(w[self.in_order]), np.ascontiguousarray(w[self.out_order]), med)
            self._w[key] = hit
        return hit

    def nbytes(self, speed: float) -> int:
        win, wout, _ = self.weights(speed)
        return sum(v.nbytes for v in self.h.values()) + win.nbytes + wout.nbytes


class PrimalCSR:
    """Primal CSR resident on one device (uploaded from a PrimalHost)."""

    def __init__(self, host: PrimalHost, device: torch.device | None = None, pinned: bool = False):
        self.device = device or _require_cuda()
        self.host = host
        self.n_bound = host.n_bound
        self.m = host.m
        self.max_out_degree = host.max_out_degree
        self.has_missing_reverse = host.has_missing_reverse
        self.pinned = pinned
        for k, v in host.h.items():
            setattr(self, k, self._up(v))
        self._w_cache: dict[float, tuple[torch.Tensor, torch.Tensor, float]] = {}

    def _up(self, arr: np.ndarray) -> torch.Tensor:
        t = torch.from_numpy(arr)
        if self.pinned:
            t = t.pin_memory()
        return t.to(self.device, non_blocking=self.pinned)

    def weights(self, speed: float):
        key = float(np.float32(speed))
        hit = self._w_cache.get(key)
        if hit is None:
            win, wout, med = self.host.weights(speed)
            hit = (self._up(win), self._up(wout), med)
            self._w_cache[key] = hit
        return hit

    def struct(self, speed: float) -> _native.PrimalGraph:
        win, wout, _ = self.weights(speed)
        g = _native.PrimalGraph()
        g.n_bound = self.n_bound
        g.n_edges = self.m
        g.max_out_degree = self.max_out_degree
        g.in_ptr = self.in_ptr.data_ptr()
        g.in_nb = self.in_nb.data_ptr()
        g.in_w = win.data_ptr()
        g.in_seglen = self.in_seglen.data_ptr()
        g.in_segimp = self.in_segimp.data_ptr()
        g.out_ptr = self.out_ptr.data_ptr()
        g.out_to = self.out_to.data_ptr()
        g.out_w = wout.data_ptr()
        g.out_cnt = self.out_cnt.data_ptr()
        g.out_seglen = self.out_seglen.data_ptr()
        g.node_w = self.node_w.data_ptr()
        return g

    def median_edge_seconds(self, speed: float) -> float:
        return self.weights(speed)[2]


class Workspace:
    """A planned, initialised workspace for one (graph, mode, thresholds) shape."""

    def __init__(self, plan: _native.Plan, n_bound: int, device: torch.device, stream=None):
        self.plan = plan
        self.n_bound = n_bound
        self.buf = torch.empty(int(plan.workspace_bytes), dtype=torch.uint8, device=device)
        self.init(stream)

    @property
    def ptr(self) -> int:
        return self.buf.data_ptr()

    @property
    def nbytes(self) -> int:
        return self.buf.numel()

    def init(self, stream=None):
        lib = _native.load()
        rc = lib.cs_workspace_init(C.byref(self.plan), self.n_bound, self.ptr, self.nbytes, stream)
        _native.check(rc, "cs_workspace_init")


def plan_primal(csr: PrimalCSR, mode: int, k: int, speed: float, cap: int = 0, max_slots: int = 0,
                mem_budget: int = 0, delta: float = 0.0, variant: int = 0) -> _native.Plan:
    lib = _native.load()
    plan = _native.Plan()
    plan.delta_seconds = delta
    plan.variant = variant
    g = csr.struct(speed)
    rc = lib.cs_plan_primal(C.byref(g), mode, k, cap, max_slots, mem_budget, C.byref(plan))
    _native.check(rc, "cs_plan_primal")
    if plan.delta_seconds <= 0:
        plan.delta_seconds = 2.0 * csr.median_edge_seconds(speed)
    return plan
