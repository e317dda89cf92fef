"""Simplest-path (angular) centrality on the dual graph: device CSR and drivers.

Dual CSR layout in HBM:
  forward   per dual node u: its outgoing dual edges in petgraph Outgoing order (newest first)
            ptr[N+1], to[E], w[E] (travel seconds, no impedance), ang[E] (angle_sum), len[E],
            exit_slot[E] / entry_slot[E] (endpoint slot of the shared primal node at each end)
  reverse   per dual node v: its incoming dual edges: rptr[N+1], rfrom[E], rid[E] (forward index)
Endpoint slots restate dual_node_endpoint_slots (rust/src/centrality.rs:533-566): in edge order,
each dual node's shared primal keys take slots 0 and 1 in order of first appearance.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native, device

DPM = 8


def endpoint_slots(src, dst, key, n_bound):
    """Slot of each edge's shared key at its source and at its target (arrays over edges)."""
    m = len(src)
    if m == 0:
        return np.zeros(0, np.uint8), np.zeros(0, np.uint8)
    if np.any(key < 0):
        e = int(np.nonzero(key < 0)[0][0])
        raise ValueError(f"dual edge {int(src[e])} -> {int(dst[e])} is missing shared_primal_node_key metadata")
    node = np.stack([src, dst], 1).reshape(-1)
    kk = np.stack([key, key], 1).reshape(-1)
    order = np.arange(2 * m)
    rec = np.zeros(2 * m, dtype=[("n", np.int64), ("k", np.int64), ("o", np.int64)])
    rec["n"], rec["k"], rec["o"] = node, kk, order
    srt = np.argsort(rec, order=("n", "k", "o"))
    r = rec[srt]
    first = np.ones(2 * m, bool)
    first[1:] = (r["n"][1:] != r["n"][:-1]) | (r["k"][1:] != r["k"][:-1])
    fo = r[first]  # first occurrence of each (node, key)
    # per node: rank of its keys by first appearance
    srt2 = np.lexsort((fo["o"], fo["n"]))
    fo = fo[srt2]
    start = np.ones(len(fo), bool)
    start[1:] = fo["n"][1:] != fo["n"][:-1]
    grp = np.cumsum(start) - 1
    first_idx = np.nonzero(start)[0]
    rank = np.arange(len(fo)) - first_idx[grp]
    if np.any(rank > 1):
        bad = int(fo["n"][np.nonzero(rank > 1)[0][0]])
        raise ValueError(f"dual node {bad} references more than two primal endpoints")
    # look up the slot of (node, key)
    q = np.zeros(2 * m, dtype=[("n", np.int64), ("k", np.int64)])
    q["n"], q["k"] = node, kk
    keys = np.zeros(len(fo), dtype=[("n", np.int64), ("k", np.int64)])
    keys["n"], keys["k"] = fo["n"], fo["k"]
    o2 = np.argsort(keys, order=("n", "k"))
    pos = np.searchsorted(keys[o2], q)
    slot = rank[o2][pos].reshape(m, 2)
    return slot[:, 0].astype(np.uint8), slot[:, 1].astype(np.uint8)


class DualCSR:
    def __init__(self, ns, dev: torch.device | None = None):
        self.device = dev or device._require_cuda()
        a = ns.arrays()
        self.arr = a
        n = ns.node_bound()
        self.n_bound = n
        ex = np.nonzero(a["e_exists"])[0]
        src = a["e_src"][ex].astype(np.int64)
        dst = a["e_dst"][ex].astype(np.int64)
        key = a["e_shared"][ex].astype(np.int64)
        exit_s, entry_s = endpoint_slots(src, dst, key, n)
        self.ex = ex
        self.m = len(ex)
        fo = np.lexsort((-ex, src)) if self.m else np.zeros(0, np.int64)
        ro = np.lexsort((-ex, dst)) if self.m else np.zeros(0, np.int64)
        pos_in_fwd = np.empty(self.m, np.int64)
        pos_in_fwd[fo] = np.arange(self.m)
        out_cnt = np.bincount(src, minlength=n) if self.m else np.zeros(n, np.int64)
        in_cnt = np.bincount(dst, minlength=n) if self.m else np.zeros(n, np.int64)
        ptr = np.zeros(n + 1, np.int64)
        rptr = np.zeros(n + 1, np.int64)
        ptr[1:] = np.cumsum(out_cnt)
        rptr[1:] = np.cumsum(in_cnt)
        self.max_degree = int(max(out_cnt.max(initial=0), in_cnt.max(initial=0)))
        self.fo, self.ro = fo, ro
        t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).astype(dt)).to(self.device)  # noqa: E731
        self.ptr = t(ptr, np.int32)
        self.to = t(dst[fo], np.int32)
        self.ang = t(a["e_ang"][ex][fo], np.float32)
        self.len = t(a["e_len"][ex][fo], np.float32)
        self.exit_slot = t(exit_s[fo], np.uint8)
        self.entry_slot = t(entry_s[fo], np.uint8)
        self.rptr = t(rptr, np.int32)
        self.rfrom = t(src[ro], np.int32)
        self.rid = t(pos_in_fwd[ro], np.int32)
        self._w: dict[float, torch.Tensor] = {}
        self._pack: dict[float, tuple[torch.Tensor, torch.Tensor]] = {}

    def w(self, speed: float) -> torch.Tensor:
        k = float(np.float32(speed))
        hit = self._w.get(k)
        if hit is None:
            w = device.edge_seconds(self.arr, speed, False)[self.ex][self.fo]
            hit = torch.from_numpy(np.ascontiguousarray(w)).to(self.device)
            self._w[k] = hit
        return hit

    def packed(self, speed: float) -> tuple[torch.Tensor, torch.Tensor]:
        """The packed 16-byte forward and reverse edge records at this speed (cs_dual_pack)."""
        k = float(np.float32(speed))
        hit = self._pack.get(k)
        if hit is None:
            m = max(1, self.m)
            fwd = torch.empty((m, 4), dtype=torch.int32, device=self.device)
            rev = torch.empty((m, 4), dtype=torch.int32, device=self.device)
            g = self._plain(speed)
            g.fwd_pack = fwd.data_ptr()
            g.rev_pack = rev.data_ptr()
            stream = torch.cuda.current_stream(self.device)
            _native.check(_native.load().cs_dual_pack(C.byref(g), fwd.data_ptr(), rev.data_ptr(),
                                                      stream.cuda_stream), "cs_dual_pack")
            stream.synchronize()  # callers launch on other streams too (the served lanes)
            hit = (fwd, rev)
            self._pack[k] = hit
        return hit

    def struct(self, speed: float) -> _native.DualGraph:
        g = self._plain(speed)
        fwd, rev = self.packed(speed)
        g.fwd_pack = fwd.data_ptr()
        g.rev_pack = rev.data_ptr()
        return g

    def _plain(self, speed: float) -> _native.DualGraph:
        g = _native.DualGraph()
        g.n_bound = self.n_bound
        g.n_edges = self.m
        g.max_out_degree = self.max_degree
        g.ptr = self.ptr.data_ptr()
        g.to = self.to.data_ptr()
        g.w = self.w(speed).data_ptr()
        g.ang = self.ang.data_ptr()
        g.len = self.len.data_ptr()
        g.exit_slot = self.exit_slot.data_ptr()
        g.entry_slot = self.entry_slot.data_ptr()
        g.rptr = self.rptr.data_ptr()
        g.rfrom = self.rfrom.data_ptr()
        g.rid = self.rid.data_ptr()
        return g


class DualWorkspace(device.Workspace):
    def init(self, stream=None):
        lib = _native.load()
        rc = lib.cs_dual_workspace_init(C.byref(self.plan), self.n_bound, self.ptr, self.nbytes, stream)
        _native.check(rc, "cs_dual_workspace_init")


def dual_csr(ns) -> DualCSR:
    c = ns._cache.get("dual_csr")
    if c is None:
        c = DualCSR(ns)
        if c.max_degree > DPM:
            raise ValueError("a dual node has more than 8 incoming or outgoing dual edges (intersections of degree "
                             "above 5); not supported by the simplest-path kernels")
        ns._cache["dual_csr"] = c
    return c


def dual_workspace(ns, csr: DualCSR, k: int, speed: float, cap: int = 0, max_slots: int = 0):
    """The dual graph's workspace, grown (never shrunk) to the thresholds this call needs."""
    from .centrality import _mem_budget

    ws = ns._cache.get("wsd")
    if ws is not None and ws.plan.lanes >= k and (cap <= 0 or ws.plan.cap >= cap) and \
            (max_slots <= 0 or ws.plan.n_slots <= max_slots):
        return ws
    if ws is not None:
        k = max(k, int(ws.plan.lanes))
        del ns._cache["wsd"]
        del ws
    torch.cuda.empty_cache()
    lib = _native.load()
    plan = _native.Plan()
    rc = lib.cs_plan_dual(C.byref(csr.struct(speed)), 0, k, cap, max_slots, _mem_budget(csr.device), C.byref(plan))
    _native.check(rc, "cs_plan_dual")
    ws = DualWorkspace(plan, csr.n_bound, csr.device)
    ns._cache["wsd"] = ws
    return ws


def estimate_states(ns, speed: float, max_seconds: int) -> int:
    """Search capacity (angular states) for sources of this dual graph up to max_seconds: twice the
    largest metric reach (dual nodes within max_seconds by shortest metric distance, from the tree
    kernel on the dual's own edges over a sample of sources) plus 30%.  A simplest route is never
    shorter than the shortest one, so the angular search reaches a subset of those nodes."""
    from .centrality import _primal_csr, estimate_reach

    key = ("dual_states", float(np.float32(speed)), int(max_seconds))
    hit = ns._cache.get(key)
    if hit is None:
        r = estimate_reach(ns, _primal_csr(ns), speed, int(max_seconds))
        hit = int(min(2 * ns.node_bound(), max(1024, -(-int(2.6 * r) // 256) * 256)))
        ns._cache[key] = hit
    return hit


def simplest_rows(ns, sp, process, dists, bets, secs, speed, tol, asu, fso, closeness, betweenness, track):
    """The device rows of centrality_simplest for the sources `process` under the plan `sp`:
    ([4][K][N] f64, [K] i64 reach counts) on the graph's device, before any post-scale.  Every
    launch searches to the largest threshold, as the reference's single search does."""
    from .centrality import _cutoff_groups, _make_query, _stream_ptr

    nb = ns.node_bound()
    K = len(dists)
    csr = dual_csr(ns)
    dev = csr.device
    proc_t = torch.from_numpy(np.ascontiguousarray(process, np.int32)).to(dev)
    wt_t = torch.from_numpy(sp.src_wt).to(dev)
    el_t = torch.from_numpy(sp.eligible).to(dev)
    g = csr.struct(speed)
    lib = _native.load()
    groups = _cutoff_groups(K)
    rows = torch.zeros((4, K, nb), dtype=torch.float64, device=dev) if len(groups) > 1 else None
    reach_all = torch.zeros(K, dtype=torch.int64, device=dev)
    for lo, hi, sel in groups:
        k = len(sel)
        gd, gb, gs = [dists[i] for i in sel], [bets[i] for i in sel], [secs[i] for i in sel]
        ws = dual_workspace(ns, csr, k, speed, cap=estimate_states(ns, speed, max(gs)))
        out = torch.zeros((4, k, nb), dtype=torch.float64, device=dev)
        reach = torch.zeros(k, dtype=torch.int32, device=dev)
        q = _make_query(gd, gb, gs, speed, tol, closeness, betweenness, track, proc_t, wt_t, el_t, asu, fso)
        o = _native.Outputs(out.data_ptr(), reach.data_ptr())
        rc = lib.cs_centrality_simplest(C.byref(g), C.byref(q), C.byref(ws.plan), ws.ptr, ws.nbytes, o, _stream_ptr())
        if rc != _native.CS_OK:
            ws.init(_stream_ptr())
        _native.check(rc, "cs_centrality_simplest")
        if rows is None:
            rows = out
        else:
            rows[:, lo:hi] = out[:, : hi - lo]
        reach_all[lo:hi] = reach[: hi - lo].to(torch.int64)
    return rows, reach_all


def finish_simplest(ns, dists, sp, data: np.ndarray, reach_tot: np.ndarray, betweenness: bool, track: bool):
    """Post-scale (source subsets) and the result object of centrality_simplest."""
    from .centrality import CentralitySimplestResult

    node_indices = ns._node_index_array()
    if betweenness and sp.is_source_indexed and sp.sample_probability is None and sp.n_sources > 0:
        scale = sp.n_live / sp.n_sources
        if scale != 1.0:
            data[3][:, node_indices] *= scale
    ns._progress = sp.n_sources
    res = CentralitySimplestResult(dists, ns.node_keys_py(), node_indices, data)
    if track:
        res.sampled_source_count = sp.sampled_count
        res.reachability_totals = [int(x) for x in reach_tot]
    return res


def run_simplest(ns, dists, bets, secs, speed, tol, asu, fso, closeness, betweenness, sp):
    track = sp.sample_probability is not None or sp.is_source_indexed
    rows, reach = simplest_rows(ns, sp, sp.process, dists, bets, secs, speed, tol, asu, fso, closeness, betweenness,
                                track)
    return finish_simplest(ns, dists, sp, rows.cpu().numpy(), reach.cpu().numpy(), betweenness, track)


class DualTreeWorkspace(device.Workspace):
    def init(self, stream=None):
        lib = _native.load()
        _native.check(lib.cs_dual_tree_workspace_init(C.byref(self.plan), self.ptr, self.nbytes, stream),
                      "cs_dual_tree_workspace_init")


def tree_workspace(ns, csr: DualCSR, n_queries: int, speed: float):
    """The dual graph's simplest-path tree workspace (capacity from the dual's metric reach)."""
    from .centrality import _mem_budget

    ws = ns._cache.get("wsdt")
    if ws is None:
        lib = _native.load()
        plan = _native.Plan()
        _native.check(lib.cs_plan_dual_tree(C.byref(csr.struct(speed)), 0, 0, _mem_budget(csr.device) // 4,
                                            C.byref(plan)), "cs_plan_dual_tree")
        ws = DualTreeWorkspace(plan, csr.n_bound, csr.device)
        ns._cache["wsdt"] = ws
    return ws


def tree_simplest_raw(ns, sources, max_seconds: int, speed: float, row_cap: int | None = None):
    """Batched simplest-path trees on the GPU: (counts, nodes, simpl_dist, agg_seconds, preds), rows
    in first-reach order, row_cap wide."""
    from .centrality import _stream_ptr

    csr = dual_csr(ns)
    dev = csr.device
    nq = len(sources)
    nb = csr.n_bound
    if row_cap is None:
        row_cap = nb
    ws = tree_workspace(ns, csr, nq, speed)
    lib = _native.load()
    src_t = torch.tensor(list(sources), dtype=torch.int32, device=dev)
    count = torch.zeros(max(nq, 1), dtype=torch.int32, device=dev)
    node = torch.empty((max(nq, 1), row_cap), dtype=torch.int32, device=dev)
    simpl = torch.empty((max(nq, 1), row_cap), dtype=torch.float32, device=dev)
    agg = torch.empty((max(nq, 1), row_cap), dtype=torch.float32, device=dev)
    pred = torch.empty((max(nq, 1), row_cap), dtype=torch.int32, device=dev)
    rc = lib.cs_tree_simplest(C.byref(csr.struct(speed)), nq, src_t.data_ptr() if nq else None, int(max_seconds),
                              C.c_float(speed), C.byref(ws.plan), ws.ptr, ws.nbytes, row_cap, count.data_ptr(),
                              node.data_ptr(), simpl.data_ptr(), agg.data_ptr(), pred.data_ptr(), _stream_ptr())
    if rc != _native.CS_OK:
        ws.init(_stream_ptr())
    _native.check(rc, "cs_tree_simplest")
    return (count.cpu().numpy()[:nq], node.cpu().numpy()[:nq], simpl.cpu().numpy()[:nq], agg.cpu().numpy()[:nq],
            pred.cpu().numpy()[:nq])


def tree_simplest(ns, sources, max_seconds, speed):
    """Per source: (visited_nodes, list[NodeVisit]) exactly as dijkstra_tree_simplest returns."""
    from .graph import NodeVisit

    counts, nodes, simpl, agg, preds = tree_simplest_raw(ns, sources, max_seconds, speed)
    nb = ns.node_bound()
    out = []
    for q in range(len(sources)):
        n = int(counts[q])
        tree = [NodeVisit() for _ in range(nb)]
        visited = nodes[q, :n].tolist()
        for i in range(n):
            t = tree[int(nodes[q, i])]
            t.visited = True
            t.discovered = True
            t.simpl_dist = float(simpl[q, i])
            t.agg_seconds = float(agg[q, i])
            p = int(preds[q, i])
            t.pred = None if p < 0 else p
        out.append((visited, tree))
    return out
