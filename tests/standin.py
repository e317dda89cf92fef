"""An oracle-backed stand-in for the C-ABI calls of the host paths (test infrastructure only).

It reads the query the host built (sources, weights, eligibility, thresholds) from the pointers
passed, runs the oracle on exactly that, and writes the rows where the host asked.  Host-side entry
points (thresholds, edge seconds) go to the real library.  `install(monkeypatch)` swaps it in for
the device CSR, workspaces and the library loader and returns use(ns) -> stand-in."""
import ctypes as C

import numpy as np
import torch

import oracle
from cityseer_gb300 import _native, centrality


def _arr(ptr, ctype, n):
    return np.ctypeslib.as_array((ctype * max(n, 1)).from_address(ptr))[:n].copy()


_GRAPHS: dict = {}  # id(ns) -> key carried in the stand-in graph struct


class _StandInLib:
    def __init__(self, ns, real, many=()):
        self.ns = ns
        self.og = oracle.OracleGraph(ns)
        self.calls = 0
        self._real = real  # host-side entry points (thresholds, edge seconds) are the library's own
        self.graphs = {}
        for g in (ns, *many):
            key = _GRAPHS.setdefault(id(g), len(_GRAPHS) + 1)
            self.graphs[key] = (g, self.og if g is ns else oracle.OracleGraph(g))

    def __getattr__(self, name):
        return getattr(self._real, name)

    def _graph(self, g_ref):
        """(ns, oracle graph) named by the stand-in graph struct passed to a call."""
        key = getattr(g_ref, "_obj", g_ref).in_ptr
        return self.graphs.get(key, (self.ns, self.og))

    def _query(self, q, nb):
        k = q.k
        d = [int(q.distances[i]) for i in range(k)]
        b = [float(q.betas[i]) for i in range(k)]
        s = [int(q.seconds[i]) for i in range(k)]
        src = _arr(q.sources, C.c_int32, int(q.n_sources)) if q.n_sources else np.zeros(0, np.int32)
        plan = {"sources": src.astype(np.int64), "eligible": _arr(q.eligible, C.c_uint8, nb),
                "src_wt": _arr(q.src_wt, C.c_float, nb), "src_take": np.ones(nb, np.uint8),
                "track_reach": bool(q.track_reach)}
        return d, b, s, plan

    def cs_centrality_shortest(self, g, q_ref, plan_ref, ws, ws_bytes, o, stream):
        ns_, og_ = self._graph(g)
        self.calls += 1
        q = q_ref._obj
        d, b, s, plan = self._query(q, ns_.node_bound())
        out, reach = oracle.centrality_shortest(og_, d, b, s, speed=q.speed_m_s, tol=q.tolerance,
                                                closeness=bool(q.compute_closeness),
                                                betweenness=bool(q.compute_betweenness), plan=plan)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        if o.reach:
            r = reach.astype(np.int32)
            C.memmove(o.reach, r.ctypes.data, r.nbytes)
        return _native.CS_OK

    def cs_centrality_simplest(self, g, q_ref, plan_ref, ws, ws_bytes, o, stream):
        ns_, og_ = self._graph(g)
        self.calls += 1
        q = q_ref._obj
        d, b, s, plan = self._query(q, ns_.node_bound())
        out, reach = oracle.centrality_simplest(og_, d, b, s, speed=q.speed_m_s, tol=q.tolerance,
                                                closeness=bool(q.compute_closeness),
                                                betweenness=bool(q.compute_betweenness), plan=plan,
                                                asu=q.angular_scaling_unit, fso=q.farness_scaling_offset)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        r = reach.astype(np.int32)
        C.memmove(o.reach, r.ctypes.data, r.nbytes)
        return _native.CS_OK

    def cs_segment_centrality(self, g, q_ref, plan_ref, ws, ws_bytes, o, stream):
        ns_, og_ = self._graph(g)
        self.calls += 1
        q = q_ref._obj
        d, b, s, plan = self._query(q, ns_.node_bound())
        live = np.asarray(ns_.node_indices())[ns_.arrays()["live"][np.asarray(ns_.node_indices())] == 1]
        assert sorted(plan["sources"].tolist()) == sorted(live.tolist())  # every live node is a source
        out = oracle.segment_centrality(og_, d, b, s, speed=q.speed_m_s, closeness=bool(q.compute_closeness),
                                        betweenness=bool(q.compute_betweenness), ns=ns_)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        return _native.CS_OK

    def cs_tree_shortest(self, g, nq, src_ptr, max_seconds, speed, plan_ref, ws, ws_bytes, row_cap, count_ptr,
                         node_ptr, agg_ptr, pred_ptr, stream):
        ns_, og_ = self._graph(g)
        """Per query the oracle's tree (dijkstra_tree_shortest): settle order, agg_seconds, pred."""
        self.calls += 1
        srcs = _arr(src_ptr, C.c_int32, nq)
        counts = np.zeros(nq, np.int32)
        for qi, src in enumerate(srcs.tolist()):
            vis, tree = oracle.tree_shortest(og_, int(src), int(max_seconds), float(speed.value))
            n = len(vis)
            counts[qi] = n if n <= row_cap else -n
            m = min(n, row_cap)
            rows = (vis[:m].astype(np.int32), tree["agg_seconds"][vis[:m]].astype(np.float32),
                    tree["pred"][vis[:m]].astype(np.int32))
            for ptr, arr in zip((node_ptr, agg_ptr, pred_ptr), rows):
                if m:
                    C.memmove(ptr + qi * row_cap * 4, arr.ctypes.data, arr.nbytes)
        C.memmove(count_ptr, counts.ctypes.data, counts.nbytes)
        return _native.CS_OK

    # batched form: every job of the table through the oracle
    def cs_workspace_init(self, *a):
        return _native.CS_OK

    def cs_batch_plan(self, jobs, n_jobs, cap, max_slots, budget, plan_ref):
        pl = plan_ref._obj
        pl.n_slots, pl.cap, pl.lanes, pl.workspace_bytes = 8, max(cap, 32), 32, 256
        pl.n_bound = max(jobs[j].g.n_bound for j in range(n_jobs))
        if pl.variant <= 0:
            pl.variant = 3
        return _native.CS_OK

    def cs_batch_run(self, jobs, jobs_dev, n_jobs, plan_ref, ws, ws_bytes, flags, stream):
        self.calls += 1
        self.items = 0
        for j in range(n_jobs):
            jb = jobs[j]
            ns, og = self.graphs[jb.g.in_ptr]
            nb = ns.node_bound()
            k = jb.k
            d = [int(jb.distances[i]) for i in range(k)]
            b = [float(jb.betas[i]) for i in range(k)]
            s = [int(jb.seconds[i]) for i in range(k)]
            src = _arr(jb.sources, C.c_int32, jb.n_sources).astype(np.int64) if jb.n_sources else np.zeros(0, np.int64)
            self.items += len(src)
            plan = {"sources": src, "eligible": _arr(jb.eligible, C.c_uint8, nb),
                    "src_wt": _arr(jb.src_wt, C.c_float, nb), "src_take": np.ones(nb, np.uint8), "track_reach": False}
            close, betw = bool(jb.compute_closeness), bool(jb.compute_betweenness)
            if jb.mode in (0, 3):
                out, _ = oracle.centrality_shortest(og, d, b, s, speed=jb.speed_m_s, tol=jb.tolerance, closeness=close,
                                                    betweenness=betw, plan=plan)
                C.memmove(jb.out, out.ctypes.data, out.nbytes)
            if jb.mode in (1, 3):
                assert sorted(src.tolist()) == [v for v in ns.node_indices() if ns.is_node_live(v)]
                seg = oracle.segment_centrality(og, d, b, s, speed=jb.speed_m_s, closeness=close, betweenness=betw,
                                                ns=ns)
                C.memmove(jb.out2 if jb.mode == 3 else jb.out, seg.ctypes.data, seg.nbytes)
        return _native.CS_OK

    def cs_batch_status(self, ws, overflowed_ref, done_ref, stream):
        overflowed_ref._obj.value = 0
        done_ref._obj.value = self.items
        return _native.CS_OK

    def cs_betweenness_od_shortest(self, g, q_ref, od_ptr, od_dst, od_w, plan_ref, ws, ws_bytes, o, stream):
        ns_, og_ = self._graph(g)
        self.calls += 1
        q = q_ref._obj
        nb = ns_.node_bound()
        d, b, s, _ = self._query(q, ns_.node_bound())
        ptr = _arr(od_ptr, C.c_int32, nb + 1)
        rows = (ptr, _arr(od_dst, C.c_int32, int(ptr[-1])), _arr(od_w, C.c_float, int(ptr[-1])))
        out = oracle.betweenness_od(og_, d, b, s, rows, speed=q.speed_m_s, tol=q.tolerance, ns=ns_)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        return _native.CS_OK


class _StandInCSR:
    def __init__(self, ns):
        self.device = torch.device("cpu")
        self.n_bound = ns.node_bound()
        self.m = int(ns.arrays()["e_exists"].sum())
        self.has_missing_reverse = False
        self.key = _GRAPHS.setdefault(id(ns), len(_GRAPHS) + 1)

    def struct(self, speed):
        g = _native.PrimalGraph()
        g.n_bound = self.n_bound
        g.in_ptr = self.key  # which graph: the stand-in library looks it up
        return g

    def median_edge_seconds(self, speed):
        return 1.0


class _StandInWS:
    plan = _native.Plan()
    ptr = None
    nbytes = 0

    def init(self, *a):
        pass


def install(monkeypatch):
    box = {}
    real = _native.load()

    def load(*a, **k):
        return box.get("lib", real)  # the library itself until a graph is registered

    monkeypatch.setattr(_native, "load", load)
    monkeypatch.setattr(centrality, "_primal_csr", lambda ns: _StandInCSR(ns))
    monkeypatch.setattr(centrality, "_workspace", lambda *a, **k: _StandInWS())
    monkeypatch.setattr(centrality, "_stream_ptr", lambda: None)
    from cityseer_gb300 import dual

    monkeypatch.setattr(dual, "dual_csr", lambda ns: _StandInCSR(ns))
    monkeypatch.setattr(dual, "dual_workspace", lambda *a, **k: _StandInWS())
    monkeypatch.setattr(dual, "estimate_states", lambda *a, **k: 1024)

    monkeypatch.setattr(centrality, "estimate_reach", lambda *a, **k: 64)
    monkeypatch.setattr(centrality, "_mem_budget", lambda *a, **k: 1 << 30)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: type("S", (), {"cuda_stream": None})())

    def use(ns, *more):
        box["lib"] = _StandInLib(ns, real, more)
        return box["lib"]

    return use


