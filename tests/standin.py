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


class _StandInLib:
    def __init__(self, ns, real):
        self.ns = ns
        self.og = oracle.OracleGraph(ns)
        self.calls = 0
        self._real = real  # host-side entry points (thresholds, edge seconds) are the library's own

    def __getattr__(self, name):
        return getattr(self._real, name)

    def _query(self, q):
        nb = self.ns.node_bound()
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
        self.calls += 1
        q = q_ref._obj
        d, b, s, plan = self._query(q)
        out, reach = oracle.centrality_shortest(self.og, d, b, s, speed=q.speed_m_s, tol=q.tolerance,
                                                closeness=bool(q.compute_closeness),
                                                betweenness=bool(q.compute_betweenness), plan=plan)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        if o.reach:
            r = reach.astype(np.int32)
            C.memmove(o.reach, r.ctypes.data, r.nbytes)
        return _native.CS_OK

    def cs_centrality_simplest(self, g, q_ref, plan_ref, ws, ws_bytes, o, stream):
        self.calls += 1
        q = q_ref._obj
        d, b, s, plan = self._query(q)
        out, reach = oracle.centrality_simplest(self.og, d, b, s, speed=q.speed_m_s, tol=q.tolerance,
                                                closeness=bool(q.compute_closeness),
                                                betweenness=bool(q.compute_betweenness), plan=plan,
                                                asu=q.angular_scaling_unit, fso=q.farness_scaling_offset)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        r = reach.astype(np.int32)
        C.memmove(o.reach, r.ctypes.data, r.nbytes)
        return _native.CS_OK

    def cs_segment_centrality(self, g, q_ref, plan_ref, ws, ws_bytes, o, stream):
        self.calls += 1
        q = q_ref._obj
        d, b, s, plan = self._query(q)
        live = np.asarray(self.ns.node_indices())[self.ns.arrays()["live"][np.asarray(self.ns.node_indices())] == 1]
        assert sorted(plan["sources"].tolist()) == sorted(live.tolist())  # every live node is a source
        out = oracle.segment_centrality(self.og, d, b, s, speed=q.speed_m_s, closeness=bool(q.compute_closeness),
                                        betweenness=bool(q.compute_betweenness), ns=self.ns)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        return _native.CS_OK

    def cs_tree_shortest(self, g, nq, src_ptr, max_seconds, speed, plan_ref, ws, ws_bytes, row_cap, count_ptr,
                         node_ptr, agg_ptr, pred_ptr, stream):
        """Per query the oracle's tree (dijkstra_tree_shortest): settle order, agg_seconds, pred."""
        self.calls += 1
        srcs = _arr(src_ptr, C.c_int32, nq)
        counts = np.zeros(nq, np.int32)
        for qi, src in enumerate(srcs.tolist()):
            vis, tree = oracle.tree_shortest(self.og, int(src), int(max_seconds), float(speed.value))
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

    def cs_betweenness_od_shortest(self, g, q_ref, od_ptr, od_dst, od_w, plan_ref, ws, ws_bytes, o, stream):
        self.calls += 1
        q = q_ref._obj
        nb = self.ns.node_bound()
        d, b, s, _ = self._query(q)
        ptr = _arr(od_ptr, C.c_int32, nb + 1)
        rows = (ptr, _arr(od_dst, C.c_int32, int(ptr[-1])), _arr(od_w, C.c_float, int(ptr[-1])))
        out = oracle.betweenness_od(self.og, d, b, s, rows, speed=q.speed_m_s, tol=q.tolerance, ns=self.ns)
        C.memmove(o.out, out.ctypes.data, out.nbytes)
        return _native.CS_OK


class _StandInCSR:
    def __init__(self, ns):
        self.device = torch.device("cpu")
        self.n_bound = ns.node_bound()
        self.has_missing_reverse = False

    def struct(self, speed):
        return _native.PrimalGraph()


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
        return box["lib"]

    monkeypatch.setattr(_native, "load", load)
    monkeypatch.setattr(centrality, "_primal_csr", lambda ns: _StandInCSR(ns))
    monkeypatch.setattr(centrality, "_workspace", lambda *a, **k: _StandInWS())
    monkeypatch.setattr(centrality, "_stream_ptr", lambda: None)
    from cityseer_gb300 import dual

    monkeypatch.setattr(dual, "dual_csr", lambda ns: _StandInCSR(ns))
    monkeypatch.setattr(dual, "dual_workspace", lambda *a, **k: _StandInWS())
    monkeypatch.setattr(dual, "estimate_states", lambda *a, **k: 1024)

    def use(ns):
        box["lib"] = _StandInLib(ns, real)
        return box["lib"]

    return use


