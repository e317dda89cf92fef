"""The host paths above the C-ABI (query building, threshold groups of 16, source plans, post-scale,
result objects, the sharded form's default share, OD rows) run on the CPU with the C-ABI calls
answered by the oracle.  The stand-in library is test infrastructure: it reads the query the host
built (sources, weights, eligibility, thresholds) from the pointers passed, runs the oracle on exactly
that, and writes the rows where the host asked.  The GPU parity tests cover the kernels themselves."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from cityseer_gb300 import _native, centrality, synth
from cityseer_gb300.centrality import OdMatrix, prepare_source_sampling, validate_tolerance
from cityseer_gb300.common import pair_distances_betas_time
from cityseer_gb300.replicas import sharded_centrality_shortest
from cityseer_gb300.tools import io
from helpers import mock_graph


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


@pytest.fixture
def stand_in(monkeypatch):
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


def _want(ns, dists, p=None, w=None, seed=None, src=None, closeness=True, betweenness=True, tol=None):
    sp = prepare_source_sampling(ns, p, w, seed, src)
    d, b, s = pair_distances_betas_time(1.33333, distances=dists)
    out, reach = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, tol=validate_tolerance(tol),
                                            closeness=closeness, betweenness=betweenness,
                                            plan=oracle.plan_from(sp, ns.node_bound()))
    return out, reach, sp


def test_shortest_host_path(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    lib = stand_in(ns)
    for kw in (dict(), dict(p=0.5, seed=4), dict(src=[1, 2, 3, 5, 8, 13]), dict(closeness=False),
               dict(betweenness=False, tol=5.0)):
        dists = [200, 800, 5000]
        want, reach, sp = _want(ns, dists, **kw)
        res = ns.centrality_shortest(distances=dists, sample_probability=kw.get("p"), random_seed=kw.get("seed"),
                                     source_indices=kw.get("src"), compute_closeness=kw.get("closeness", True),
                                     compute_betweenness=kw.get("betweenness", True), tolerance=kw.get("tol"))
        np.testing.assert_array_equal(res._data, want)
        if kw.get("p") or kw.get("src"):
            assert res.reachability_totals == [int(x) for x in reach]
            assert res.sampled_source_count == sp.sampled_count
    assert lib.calls == 5


def test_more_than_sixteen_thresholds_run_in_groups(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    lib = stand_in(ns)
    dists = list(range(100, 2100, 100))  # 20 thresholds: groups of 16 and 4
    res = ns.centrality_shortest(distances=dists)
    want, _, _ = _want(ns, dists)
    np.testing.assert_array_equal(res._data, want)
    assert lib.calls == 2


def test_sharded_default_share_equals_the_plain_call(stand_in):
    p, dists = synth.lattice_config("c1", side=12)
    ns = synth.primal_structure(p)
    stand_in(ns)
    plain = ns.centrality_shortest(distances=dists, source_indices=list(range(0, 144, 3)))
    shard = sharded_centrality_shortest(ns, distances=dists, source_indices=list(range(0, 144, 3)))
    np.testing.assert_array_equal(shard._data, plain._data)
    assert shard.reachability_totals == plain.reachability_totals


def test_od_host_path(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    stand_in(ns)
    rng = np.random.default_rng(2)
    idx = np.asarray(ns.node_indices())
    od = OdMatrix(rng.choice(idx, 300).tolist(), rng.choice(idx, 300).tolist(), rng.uniform(0, 3, 300).tolist())
    res = ns.betweenness_od_shortest(od, distances=[300, 1200])
    d, b, s = pair_distances_betas_time(1.33333, distances=[300, 1200])
    want = oracle.betweenness_od(oracle.OracleGraph(ns), d, b, s, od.rows(ns.node_bound()), ns=ns)
    np.testing.assert_array_equal(res._data, want)


def test_simplest_host_path(stand_in):
    from cityseer_gb300.tools import graphs

    ns = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    lib = stand_in(ns)
    cases = (dict(), dict(p=0.5, seed=8), dict(src=[0, 4, 9, 16, 25, 36]), dict(asu=90.0, fso=2.0, closeness=True),
             dict(dists=list(range(100, 2000, 100))))
    for kw in cases:
        dists = kw.get("dists", [300, 1200])
        sp = prepare_source_sampling(ns, kw.get("p"), None, kw.get("seed"), kw.get("src"))
        d, b, s = pair_distances_betas_time(1.33333, distances=dists)
        want, reach = oracle.centrality_simplest(oracle.OracleGraph(ns), d, b, s, tol=validate_tolerance(None),
                                                 plan=oracle.plan_from(sp, ns.node_bound()),
                                                 asu=kw.get("asu", 180.0), fso=kw.get("fso", 1.0))
        res = ns.centrality_simplest(distances=dists, sample_probability=kw.get("p"), random_seed=kw.get("seed"),
                                     source_indices=kw.get("src"), angular_scaling_unit=kw.get("asu"),
                                     farness_scaling_offset=kw.get("fso"))
        np.testing.assert_array_equal(res._data, want)
        if kw.get("p") or kw.get("src"):
            assert res.reachability_totals == [int(x) for x in reach]
    assert lib.calls == 6  # 19 thresholds: two groups


def test_segment_host_path(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    ns.set_node_live(ns.node_indices()[3], False)
    lib = stand_in(ns)
    for dists in ([200, 600], list(range(50, 1000, 50))):
        res = ns.segment_centrality(distances=dists)
        d, b, s = pair_distances_betas_time(1.33333, distances=dists)
        np.testing.assert_array_equal(res._data, oracle.segment_centrality(oracle.OracleGraph(ns), d, b, s, ns=ns))
    assert lib.calls == 3
