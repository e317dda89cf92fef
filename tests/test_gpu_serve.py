"""Served form: every query's result is the same served alone, served in a mix of concurrent
queries of other graphs, sizes, thresholds and modes, and computed by the plain call."""
import numpy as np
import pytest

from cityseer_gb300 import synth
from cityseer_gb300.serve import Query, Server, latency_summary

from helpers import assert_close_sums

pytestmark = pytest.mark.gpu

EXACT = {"node_density", "node_cycles"}


def _world():
    prims, duals = {}, {}
    for gid, side in enumerate((20, 28, 12)):
        p = synth.lattice(side=side, spacing=100.0, jitter=20.0, drop=0.15, seed=40 + gid)
        prims[gid] = synth.primal_structure(p)
        if gid < 2:
            duals[gid] = synth.dual_structure(p)
    return prims, duals


def _queries(prims, duals, n=28, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        r = rng.random()
        mode = "shortest" if r < 0.55 else ("segment" if r < 0.7 else ("simplest" if r < 0.92 else "isochrone"))
        gid = int(rng.integers(0, 2 if mode == "simplest" else 3))
        ns = duals[gid] if mode == "simplest" else prims[gid]
        idx = np.asarray(ns.node_indices())
        size = int(np.exp(rng.uniform(0, np.log(min(300, len(idx))))))
        src = np.sort(rng.choice(idx, size=size, replace=False)).tolist()
        k = int(rng.integers(1, 5))
        dmax = int(rng.uniform(300, 1500))
        dists = sorted(set([dmax] + [int(rng.uniform(100, dmax)) for _ in range(k - 1)]))
        betw = bool(rng.random() < 0.8)
        out.append(Query(gid, src, dists, mode, compute_closeness=True, compute_betweenness=betw))
    return out


def _rows(res, mode):
    names = {"shortest": ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta",
                          "node_betweenness", "node_betweenness_beta"),
             "segment": ("segment_density", "segment_harmonic", "segment_beta", "segment_betweenness"),
             "simplest": ("node_density", "node_farness", "node_harmonic", "node_betweenness")}[mode]
    return {nm: getattr(res, nm) for nm in names}


def _same(a, b, q, what):
    if q.mode == "isochrone":
        ca, na, aa, pa = a
        cb, nb_, ab, pb = b
        np.testing.assert_array_equal(ca, cb, err_msg=what)
        for i in range(len(ca)):
            np.testing.assert_array_equal(na[i, :ca[i]], nb_[i, :cb[i]], err_msg=what)
            np.testing.assert_array_equal(aa[i, :ca[i]], ab[i, :cb[i]], err_msg=what)
        return
    ra, rb = _rows(a, q.mode), _rows(b, q.mode)
    for nm in ra:
        for d in q.distances:
            if nm in EXACT and q.mode == "shortest":
                np.testing.assert_array_equal(ra[nm][d], rb[nm][d], err_msg=f"{what} {nm}[{d}]")
            else:
                assert_close_sums(ra[nm][d], rb[nm][d], rtol=1e-9, atol=1e-9, what=f"{what} {nm}[{d}]")


def _plain(q, prims, duals):
    if q.mode == "shortest":
        return prims[q.graph].centrality_shortest(distances=q.distances, source_indices=q.sources,
                                                  compute_betweenness=q.compute_betweenness)
    if q.mode == "simplest":
        return duals[q.graph].centrality_simplest(distances=q.distances, source_indices=q.sources,
                                                  compute_betweenness=q.compute_betweenness)
    return None


def test_served_alone_equals_mix_equals_plain():
    prims, duals = _world()
    qs = _queries(prims, duals)
    srv = Server(prims, duals, max_distance=1500, wave_cost=64)
    with srv:
        mix = [srv.submit(q) for q in qs]
        srv.drain(timeout=300)
        alone = []
        for q in qs:
            t = srv.submit(q)
            assert t.wait(120)
            alone.append(t)
    assert srv.stats()["waves"] > 1
    for i, (q, tm, ta) in enumerate(zip(qs, mix, alone)):
        rm, ra = tm.result(), ta.result()
        _same(rm, ra, q, f"query {i} ({q.mode}, graph {q.graph}, {len(q.sources)} sources) mix vs alone")
        rp = _plain(q, prims, duals)
        if rp is not None:
            _same(rm, rp, q, f"query {i} ({q.mode}) served vs plain call")
    s = latency_summary(mix)
    assert s["n"] == len(qs)


def test_served_overflow_rerun_and_empty_query():
    prims, duals = _world()
    qs = [q for q in _queries(prims, duals, n=14, seed=11) if q.mode in ("shortest", "segment", "simplest")]
    qs.append(Query(1, [], [800], "shortest"))
    # capacity 48 < reach: most sources overflow in the async waves and are re-run synchronously
    # (primal and dual waves alike)
    srv = Server(prims, duals, max_distance=1500, cap=48, max_slots=64)
    with srv:
        ts = [srv.submit(q) for q in qs]
        srv.drain(timeout=300)
    n_checked = 0
    for i, (q, t) in enumerate(zip(qs[:-1], ts[:-1])):
        ref = _plain(q, prims, duals)
        if ref is not None:
            _same(t.result(), ref, q, f"query {i} ({q.mode}, cap 48) vs plain call")
            n_checked += 1
        else:
            assert t.result() is not None
    assert n_checked > 0
    assert np.all(ts[-1].result().node_density[800] == 0.0)


def test_served_rejects_bad_queries():
    prims, duals = _world()
    srv = Server(prims, None, max_distance=1000)
    with pytest.raises(ValueError):
        srv.submit(Query(0, [0], [1200]))
    with pytest.raises(ValueError):
        srv.submit(Query(0, [0], [100, 200, 300, 400, 500]))
    with pytest.raises(ValueError):
        srv.submit(Query(0, [0], [500], mode="simplest"))
    with srv:
        t = srv.submit(Query(0, [10 ** 7], [500]))
        assert t.wait(60)
    with pytest.raises(ValueError):
        t.result()
