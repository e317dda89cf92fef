"""Batched persistent form: one launch over many graphs, thresholds and modes must give each job the
same result as its own plain call (which the other GPU tests pin to the oracle)."""
import numpy as np
import pytest

from cityseer_gb300 import synth
from cityseer_gb300.batch import Batch

from helpers import assert_close_sums, mock_graph, structure

pytestmark = pytest.mark.gpu

SHORT_ROWS = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
              "node_betweenness_beta")
SEG_ROWS = ("segment_density", "segment_harmonic", "segment_beta", "segment_betweenness")
# integer sums are exact in any order; float sums differ only by atomic summation order
EXACT = {"node_density", "node_cycles"}


def _graphs():
    p1, _ = synth.lattice_config("c1", side=14)
    p2, _ = synth.lattice_config("c2", side=18)
    p3, _ = synth.lattice_config("c3", side=10)
    _, _, mock = structure(mock_graph())
    return [synth.primal_structure(p1), synth.primal_structure(p2), synth.primal_structure(p3), mock]


def _jobs(gs):
    return [
        dict(ns=gs[0], mode="shortest", distances=[500, 1000]),
        dict(ns=gs[1], mode="segment", distances=[400, 800, 1200]),
        dict(ns=gs[2], mode="shortest", distances=[400, 800, 1600, 3200], compute_betweenness=False),
        dict(ns=gs[3], mode="shortest", distances=[200, 500]),
        dict(ns=gs[0], mode="segment", distances=[600]),
        dict(ns=gs[1], mode="shortest", distances=[300, 700, 1200], compute_closeness=False),
    ]


def _plain(spec):
    ns = spec["ns"]
    kw = dict(distances=spec["distances"], compute_closeness=spec.get("compute_closeness", True),
              compute_betweenness=spec.get("compute_betweenness", True))
    if spec["mode"] == "shortest":
        return ns.centrality_shortest(**kw), SHORT_ROWS
    return ns.segment_centrality(**kw), SEG_ROWS


def _check(got, spec, what):
    want, rows = _plain(spec)
    for name in rows:
        g, w = getattr(got, name), getattr(want, name)
        for d in spec["distances"]:
            if name in EXACT:
                np.testing.assert_array_equal(g[d], w[d], err_msg=f"{what} {name}[{d}]")
            else:
                assert_close_sums(g[d], w[d], rtol=1e-9, atol=1e-9, what=f"{what} {name}[{d}]")


def test_batch_matches_plain_calls():
    jobs = _jobs(_graphs())
    b = Batch(jobs)
    assert b.n_items == sum(len(j["ns"].node_indices()) for j in jobs)
    b.run()
    overflowed, done = b.status()
    assert overflowed == 0 and done == b.n_items
    for j, (res, spec) in enumerate(zip(b.results(), jobs)):
        _check(res, spec, f"job {j} ({spec['mode']})")


def test_batch_fused_shortest_segment():
    """A shortest-path job and a segment job on the same graph and thresholds run as one fused job
    (one search per source feeds both) and still equal their plain calls."""
    gs = _graphs()
    jobs = [dict(ns=gs[0], mode="shortest", distances=[500, 1000]),
            dict(ns=gs[0], mode="segment", distances=[500, 1000]),
            dict(ns=gs[1], mode="segment", distances=[300, 800, 1600]),
            dict(ns=gs[1], mode="shortest", distances=[300, 800, 1600]),
            dict(ns=gs[2], mode="segment", distances=[700])]
    b = Batch(jobs, fuse=True)
    assert b.n_fused == 2
    assert b.n_items == sum(len(j["ns"].node_indices()) for j in jobs) - len(gs[0].node_indices()) - \
        len(gs[1].node_indices())
    b.run()
    for j, (res, spec) in enumerate(zip(b.results(), jobs)):
        _check(res, spec, f"job {j} ({spec['mode']}, fused)")
    b.zero_outputs()
    b.capture()
    b.replay()
    for j, (res, spec) in enumerate(zip(b.results(), jobs)):
        _check(res, spec, f"job {j} ({spec['mode']}, fused, graph replay)")


def test_batch_overflow_retry():
    # capacity 48 < reach: most sources overflow and are redone in-call at full capacity
    jobs = _jobs(_graphs())[:3]
    b = Batch(jobs, cap=48, max_slots=64)
    b.run()
    for j, (res, spec) in enumerate(zip(b.results(), jobs)):
        _check(res, spec, f"job {j} ({spec['mode']}, cap 48)")


def test_batch_graph_capture_replay():
    jobs = _jobs(_graphs())
    b = Batch(jobs)
    b.capture()
    for _ in range(2):
        b.replay()
        overflowed, done = b.status()
        assert overflowed == 0 and done == b.n_items
    for j, (res, spec) in enumerate(zip(b.results(), jobs)):
        _check(res, spec, f"job {j} ({spec['mode']}, graph replay)")


def test_batch_rejects_bad_jobs():
    gs = _graphs()
    with pytest.raises(ValueError):
        Batch([dict(ns=gs[0], mode="shortest", distances=list(range(100, 1800, 100)))])
    with pytest.raises(KeyError):
        Batch([dict(ns=gs[0], mode="angular", distances=[500])])


def test_autotuned_schedule_matches_default(tmp_path, monkeypatch):
    """The autotuner times every (band width, register budget) candidate on a sample of sources and
    caches the fastest; a batch built from the cached schedule gives the same rows as the default
    schedule's plain calls."""
    from cityseer_gb300 import autotune, centrality

    monkeypatch.setenv("CS_AUTOTUNE_CACHE", str(tmp_path / "autotune.json"))
    gs = _graphs()
    spec = dict(ns=gs[1], mode="shortest", distances=[400, 900])
    res = autotune.tune(spec["ns"], "shortest", spec["distances"], sample=256)
    assert res["tuned"] and len(res["trials"]) == len(autotune.DELTA_MULTS) * len(autotune.VARIANTS)
    csr = centrality._primal_csr(spec["ns"])
    from cityseer_gb300.common import pair_distances_betas_time

    d, _, s = pair_distances_betas_time(1.33333, distances=spec["distances"])
    hit = autotune.lookup(spec["ns"], csr, "shortest", d, s, 1.33333)
    assert hit["tuned"] and hit["variant"] == res["variant"]
    b = Batch([spec])
    b.run()
    _check(b.results()[0], spec, "tuned batch")
