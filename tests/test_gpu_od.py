"""GPU parity: betweenness_od_shortest through the C-ABI (cs_betweenness_od_shortest) vs the oracle."""
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, synth
from cityseer_gb300.centrality import OdMatrix, validate_tolerance
from cityseer_gb300.metrics import networks

from helpers import assert_close_sums, mock_graph, structure

pytestmark = pytest.mark.gpu

# trip weights are arbitrary f32 values; the GPU carries the seeds and dependencies in f64 as the
# reference does (rust/src/centrality.rs:2495-2512), so only the summation order differs
RTOL = 1e-9
ATOL = 1e-9


def _random_od(ns, n_pairs, seed, zero_frac=0.1):
    rng = np.random.default_rng(seed)
    idx = np.asarray(ns.node_indices())
    o = rng.choice(idx, n_pairs)
    d = rng.choice(idx, n_pairs)
    d[:5] = o[:5]  # origin == destination: no effect in the reference
    w = rng.uniform(0.1, 5.0, n_pairs).astype(np.float32)
    w[rng.random(n_pairs) < zero_frac] = 0.0
    # repeated pairs: the last weight counts
    o = np.concatenate([o, o[:20]])
    d = np.concatenate([d, d[:20]])
    w = np.concatenate([w, rng.uniform(0.1, 5.0, 20).astype(np.float32)])
    return OdMatrix(o.tolist(), d.tolist(), w.tolist())


def _check(ns, od, dists, tolerance=None, what=""):
    res = ns.betweenness_od_shortest(od, distances=dists, tolerance=tolerance)
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    ref = oracle.betweenness_od(oracle.OracleGraph(ns), d, b, s, od.rows(ns.node_bound()),
                                tol=validate_tolerance(tolerance), ns=ns)
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(("node_betweenness", "node_betweenness_beta")):
        got = getattr(res, name)
        for i, dd in enumerate(d):
            assert_close_sums(got[dd], ref[m, i][idx], rtol=RTOL, atol=ATOL, what=f"{what} {name}[{dd}]")
    return res, ref


def test_mock_graph_random_od():
    _, _, ns = structure(mock_graph())
    od = _random_od(ns, 400, 1)
    res, ref = _check(ns, od, [200, 500, 1500], what="mock")
    assert ref[0].max() > 0
    _check(ns, od, [300, 5000], tolerance=5.0, what="mock tol 5%")


def test_lattice_c1_random_od_and_subset_of_origins():
    p, dists = synth.lattice_config("c1")
    ns = synth.primal_structure(p)
    _check(ns, _random_od(ns, 6000, 2), dists, what="c1")
    # few origins with dense rows
    rng = np.random.default_rng(3)
    idx = np.asarray(ns.node_indices())
    o = np.repeat(rng.choice(idx, 7, replace=False), 300)
    d = rng.choice(idx, len(o))
    od = OdMatrix(o.tolist(), d.tolist(), rng.uniform(1, 2, len(o)).tolist())
    _check(ns, od, dists, what="c1 dense rows")


def test_all_pairs_equals_twice_shortest_betweenness():
    p, _ = synth.lattice_config("c1", side=16)
    ns = synth.primal_structure(p)
    idx = ns.node_indices()
    o = [a for a in idx for b in idx if a != b]
    t = [b for a in idx for b in idx if a != b]
    res = ns.betweenness_od_shortest(OdMatrix(o, t, [1.0] * len(o)), distances=[400, 900])
    short = ns.centrality_shortest(distances=[400, 900], compute_closeness=False)
    for dd in (400, 900):
        assert_close_sums(res.node_betweenness[dd], 2.0 * short.node_betweenness[dd], rtol=1e-9, atol=1e-9,
                          what=f"all pairs [{dd}]")
        assert_close_sums(res.node_betweenness_beta[dd], 2.0 * short.node_betweenness_beta[dd], rtol=1e-9,
                          atol=1e-9, what=f"all pairs beta [{dd}]")


def test_edge_cases_and_wrapper():
    p, _ = synth.lattice_config("c1", side=12)
    ns = synth.primal_structure(p)
    idx = ns.node_indices()
    # zero weights (tests/test_sampling.py:708-724) and an empty matrix give zeros
    res = ns.betweenness_od_shortest(OdMatrix([idx[0], idx[1]], [idx[1], idx[2]], [0.0, 0.0]), distances=[500])
    assert np.all(res.node_betweenness[500] == 0.0)
    res = ns.betweenness_od_shortest(OdMatrix([], [], []), distances=[500])
    assert np.all(res.node_betweenness[500] == 0.0) and len(res.node_betweenness[500]) == len(idx)
    # a destination beyond the node bound
    with pytest.raises(ValueError):
        ns.betweenness_od_shortest(OdMatrix([idx[0]], [ns.node_bound() + 3], [1.0]), distances=[500])
    # a removed origin and a non-live origin are skipped
    od = _random_od(ns, 500, 4)
    ns.remove_street_node(idx[10])
    ns.set_node_live(idx[11], False)
    _check(ns, od, [300, 700], what="gaps")
    # the networks wrapper writes cc_betweenness_{d} / cc_betweenness_beta_{d}
    out = networks.betweenness_od(ns, None, od, distances=[300, 700])
    assert set(out) >= {"cc_betweenness_300", "cc_betweenness_beta_700"}
