"""Source sampling with inverse-probability weights (rust/src/centrality.rs:1032-1139), checked the way
the reference's own sampling tests check it (tests/test_sampling.py: reproducibility, p = 1, IPW
convergence, target coverage, sampling weights, simplest paths, betweenness), on the host plan
(`prepare_source_sampling`, with the StdRng stream) and the oracle's centralities, without a GPU.
The GPU path consumes the same plan; its parity with the oracle is in the -m gpu tests."""
import numpy as np
import pytest

import oracle
from cityseer_gb300.centrality import prepare_source_sampling, validate_tolerance
from cityseer_gb300.common import pair_distances_betas_time
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph

D = 500


@pytest.fixture(scope="module")
def primal():
    _, _, ns = io.network_structure_from_nx(mock_graph())
    return ns, oracle.OracleGraph(ns)


@pytest.fixture(scope="module")
def dual():
    _, _, ns = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))
    return ns, oracle.OracleGraph(ns)


def _rows(g, p=None, seed=None, weights=None, closeness=True, betweenness=False, simplest=False):
    ns, og = g
    sp = prepare_source_sampling(ns, p, weights, seed, None)
    plan = oracle.plan_from(sp, ns.node_bound())
    d, b, s = pair_distances_betas_time(1.33333, distances=[D])
    fn = oracle.centrality_simplest if simplest else oracle.centrality_shortest
    out, _ = fn(og, d, b, s, tol=validate_tolerance(None), closeness=closeness, betweenness=betweenness, plan=plan)
    return out[:, 0][:, np.asarray(ns.node_indices())]


def _rel_err(avg, full):
    m = full > 0
    return float(np.mean(np.abs(avg[m] - full[m]) / full[m]))


def test_p_one_matches_full(primal):
    np.testing.assert_array_equal(_rows(primal, 1.0, 42)[0], _rows(primal)[0])


def test_same_seed_same_result_other_seed_differs(primal):
    a, b, c = _rows(primal, 0.5, 42)[0], _rows(primal, 0.5, 42)[0], _rows(primal, 0.5, 43)[0]
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)


def test_averaged_density_converges(primal):
    full = _rows(primal)[0]
    avg = np.mean([_rows(primal, 0.5, seed)[0] for seed in range(20)], axis=0)
    assert _rel_err(avg, full) < 0.15


def test_ipw_keeps_the_mean_across_probabilities(primal):
    full = _rows(primal)[0]
    full_mean = full[full > 0].mean()
    for p in (0.3, 0.5, 0.7):
        means = []
        for seed in range(25):
            dens = _rows(primal, p, seed)[0]
            m = (dens > 0) & (full > 0)
            if m.any():
                means.append(dens[m].mean())
        assert abs(np.mean(means) - full_mean) / full_mean < 0.25, p


def test_target_coverage(primal):
    full, samp = _rows(primal)[0], _rows(primal, 0.5, 42)[0]
    m = full > 0
    assert (m & (samp > 0)).sum() / m.sum() > 0.9
    full_c, samp_c = _rows(primal)[2], _rows(primal, 0.5, 42)[2]
    mc = full_c > 0
    if mc.sum() > 1:
        assert np.corrcoef(full_c[mc], samp_c[mc])[0, 1] > 0.6


def test_sampling_weights(primal):
    ns, _ = primal
    n = ns.node_count()
    half = [1.0 if i < n // 2 else 0.0 for i in range(n)]
    sp = prepare_source_sampling(ns, 1.0, half, None, None)
    assert set(sp.process.tolist()) <= set(np.asarray(ns.node_indices())[: n // 2].tolist())
    assert (_rows(primal, 1.0, None, half)[0] > 0).sum() > 0
    uni = np.mean([_rows(primal, 1.0, seed, [0.5] * n)[0] for seed in range(25)], axis=0)
    plain = np.mean([_rows(primal, 0.5, seed)[0] for seed in range(25)], axis=0)
    m = (uni > 0) & (plain > 0)
    assert np.corrcoef(uni[m], plain[m])[0, 1] > 0.95


def test_simplest_sampling(dual):
    a = _rows(dual, 0.3, 42, simplest=True)[0]
    np.testing.assert_array_equal(a, _rows(dual, 0.3, 42, simplest=True)[0])
    full = _rows(dual, simplest=True)[0]
    avg = np.mean([_rows(dual, 0.5, seed, simplest=True)[0] for seed in range(15)], axis=0)
    assert _rel_err(avg, full) < 0.20


def test_betweenness_sampling_converges(primal):
    full = _rows(primal, closeness=False, betweenness=True)[5]
    avg = np.mean([_rows(primal, 0.5, seed, closeness=False, betweenness=True)[5] for seed in range(20)], axis=0)
    assert _rel_err(avg, full) < 0.25


def test_hoeffding_model():
    """The reach -> p model (pysrc/cityseer/sampling.py:32-104; tests/test_sampling.py:414-490)."""
    import math

    from cityseer_gb300 import sampling

    assert (sampling.HOEFFDING_EPSILON, sampling.HOEFFDING_DELTA) == (0.06, 0.1)
    k = math.log(2 * 1000.0 / 0.1) / (2 * 0.1 ** 2)
    assert sampling.compute_hoeffding_p(1000.0, epsilon=0.1, delta=0.1) == pytest.approx(min(1.0, k / 1000.0))
    ps = [sampling.compute_hoeffding_p(r) for r in (200.0, 500.0, 1000.0, 5000.0, 10000.0)]
    assert all(a >= b for a, b in zip(ps, ps[1:]))
    for bad in (sampling.compute_hoeffding_p(50.0), sampling.compute_hoeffding_p(0), sampling.compute_hoeffding_p(-100),
                sampling.compute_hoeffding_p(1000.0, delta=0.0), sampling.compute_hoeffding_p(1000.0, delta=1.0)):
        assert bad == 1.0
    pd = [sampling.compute_distance_p(d) for d in (500, 1000, 2000, 5000, 10000, 20000)]
    assert all(a >= b for a, b in zip(pd, pd[1:])) and 0.0 < sampling.compute_distance_p(2000) <= 1.0
    assert sampling.compute_distance_p(100) == 1.0 and sampling.compute_distance_p(0) == 1.0
    assert sampling.compute_distance_p(5000, epsilon=0.05) >= sampling.compute_distance_p(5000, epsilon=0.1)


def test_tolerance_zero_is_the_default_and_tolerance_moves_betweenness(primal):
    """tests/test_sampling.py:574-618: tolerance 0 equals the default; a wide tolerance spreads
    betweenness over near-equal paths."""
    ns, og = primal
    d, b, s = pair_distances_betas_time(1.33333, distances=[D])
    plan = oracle.all_sources_plan(ns)
    default, _ = oracle.centrality_shortest(og, d, b, s, tol=validate_tolerance(None), plan=plan)
    zero, _ = oracle.centrality_shortest(og, d, b, s, tol=validate_tolerance(0.0), plan=plan)
    wide, _ = oracle.centrality_shortest(og, d, b, s, tol=validate_tolerance(10.0), plan=plan)
    np.testing.assert_array_equal(default, zero)
    assert not np.allclose(default[5], wide[5])
