"""GPU parity at the benchmark configurations' full sizes, against the oracle.

* The 202,500-node lattice the benchmark times (450x450 at 80 m, diagonals, d = 500/1000/2000/5000 m):
  every output row on 512 evenly strided sources (through source_indices), shortest-path trees at
  3,750 s on a strided subset, and the unweighted betweenness bit for bit on sources whose paths
  are unique within a threshold.
* The curved 250x250 lattice's dual (124,500 dual nodes, d = 500/1000/2000 m): simplest-path
  centrality on 256 strided sources, with the parallel search and with every source forced through
  the exact sequential search.
* An unjittered 300x300 grid at 20 km with a 2% tolerance: equal-cost paths everywhere, so the
  Brandes path counts reach ~1e74 (beyond f32); the kernels carry them, the factors, the seeds and
  the dependencies in f64 as the reference does (rust/src/centrality.rs:397, 823-873, 1806-1808).

Tolerances: reach counts, density and circuit-rank cycles are bit-exact; betweenness (f64
throughout, only the summation order differs) to 1e-9 relative; f32-term closeness sums to the
contract's 1e-5 relative.
"""
import os

import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, synth
from cityseer_gb300.centrality import prepare_source_sampling, validate_tolerance
from helpers import assert_close_sums

ROWS = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
        "node_betweenness_beta")
EXACT = {"node_density", "node_cycles"}
BETW = {"node_betweenness", "node_betweenness_beta"}
RTOL_BETW = 1e-9
SPEED = 1.33333


def _strided(ns, n):
    idx = np.asarray(ns.node_indices())
    return idx[np.linspace(0, len(idx) - 1, n).astype(np.int64)].tolist()


def _oracle_shortest(ns, dists, tol=None, source_indices=None):
    d, b, s = common.pair_distances_betas_time(SPEED, distances=dists)
    sp = prepare_source_sampling(ns, None, None, None, source_indices)
    ref, reach = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, tol=validate_tolerance(tol),
                                            plan=oracle.plan_from(sp, ns.node_bound()),
                                            nthreads=oracle.default_threads())
    return ref, reach, d


def _compare(ns, res, ref, d, what, exact_betw_rows=()):
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(ROWS):
        got = getattr(res, name)
        for i, dist in enumerate(d):
            want = ref[m, i][idx]
            if name in EXACT or (name == "node_betweenness" and i in exact_betw_rows):
                np.testing.assert_array_equal(got[dist], want, err_msg=f"{what} {name}[{dist}]")
            elif name in BETW:
                assert_close_sums(got[dist], want, rtol=RTOL_BETW, atol=1e-12, what=f"{what} {name}[{dist}]")
            else:
                assert_close_sums(got[dist], want, what=f"{what} {name}[{dist}]")


@pytest.fixture(scope="module")
def lattice450():
    p, dists = synth.lattice_config("c2")
    return synth.primal_structure(p), dists


@pytest.mark.gpu
def test_lattice450_strided_sources_all_rows(lattice450):
    ns, dists = lattice450
    srcs = _strided(ns, 512)
    res = ns.centrality_shortest(distances=dists, source_indices=srcs)
    ref, reach, d = _oracle_shortest(ns, dists, source_indices=srcs)
    _compare(ns, res, ref, d, "450x450, 512 sources")
    assert res.reachability_totals == [int(x) for x in reach]
    assert res.sampled_source_count == len(srcs)


@pytest.mark.gpu
def test_lattice450_unique_path_sources_bit_exact(lattice450):
    """Sources whose shortest paths within 500 m (and within 1000 m) are unique in the oracle's
    traversal: their betweenness rows at those thresholds are sums of half-integers, exact in any
    order, so the GPU's must equal the oracle's bit for bit."""
    ns, dists = lattice450
    d, b, s = common.pair_distances_betas_time(SPEED, distances=dists)
    og = oracle.OracleGraph(ns)
    unique = {0: [], 1: []}
    for src in _strided(ns, 256):
        t = oracle.brandes_debug(og, src, max(s), SPEED, pmax=8)
        o = t["order"]
        for k in unique:
            within = t["agg_seconds"][o] <= s[k]
            if np.all(t["sigma"][o][within] == 1.0):
                unique[k].append(src)
    for k, srcs in unique.items():
        assert len(srcs) >= 64, (k, len(srcs))
        res = ns.centrality_shortest(distances=dists, source_indices=srcs)
        ref, reach, d = _oracle_shortest(ns, dists, source_indices=srcs)
        _compare(ns, res, ref, d, f"450x450, unique paths within {d[k]} m", exact_betw_rows=(k,))


@pytest.mark.gpu
def test_lattice450_trees_at_5km(lattice450):
    ns, _ = lattice450
    og = oracle.OracleGraph(ns)
    srcs = _strided(ns, 48)
    trees = ns.dijkstra_tree_shortest_batch(srcs, 3750, SPEED)
    for src, (visited, tree) in zip(srcs, trees):
        vis_ref, t_ref = oracle.tree_shortest(og, src, 3750, SPEED)
        assert sorted(visited) == sorted(vis_ref.tolist()), src
        for v in vis_ref:
            assert tree[v].agg_seconds == t_ref["agg_seconds"][v]
            assert np.float32(tree[v].short_dist) == t_ref["short_dist"][v]
            assert (tree[v].pred if tree[v].pred is not None else -1) == int(t_ref["pred"][v])


@pytest.mark.gpu
def test_exact_grid_20km_tolerance_f64_path_counts():
    """Every path of equal length ties exactly on an unjittered grid, and the 2% tolerance widens the
    predecessor sets further: path counts grow binomially (the oracle's reach 1e73 at 20 km)."""
    g = synth.lattice(side=300, spacing=80.0, jitter=0.0, drop=0.0, seed=7)
    ns = synth.primal_structure(g)
    dists = [2000, 20000]
    d, b, s = common.pair_distances_betas_time(SPEED, distances=dists)
    t = oracle.brandes_debug(oracle.OracleGraph(ns), 150 * 300 + 150, max(s), SPEED, tol=0.02, pmax=8)
    assert t["sigma"].max() > 1e60  # far beyond f32
    srcs = _strided(ns, 16)
    res = ns.centrality_shortest(distances=dists, tolerance=2.0, source_indices=srcs)
    ref, reach, d = _oracle_shortest(ns, dists, tol=2.0, source_indices=srcs)
    for name in ROWS:
        for dist in d:
            assert np.all(np.isfinite(getattr(res, name)[dist])), name
    _compare(ns, res, ref, d, "exact grid 20 km, tolerance 2%")


@pytest.fixture(scope="module")
def curved_dual():
    p, dists = synth.lattice_config("c3")
    return synth.dual_structure(p), dists


def _simplest(ns, dists, srcs, exact):
    d, b, s = common.pair_distances_betas_time(SPEED, distances=dists)
    env = {True: "CS_DUAL_FORCE_EXACT", "wide": "CS_DUAL_WIDE"}.get(exact)
    if env:
        os.environ[env] = "1"  # every source through the exact heap search / the widened search
    try:
        res = ns.centrality_simplest(distances=dists, source_indices=srcs)
    finally:
        if env:
            os.environ.pop(env)
    sp = prepare_source_sampling(ns, None, None, None, srcs)
    ref, reach = oracle.centrality_simplest(oracle.OracleGraph(ns), d, b, s, plan=oracle.plan_from(sp, ns.node_bound()),
                                            nthreads=oracle.default_threads())
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(("node_density", "node_farness", "node_harmonic", "node_betweenness")):
        got = getattr(res, name)
        for i, dist in enumerate(d):
            want = ref[m, i][idx]
            if name == "node_density":
                np.testing.assert_array_equal(got[dist], want, err_msg=f"{name}[{dist}]")
            elif name == "node_betweenness":
                assert_close_sums(got[dist], want, rtol=RTOL_BETW, atol=1e-12, what=f"{name}[{dist}]")
            else:
                assert_close_sums(got[dist], want, what=f"{name}[{dist}]")
    assert res.reachability_totals == [int(x) for x in reach]


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [False, True, "wide"])
def test_curved250_dual_simplest(curved_dual, exact):
    ns, dists = curved_dual
    _simplest(ns, dists, _strided(ns, 256), exact)


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [False, "wide"])
def test_curved250_dual_simplest_at_5km(curved_dual, exact):
    """The full curved dual at 2 and 5 km, where most sources relax states whose offers a later
    relaxation withdraws and replay rounds are most frequent: every row against the oracle."""
    ns, _ = curved_dual
    _simplest(ns, [2000, 5000], _strided(ns, 48), exact)
