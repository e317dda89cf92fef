"""cityseer.metrics.networks wrappers on the CPU (the reference's tests/metrics/test_networks.py:
11-244): the cc_* columns equal the raw results for every flag combination and for distances or
betas given, simplest scaling options, segment columns, and seeded sampled schedules are
deterministic.  The C-ABI calls are answered by the oracle-backed stand-in (tests/standin.py)."""
import numpy as np
import pytest

import standin
from cityseer_gb300 import config
from cityseer_gb300.common import betas_from_distances
from cityseer_gb300.metrics import networks
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph

DISTS = [400, 800]


@pytest.fixture
def stand_in(monkeypatch):
    return standin.install(monkeypatch)


def test_node_centrality_shortest_columns(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    stand_in(ns)
    betas = betas_from_distances(DISTS)
    close = ns.centrality_shortest(compute_closeness=True, compute_betweenness=False, betas=betas)
    betw = ns.centrality_shortest(compute_closeness=False, compute_betweenness=True, distances=DISTS)
    for c, b in [(False, True), (True, False), (True, True)]:
        for d_in, b_in in [(DISTS, None), (None, betas)]:
            cols = networks.node_centrality_shortest(ns, {}, distances=d_in, betas=b_in, compute_closeness=c,
                                                     compute_betweenness=b)
            for d in DISTS:
                if c:
                    for m, attr in (("beta", "node_beta"), ("cycles", "node_cycles"), ("density", "node_density"),
                                    ("farness", "node_farness"), ("harmonic", "node_harmonic")):
                        np.testing.assert_allclose(cols[config.prep_gdf_key(m, d)], getattr(close, attr)[d])
                    with np.errstate(divide="ignore", invalid="ignore"):
                        np.testing.assert_allclose(cols[config.prep_gdf_key("hillier", d)],
                                                   close.node_density[d] ** 2 / close.node_farness[d])
                if b:
                    for m, attr in (("betweenness", "node_betweenness"), ("betweenness_beta", "node_betweenness_beta")):
                        np.testing.assert_allclose(cols[config.prep_gdf_key(m, d)], getattr(betw, attr)[d])
                if not c:
                    assert config.prep_gdf_key("density", d) not in cols
                if not b:
                    assert config.prep_gdf_key("betweenness", d) not in cols


def test_node_centrality_simplest_columns(stand_in):
    ns = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    stand_in(ns)
    betas = betas_from_distances(DISTS)
    betw = ns.centrality_simplest(compute_closeness=False, compute_betweenness=True, betas=betas)
    for d_in, b_in in [(DISTS, None), (None, betas)]:
        for fso, asu in [(0, 180), (0, 90), (1, 180)]:
            cols = networks.node_centrality_simplest(ns, {}, distances=d_in, betas=b_in, farness_scaling_offset=fso,
                                                     angular_scaling_unit=asu)
            close = ns.centrality_simplest(compute_closeness=True, compute_betweenness=False, betas=betas,
                                           farness_scaling_offset=fso, angular_scaling_unit=asu)
            for d in DISTS:
                for m, attr in (("density", "node_density"), ("farness", "node_farness"),
                                ("harmonic", "node_harmonic")):
                    np.testing.assert_allclose(cols[config.prep_gdf_key(m, d, angular=True)], getattr(close, attr)[d])
                with np.errstate(divide="ignore", invalid="ignore"):
                    np.testing.assert_allclose(cols[config.prep_gdf_key("hillier", d, angular=True)],
                                               close.node_density[d] ** 2 / close.node_farness[d])
                np.testing.assert_allclose(cols[config.prep_gdf_key("betweenness", d, angular=True)],
                                           betw.node_betweenness[d])


def test_segment_centrality_columns(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    stand_in(ns)
    betas = betas_from_distances(DISTS)
    for c, b in [(False, True), (True, False), (True, True)]:
        raw = ns.segment_centrality(betas=betas, compute_closeness=c, compute_betweenness=b)
        for d_in, b_in in [(DISTS, None), (None, betas)]:
            cols = networks.segment_centrality(ns, {}, distances=d_in, betas=b_in, compute_closeness=c,
                                               compute_betweenness=b)
            for d in DISTS:
                if c:
                    for m, attr in (("seg_density", "segment_density"), ("seg_harmonic", "segment_harmonic"),
                                    ("seg_beta", "segment_beta")):
                        np.testing.assert_allclose(cols[config.prep_gdf_key(m, d)], getattr(raw, attr)[d])
                if b:
                    np.testing.assert_allclose(cols[config.prep_gdf_key("seg_betweenness", d)],
                                               raw.segment_betweenness[d])


def test_closeness_wrappers_and_seeded_sampling(stand_in):
    ns = io.network_structure_from_nx(mock_graph())[2]
    stand_in(ns)
    dists = [200, 400, 800]
    from cityseer_gb300 import sampling

    assert sampling.compute_distance_p(800, epsilon=0.3) < 1.0  # the 800 m column is sampled
    r1 = networks.closeness_shortest(ns, {}, distances=dists, random_seed=42, sample=True, epsilon=0.3)
    r2 = networks.closeness_shortest(ns, {}, distances=dists, random_seed=42, sample=True, epsilon=0.3)
    r3 = networks.closeness_shortest(ns, {}, distances=dists, random_seed=43, sample=True, epsilon=0.3)
    assert not np.array_equal(r1[config.prep_gdf_key("density", 800)], r3[config.prep_gdf_key("density", 800)])
    for d in dists:
        for m in ("harmonic", "density", "farness", "beta", "cycles", "hillier"):
            assert config.prep_gdf_key(m, d) in r1
        np.testing.assert_array_equal(r1[config.prep_gdf_key("density", d)], r2[config.prep_gdf_key("density", d)])
    nsd = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    stand_in(nsd)
    s1 = networks.closeness_simplest(nsd, {}, distances=dists, random_seed=42)
    s2 = networks.closeness_simplest(nsd, {}, distances=dists, random_seed=42)
    for d in dists:
        for m in ("harmonic", "density", "farness", "hillier"):
            assert config.prep_gdf_key(m, d, angular=True) in s1
        key = config.prep_gdf_key("density", d, angular=True)
        np.testing.assert_array_equal(s1[key], s2[key])
