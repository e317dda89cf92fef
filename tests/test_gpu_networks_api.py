"""Through the public Python API: metrics.networks wrappers write the reference's column keys with
the raw results (pysrc/cityseer/metrics/networks.py; tests/metrics/test_networks.py:11-176)."""
import numpy as np
import pytest

from cityseer_gb300 import config
from cityseer_gb300.metrics import networks
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph


@pytest.mark.gpu
def test_node_centrality_shortest_columns():
    nodes, _, ns = io.network_structure_from_nx(mock_graph())
    dists = [400, 800]
    frame = networks.node_centrality_shortest(ns, {}, distances=dists)
    raw = ns.centrality_shortest(distances=dists)
    for d in dists:
        for measure, attr in (("beta", "node_beta"), ("cycles", "node_cycles"), ("density", "node_density"),
                              ("farness", "node_farness"), ("harmonic", "node_harmonic"),
                              ("betweenness", "node_betweenness"), ("betweenness_beta", "node_betweenness_beta")):
            np.testing.assert_allclose(frame[config.prep_gdf_key(measure, d)], getattr(raw, attr)[d], rtol=1e-6)
        with np.errstate(divide="ignore", invalid="ignore"):
            hill = raw.node_density[d] ** 2 / raw.node_farness[d]
        np.testing.assert_allclose(frame[f"cc_hillier_{d}"], hill, rtol=1e-6)
    # betas instead of distances resolve to the same columns
    frame2 = networks.node_centrality_shortest(ns, {}, betas=[0.01, 0.005])
    assert "cc_density_400" in frame2 and "cc_density_800" in frame2
    # closeness-only / betweenness-only wrappers
    f3 = networks.closeness_shortest(ns, {}, distances=[400])
    assert "cc_density_400" in f3 and "cc_betweenness_400" not in f3


@pytest.mark.gpu
def test_simplest_and_segment_columns():
    g = mock_graph()
    _, _, nsd = io.network_structure_from_nx(graphs.nx_to_dual(g))
    frame = networks.node_centrality_simplest(nsd, {}, distances=[500])
    raw = nsd.centrality_simplest(distances=[500], angular_scaling_unit=90)
    np.testing.assert_allclose(frame["cc_harmonic_500_ang"], raw.node_harmonic[500], rtol=1e-6)
    np.testing.assert_allclose(frame["cc_betweenness_500_ang"], raw.node_betweenness[500], rtol=1e-6)
    _, _, ns = io.network_structure_from_nx(g)
    with pytest.raises(ValueError, match="dual graph"):
        networks.node_centrality_simplest(ns, {}, distances=[500])
    seg = networks.segment_centrality(ns, {}, distances=[500])
    raw = ns.segment_centrality(distances=[500])
    np.testing.assert_allclose(seg["cc_seg_density_500"], raw.segment_density[500], rtol=1e-6)
    np.testing.assert_allclose(seg["cc_seg_betweenness_500"], raw.segment_betweenness[500], rtol=1e-6)


@pytest.mark.gpu
def test_sampled_schedule_runs():
    nodes, _, ns = io.network_structure_from_nx(mock_graph())
    frame = networks.node_centrality_shortest(ns, {}, distances=[500, 20000], sample=True, random_seed=1)
    assert "cc_density_20000" in frame and np.all(np.isfinite(frame["cc_density_500"]))


@pytest.mark.gpu
def test_progress_is_live_during_a_call():
    """progress() reads the completed-source count from the device while the call runs (the
    reference's progress counter, rust/src/graph.rs:387-415), and equals the source count after."""
    import threading
    import time

    from cityseer_gb300 import synth

    p, dists = synth.lattice_config("c2")
    ns = synth.primal_structure(p)
    ns.centrality_shortest(distances=dists, source_indices=[0])  # device state in place
    seen = []
    th = threading.Thread(target=lambda: ns.centrality_shortest(distances=dists))
    th.start()
    while th.is_alive():
        seen.append(ns.progress())
        time.sleep(0.002)
    th.join()
    n = ns.node_count()
    assert ns.progress() == n
    assert all(0 <= x <= n for x in seen)
    assert any(0 < x < n for x in seen), seen[:20]
