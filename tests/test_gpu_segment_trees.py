"""GPU parity: segment_centrality and shortest-path trees (isochrones) vs the oracle."""
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, synth
from helpers import assert_close_sums, diamond_graph, mock_graph, structure

SEG_ROWS = ("segment_density", "segment_harmonic", "segment_beta", "segment_betweenness")


def _seg(ns, dists):
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    res = ns.segment_centrality(distances=dists)
    ref = oracle.segment_centrality(oracle.OracleGraph(ns), d, b, s, ns=ns)
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(SEG_ROWS):
        got = getattr(res, name)
        for i, dist in enumerate(d):
            # sums of f32 integrals in a different order; harmonic/beta integrals use logf/expf
            assert_close_sums(got[dist], ref[m, i][idx], rtol=1e-5, atol=1e-6, what=f"{name}[{dist}]")


@pytest.mark.gpu
def test_segment_lattice_mock_diamond():
    p, dists = synth.lattice_config("c1")
    _seg(synth.primal_structure(p), dists)
    _seg(structure(mock_graph())[2], [200, 400, 800, 5000])
    _seg(structure(diamond_graph())[2], [50, 150, 250])


@pytest.mark.gpu
def test_trees_bit_exact():
    for ns in (synth.primal_structure(synth.lattice_config("c1")[0]), structure(mock_graph())[2]):
        og = oracle.OracleGraph(ns)
        srcs = ns.node_indices()[::7]
        for max_seconds in (0, 375, 1500, 3750):
            trees = ns.dijkstra_tree_shortest_batch(srcs, max_seconds, 1.33333)
            for src, (visited, tree) in zip(srcs, trees):
                vis_ref, t_ref = oracle.tree_shortest(og, src, max_seconds, 1.33333)
                assert sorted(visited) == sorted(vis_ref.tolist())
                for v in vis_ref:
                    assert tree[v].agg_seconds == t_ref["agg_seconds"][v]
                    assert np.float32(tree[v].short_dist) == t_ref["short_dist"][v]
                    want_pred = int(t_ref["pred"][v])
                    assert (tree[v].pred if tree[v].pred is not None else -1) == want_pred
                # settle order: equal unless two nodes share a distance
                dref = t_ref["agg_seconds"][vis_ref]
                if len(np.unique(dref)) == len(dref):
                    assert visited == vis_ref.tolist()
