"""GPU parity: centrality_shortest through the C-ABI vs the oracle (cs_oracle.c)."""
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, synth

from helpers import assert_close_sums, diamond_graph, mock_graph, structure

ROWS = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
        "node_betweenness_beta")
# Integer-valued sums are exact in any order.  Betweenness is a sum of half-integers when every
# source's shortest paths are unique (sigma == 1), exact then; where the reference's 1e-4 near-tie
# rule splits paths (sigma > 1) the terms are non-dyadic fractions and only the f64 summation
# order differs (checked to 1e-12 here, and bit-exact on tie-free sources below).
EXACT = {"node_density", "node_cycles"}
RTOL_ORDER = 1e-12


def _compare(ns, res, ref, dists, exact_rows=EXACT, what="", betw_exact=False):
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(ROWS):
        got = getattr(res, name)
        for i, d in enumerate(dists):
            want = ref[m, i][idx]
            if name in exact_rows or (betw_exact and name == "node_betweenness"):
                np.testing.assert_array_equal(got[d], want, err_msg=f"{what} {name}[{d}]")
            elif name == "node_betweenness":
                assert_close_sums(got[d], want, rtol=RTOL_ORDER, atol=1e-12, what=f"{what} {name}[{d}]")
            else:
                assert_close_sums(got[d], want, what=f"{what} {name}[{d}]")


def tie_free_sources(ns, dists, limit=None):
    """Sources whose Brandes traversal (oracle) has sigma == 1 everywhere."""
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    og = oracle.OracleGraph(ns)
    out = []
    for src in ns.node_indices():
        t = oracle.brandes_debug(og, src, max(s), 1.33333)
        if np.all(t["sigma"][t["order"]] == 1.0):
            out.append(src)
        if limit and len(out) >= limit:
            break
    return out


def _run(ns, dists, **kw):
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    res = ns.centrality_shortest(distances=dists, **kw)
    og = oracle.OracleGraph(ns)
    tol = kw.get("tolerance")
    from cityseer_gb300.centrality import prepare_source_sampling, validate_tolerance

    sp = prepare_source_sampling(ns, kw.get("sample_probability"), kw.get("sampling_weights"),
                                 kw.get("random_seed"), kw.get("source_indices"))
    ref, reach = oracle.centrality_shortest(og, d, b, s, tol=validate_tolerance(tol),
                                            closeness=kw.get("compute_closeness", True) is not False,
                                            betweenness=kw.get("compute_betweenness", True) is not False,
                                            plan=oracle.plan_from(sp, ns.node_bound()))
    return res, ref, reach, d


@pytest.mark.gpu
def test_lattice_c1_full():
    p, dists = synth.lattice_config("c1")
    ns = synth.primal_structure(p)
    res, ref, _, d = _run(ns, dists)
    _compare(ns, res, ref, d, what="c1")


@pytest.mark.gpu
def test_mock_graph_5km_and_small():
    ns = structure(mock_graph())[2]
    for dists in ([5000], [200, 400, 800, 1600]):
        res, ref, _, d = _run(ns, dists)
        _compare(ns, res, ref, d, what=f"mock {dists}")


@pytest.mark.gpu
def test_diamond_golden():
    ns = structure(diamond_graph())[2]
    res, ref, _, d = _run(ns, [50, 150, 250])
    _compare(ns, res, ref, d, what="diamond")


@pytest.mark.gpu
def test_lattice_c1_tie_free_bit_exact():
    p, dists = synth.lattice_config("c1")
    ns = synth.primal_structure(p)
    srcs = tie_free_sources(ns, dists)
    assert len(srcs) > 100
    res, ref, reach, d = _run(ns, dists, source_indices=srcs)
    _compare(ns, res, ref, d, what="c1 tie-free", betw_exact=True)
    assert res.reachability_totals == [int(x) for x in reach]
    assert res.sampled_source_count == len(srcs)
