"""GPU parity: centrality_shortest through the C-ABI vs the oracle (cs_oracle.c)."""
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, synth

from helpers import assert_close_sums, diamond_graph, mock_graph, structure

ROWS = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
        "node_betweenness_beta")
# Integer-valued sums are exact in any order.  Betweenness is a sum of half-integers when every
# source's shortest paths are unique (sigma == 1), exact then (bit-exact test on tie-free sources
# below); where the reference's 1e-4 near-tie rule splits paths (sigma > 1) the dependencies are
# non-dyadic fractions.  The kernel carries path counts, factors, seeds and dependencies in f64 as
# the reference does, so only the summation order differs: 1e-9 relative.
EXACT = {"node_density", "node_cycles"}
RTOL_ORDER = 1e-9


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


@pytest.mark.gpu
def test_phase2_tolerance_and_weights():
    p, dists = synth.lattice_config("c1", side=24)
    ns = synth.primal_structure(p)
    res, ref, _, d = _run(ns, dists, tolerance=2.0)
    _compare(ns, res, ref, d, what="tolerance 2%")
    w = np.random.default_rng(5).uniform(0.5, 2.0, ns.node_count()).astype(np.float32)
    nsw = synth.primal_structure(p)
    nsw._weight.view()[:] = w
    nsw._touch()
    res, ref, _, d = _run(nsw, dists)
    _compare(nsw, res, ref, d, exact_rows=set(), what="node weights")


@pytest.mark.gpu
def test_sampling_and_source_subsets():
    p, dists = synth.lattice_config("c1", side=24)
    ns = synth.primal_structure(p)
    res, ref, reach, d = _run(ns, dists, sample_probability=0.4, random_seed=11)
    _compare(ns, res, ref, d, what="sampled")
    assert res.reachability_totals == [int(x) for x in reach] and res.sampled_source_count > 0
    n = ns.node_count()
    sw = np.linspace(0.0, 1.0, n).astype(np.float32)
    res, ref, reach, d = _run(ns, dists, sample_probability=0.8, sampling_weights=sw, random_seed=3)
    _compare(ns, res, ref, d, what="sampling weights")
    ns.set_node_live(5, False)
    res, ref, _, d = _run(ns, dists, compute_closeness=False)
    _compare(ns, res, ref, d, what="betweenness only, one node not live")
    res, ref, _, d = _run(ns, dists, compute_betweenness=False)
    _compare(ns, res, ref, d, what="closeness only")


@pytest.mark.gpu
def test_capacity_overflow_is_retried_inside_the_call():
    """Force a reach capacity far below the reach: every source overflows its slot, the call
    resets the slots and redoes the sources at full capacity; results are unchanged."""
    import ctypes as C

    import torch

    from cityseer_gb300 import _native, centrality, device

    p, dists = synth.lattice_config("c1", side=20)
    ns = synth.primal_structure(p)
    want = ns.centrality_shortest(distances=dists)
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    csr = centrality._primal_csr(ns)
    plan = device.plan_primal(csr, 0, len(d), 1.33333, cap=40, max_slots=64)
    assert plan.cap == 40
    ws = device.Workspace(plan, csr.n_bound, csr.device)
    sp = centrality.prepare_source_sampling(ns, None, None, None, None)
    dev = csr.device
    q = centrality._make_query(d, b, s, 1.33333, 1e-4, True, True, False, torch.from_numpy(sp.process).to(dev),
                               torch.from_numpy(sp.src_wt).to(dev), torch.from_numpy(sp.eligible).to(dev))
    out = torch.zeros((7, len(d), csr.n_bound), dtype=torch.float64, device=dev)
    reach = torch.zeros(len(d), dtype=torch.int32, device=dev)
    lib = _native.load()
    rc = lib.cs_centrality_shortest(C.byref(csr.struct(1.33333)), C.byref(q), C.byref(plan), ws.ptr, ws.nbytes,
                                    _native.Outputs(out.data_ptr(), reach.data_ptr()), None)
    _native.check(rc)
    got = out.cpu().numpy()
    counters = centrality.last_counters()
    assert counters[3] >= 2, counters  # main launch and the full-capacity retry launch
    assert counters[0] == len(sp.process), counters
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(ROWS):
        for i, dist in enumerate(d):
            np.testing.assert_allclose(got[m, i][idx], getattr(want, name)[dist], rtol=1e-9, atol=1e-9)


@pytest.mark.gpu
def test_removed_nodes_and_index_gaps():
    p, dists = synth.lattice_config("c1", side=16)
    ns = synth.primal_structure(p)
    for v in (3, 40, 41, 100):
        ns.remove_street_node(v)
    res, ref, _, d = _run(ns, dists)
    assert len(res.node_indices) == ns.node_count()
    _compare(ns, res, ref, d, what="gaps")


@pytest.mark.gpu
def test_beta_seed_exp_f64_accuracy():
    """The beta-weighted seeds w * exp(-(beta * cost)) of the betweenness kernels against numpy's f64
    exp of the same exact f32 x f32 product (the reference's arithmetic), over betas 4 / d for
    d in 100 m .. 20 km and costs 0 .. 2 d, plus out-of-table arguments."""
    import torch

    from cityseer_gb300 import _native

    rng = np.random.default_rng(3)
    n = 1 << 20
    d = rng.uniform(100.0, 20000.0, n)
    beta = np.round(4.0 / d, 5).astype(np.float32)
    cost = (rng.uniform(0.0, 2.0, n) * d).astype(np.float32)
    w = rng.choice(np.array([0.5, 1.0, 0.37, 3.0], np.float32), n)
    beta[:64] = rng.uniform(0.05, 0.5, 64).astype(np.float32)  # arguments beyond the table (>= 8)
    dev = torch.device("cuda", 0)
    tw, tb, tc = (torch.from_numpy(x).to(dev) for x in (w, beta, cost))
    out = torch.empty(n, dtype=torch.float64, device=dev)
    _native.check(_native.load().cs_debug_seed_exp(tw.data_ptr(), tb.data_ptr(), tc.data_ptr(), out.data_ptr(), n,
                                                   None), "cs_debug_seed_exp")
    got = out.cpu().numpy()
    want = w.astype(np.float64) * np.exp(-(beta.astype(np.float64) * cost.astype(np.float64)))
    rel = np.abs(got - want) / np.maximum(want, 1e-200)
    assert rel.max() < 5e-14, (rel.max(), int(rel.argmax()))


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", ["0", "1"])
def test_both_schedules_against_the_oracle(schedule, monkeypatch):
    """A call runs one warp per source (throughput) or one block per source (latency) by its source
    count; each schedule, forced for every call, matches the oracle: C1 with every source, a 2%
    tolerance, sampling weights and a source subset."""
    monkeypatch.setenv("CS_BLOCK_PER_SOURCE", schedule)
    p, dists = synth.lattice_config("c1")
    ns = synth.primal_structure(p)
    res, ref, _, d = _run(ns, dists)
    _compare(ns, res, ref, d, what=f"c1 schedule {schedule}")
    p24, dists24 = synth.lattice_config("c1", side=24)
    ns24 = synth.primal_structure(p24)
    res, ref, _, d = _run(ns24, dists24, tolerance=2.0)
    _compare(ns24, res, ref, d, what=f"tolerance 2% schedule {schedule}")
    res, ref, reach, d = _run(ns24, dists24, source_indices=list(range(0, 576, 7)))
    _compare(ns24, res, ref, d, what=f"subset schedule {schedule}")
    assert res.reachability_totals == [int(x) for x in reach]
