"""GPU parity: centrality_simplest (angular, dual graph) through the C-ABI vs the oracle."""
import os

import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, synth
from cityseer_gb300.centrality import prepare_source_sampling, validate_tolerance
from cityseer_gb300.tools import graphs, io
from helpers import FIX, assert_close_sums, diamond_graph, mock_graph, nx_from_spec

ROWS = ("node_density", "node_farness", "node_harmonic", "node_betweenness")


def _dual(g):
    return io.network_structure_from_nx(graphs.nx_to_dual(g))


def _run(ns, dists, exact=False, **kw):
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    env = {True: "CS_DUAL_FORCE_EXACT", "wide": "CS_DUAL_WIDE"}.get(exact)
    if env:
        os.environ[env] = "1"  # every source through the exact heap search / the widened search
    try:
        res = ns.centrality_simplest(distances=dists, **kw)
    finally:
        if env:
            os.environ.pop(env)
    sp = prepare_source_sampling(ns, kw.get("sample_probability"), kw.get("sampling_weights"), kw.get("random_seed"),
                                 kw.get("source_indices"))
    ref, reach = oracle.centrality_simplest(oracle.OracleGraph(ns), d, b, s, tol=validate_tolerance(kw.get("tolerance")),
                                            closeness=kw.get("compute_closeness", True) is not False,
                                            betweenness=kw.get("compute_betweenness", True) is not False,
                                            plan=oracle.plan_from(sp, ns.node_bound()),
                                            asu=kw.get("angular_scaling_unit", 180.0),
                                            fso=kw.get("farness_scaling_offset", 1.0))
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(ROWS):
        got = getattr(res, name)
        for i, dist in enumerate(d):
            want = ref[m, i][idx]
            if name == "node_density":
                np.testing.assert_array_equal(got[dist], want, err_msg=f"{name}[{dist}]")
            elif name == "node_betweenness":
                assert_close_sums(got[dist], want, rtol=1e-9, atol=1e-9, what=f"{name}[{dist}]")  # f64 sigma and dependencies
            else:
                assert_close_sums(got[dist], want, what=f"{name}[{dist}]")
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [False, True, "wide"])
def test_simplest_small_graphs(exact):
    _run(_dual(diamond_graph())[2], [50, 150, 250], exact=exact)
    _run(_dual(mock_graph())[2], [200, 500, 2000, 5000], exact=exact)
    _run(_dual(nx_from_spec(FIX["helpers"]["make_angular_plateau_graph"]))[2], [1000], exact=exact)


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [False, True, "wide"])
def test_simplest_curved_lattice_dual(exact):
    p, dists = synth.lattice_config("c3", side=16)
    _run(synth.dual_structure(p), dists, exact=exact)


@pytest.mark.gpu
def test_simplest_options():
    ns = _dual(mock_graph())[2]
    _run(ns, [500, 2000], tolerance=3.0)
    _run(ns, [500, 2000], angular_scaling_unit=90, farness_scaling_offset=2)
    _run(ns, [500, 2000], source_indices=[0, 5, 9, 20])
    _run(ns, [500, 2000], compute_closeness=False)


@pytest.mark.gpu
def test_simplest_diamond_golden_harmonic():
    ns = _dual(diamond_graph())[2]
    res = ns.centrality_simplest(distances=[50, 150, 250], compute_betweenness=False)
    gold = [g for g in FIX["centrality"]["local_centrality_all"] if g["result"] == "node_result_simplest"]
    for gd in gold:
        assert np.allclose(getattr(res, gd["attr"])[gd["distance"]], gd["values"], atol=0.01, rtol=1e-4)


@pytest.mark.gpu
def test_simplest_capacity_chain_and_replay_counts():
    """A plan with a tiny capacity makes most sources overflow; they run again at 4x capacities
    until they fit, and the results equal the default plan's (itself checked against the oracle)."""
    import ctypes as C

    import torch

    from cityseer_gb300 import _native, centrality, dual

    p, dists = synth.lattice_config("c3", side=14)
    ns = synth.dual_structure(p)
    want = _run(ns, dists)
    lib = _native.load()
    over, inexact = C.c_int64(), C.c_int64()
    lib.cs_last_retries(C.byref(over), C.byref(inexact))
    assert inexact.value < len(ns.node_indices())
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    csr = dual.dual_csr(ns)
    plan = _native.Plan()
    _native.check(lib.cs_plan_dual(C.byref(csr.struct(1.33333)), 0, len(d), 64, 64, 0, C.byref(plan)), "plan")
    ws = dual.DualWorkspace(plan, csr.n_bound, csr.device)
    sp = prepare_source_sampling(ns, None, None, None, None)
    dev = csr.device
    keep = [torch.from_numpy(x).to(dev) for x in (sp.process, sp.src_wt, sp.eligible)]
    q = centrality._make_query(d, b, s, 1.33333, 1e-4, True, True, False, *keep)
    out = torch.zeros((4, len(d), csr.n_bound), dtype=torch.float64, device=dev)
    _native.check(lib.cs_centrality_simplest(C.byref(csr.struct(1.33333)), C.byref(q), C.byref(plan), ws.ptr,
                                             ws.nbytes, _native.Outputs(out.data_ptr(), None),
                                             torch.cuda.current_stream().cuda_stream), "simplest small cap")
    lib.cs_last_retries(C.byref(over), C.byref(inexact))
    assert over.value > 0
    got = out.cpu().numpy()
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(ROWS):
        for i, dist in enumerate(d):
            if name == "node_density":
                np.testing.assert_array_equal(got[m, i][idx], getattr(want, name)[dist])
            else:
                assert_close_sums(got[m, i][idx], getattr(want, name)[dist], rtol=1e-9, atol=1e-9,
                                  what=f"{name}[{dist}] (cap 64)")
