"""GPU: the synchronous batched simplest-path run (cs_dual_batch_run without CS_BATCH_ASYNC) over jobs on
two dual graphs equals plain cs_centrality_simplest calls, row for row, with a capacity small enough
that most items overflow and run again at larger capacities, and with every item through the widened
search.  Also: a dual graph without packed edge records is refused."""
import ctypes as C
import os

import numpy as np
import pytest

from cityseer_gb300 import common, synth
from cityseer_gb300.centrality import TIE_EPSILON, prepare_source_sampling
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph

SPEED = 1.33333


def _graphs():
    a = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    p, _ = synth.lattice_config("c3", side=14)
    return [(a, [200, 800, 2000], 0), (synth.dual_structure(p), [500, 1200], 3)]


def _plain_rows(ns, dists, srcs):
    from cityseer_gb300 import dual

    d, b, s = common.pair_distances_betas_time(SPEED, distances=dists)
    sp = prepare_source_sampling(ns, None, None, None, srcs)
    rows, _ = dual.simplest_rows(ns, sp, sp.process, d, b, s, SPEED, float(TIE_EPSILON), 180.0, 1.0, True, True,
                                 False)
    return rows.cpu().numpy(), sp


def _batch(cases, cap, env=None):
    import torch

    from cityseer_gb300 import _native, dual

    lib = _native.load()
    dev = torch.device("cuda", 0)
    n = len(cases)
    jobs = (_native.DualBatchJob * n)()
    keep, outs = [], []
    for j, (ns, dists, srcs, sp) in enumerate(cases):
        d, b, s = common.pair_distances_betas_time(SPEED, distances=dists)
        csr = dual.dual_csr(ns)
        nb = csr.n_bound
        src_t = torch.from_numpy(np.asarray(srcs, np.int32)).to(dev)
        wt_t = torch.from_numpy(sp.src_wt).to(dev)
        el_t = torch.from_numpy(sp.eligible).to(dev)
        out = torch.zeros((4, len(d), nb), dtype=torch.float64, device=dev)
        bucket = torch.zeros((3, len(d), nb), dtype=torch.float64, device=dev)
        jb = jobs[j]
        jb.g = csr.struct(SPEED)
        jb.k = len(d)
        for i, ss in enumerate(s):
            jb.seconds[i] = ss
        jb.tolerance = float(TIE_EPSILON)
        jb.angular_scaling_unit = 180.0
        jb.farness_scaling_offset = 1.0
        jb.compute_closeness = 1
        jb.compute_betweenness = 1
        jb.n_sources = len(srcs)
        jb.sources = src_t.data_ptr()
        jb.src_wt = wt_t.data_ptr()
        jb.eligible = el_t.data_ptr()
        jb.out = out.data_ptr()
        jb.bucket = bucket.data_ptr()
        keep += [src_t, wt_t, el_t, bucket]
        outs.append(out)
    n_items = C.c_int64()
    _native.check(lib.cs_dual_batch_prepare(jobs, n, C.byref(n_items)), "cs_dual_batch_prepare")
    plan = _native.Plan()
    _native.check(lib.cs_dual_batch_plan(jobs, n, cap, 64, 0, C.byref(plan)), "cs_dual_batch_plan")
    ws = dual.DualWorkspace(plan, plan.n_bound, dev)
    raw = bytes(jobs)
    jobs_dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)
    stream = torch.cuda.current_stream()
    if env:
        os.environ[env] = "1"
    try:
        _native.check(lib.cs_dual_batch_run(jobs, jobs_dev.data_ptr(), n, C.byref(plan), ws.ptr, ws.nbytes, 0,
                                            stream.cuda_stream), "cs_dual_batch_run")
    finally:
        if env:
            os.environ.pop(env)
    torch.cuda.synchronize()
    over, exact = C.c_int64(), C.c_int64()
    lib.cs_last_retries(C.byref(over), C.byref(exact))
    return [o.cpu().numpy() for o in outs], over.value


@pytest.mark.gpu
@pytest.mark.parametrize("env", [None, "CS_DUAL_WIDE"])
def test_sync_dual_batch_equals_plain_calls(env):
    cases, want = [], []
    for ns, dists, stride in _graphs():
        idx = np.asarray(ns.node_indices())
        srcs = [int(x) for x in idx[:: max(1, stride)]] if stride else [int(x) for x in idx]
        rows, sp = _plain_rows(ns, dists, srcs)
        cases.append((ns, dists, srcs, sp))
        want.append(rows)
    got, over = _batch(cases, cap=64, env=env)
    if env is None:
        assert over > 0  # capacity 64 < reach: the overflow chain ran
    for j, (g, w) in enumerate(zip(got, want)):
        np.testing.assert_array_equal(g[0], w[0], err_msg=f"job {j} density")
        for r in (1, 2, 3):
            np.testing.assert_allclose(g[r], w[r], rtol=1e-9, atol=1e-9, err_msg=f"job {j} row {r}")


@pytest.mark.gpu
def test_dual_graph_without_packed_records_is_refused():
    import torch

    from cityseer_gb300 import _native, centrality, dual

    ns = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    csr = dual.dual_csr(ns)
    g = csr.struct(SPEED)
    g.fwd_pack = None
    d, b, s = common.pair_distances_betas_time(SPEED, distances=[500])
    sp = prepare_source_sampling(ns, None, None, None, None)
    dev = csr.device
    keep = [torch.from_numpy(x).to(dev) for x in (sp.process, sp.src_wt, sp.eligible)]
    q = centrality._make_query(d, b, s, SPEED, float(TIE_EPSILON), True, True, False, *keep)
    ws = dual.dual_workspace(ns, csr, 1, SPEED, cap=256)
    out = torch.zeros((4, 1, csr.n_bound), dtype=torch.float64, device=dev)
    lib = _native.load()
    rc = lib.cs_centrality_simplest(C.byref(g), C.byref(q), C.byref(ws.plan), ws.ptr, ws.nbytes,
                                    _native.Outputs(out.data_ptr(), None), torch.cuda.current_stream().cuda_stream)
    assert rc == _native.CS_ERR_ARG
    assert "packed edge records" in _native.last_error()
