"""Multi-GPU form (replicas): the throughput reduction over ranks, run as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from cityseer_gb300.replicas import job_throughput


def _free_port() -> int:
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r processed 1000 + r units in 2 + r seconds: the job is as slow as its slowest rank
        value, t_max = job_throughput(1000.0 + rank, 2.0 + rank)
        q.put((rank, value, t_max))
    finally:
        dist.destroy_process_group()


def test_single_process_no_group():
    assert job_throughput(500.0, 2.0) == (250.0, 2.0)


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(90)
        assert pr.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, t_max in got:
        assert t_max == 3.0
        assert value == pytest.approx((1000.0 + 1001.0) / 3.0)


def _oracle_rows(ns, sp, process, dists, bets, secs, speed, tol, closeness, betweenness, track):
    """One rank's share on the CPU: the oracle over `process` under the plan's weights."""
    import numpy as np

    import oracle

    plan = oracle.plan_from(sp, ns.node_bound())
    plan["sources"] = np.asarray(process, np.int64)
    plan["betweenness_scale"] = 1.0  # the sharded form scales after the reduction
    out, reach = oracle.centrality_shortest(oracle.OracleGraph(ns), dists, bets, secs, speed=speed, tol=tol,
                                            closeness=closeness, betweenness=betweenness, plan=plan)
    return torch.from_numpy(out), torch.from_numpy(reach.astype(np.int64))


def _oracle_rows_simplest(ns, sp, process, dists, bets, secs, speed, tol, asu, fso, closeness, betweenness, track):
    import numpy as np

    import oracle

    plan = oracle.plan_from(sp, ns.node_bound())
    plan["sources"] = np.asarray(process, np.int64)
    plan["betweenness_scale"] = 1.0
    out, reach = oracle.centrality_simplest(oracle.OracleGraph(ns), dists, bets, secs, speed=speed, tol=tol,
                                            closeness=closeness, betweenness=betweenness, plan=plan, asu=asu,
                                            fso=fso)
    return torch.from_numpy(out), torch.from_numpy(reach.astype(np.int64))


def _oracle_rows_segment(ns, sources, dists, bets, secs, speed, closeness, betweenness):
    """One rank's share of segment centrality: the oracle over the live nodes, restricted to
    `sources` through the node liveness the oracle reads (a stand-in for the GPU's source list)."""
    import numpy as np

    import oracle

    saved = ns._live.view().copy()
    try:
        keep = np.zeros_like(saved)
        keep[np.asarray(sources, np.int64)] = saved[np.asarray(sources, np.int64)]
        ns._live.view()[:] = keep
        ns._touch()
        out = oracle.segment_centrality(oracle.OracleGraph(ns), dists, bets, secs, speed=speed, closeness=closeness,
                                        betweenness=betweenness, ns=ns)
    finally:
        ns._live.view()[:] = saved
        ns._touch()
    return torch.from_numpy(out)


_SHARD_CASES = [
    dict(distances=[200, 800, 5000]),
    dict(distances=[400, 1600], sample_probability=0.5, random_seed=9),
    dict(distances=[600], source_indices=[0, 3, 5, 8, 13, 21, 34, 40], compute_closeness=False),
]


def _shard_rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from cityseer_gb300.replicas import sharded_centrality_shortest
        from cityseer_gb300.tools import io
        from helpers import mock_graph

        ns = io.network_structure_from_nx(mock_graph())[2]
        for j, kw in enumerate(_SHARD_CASES):
            r = sharded_centrality_shortest(ns, rows_fn=_oracle_rows, **kw)
            q.put((rank, j, r._data, r.reachability_totals, r.sampled_source_count))
        from cityseer_gb300.replicas import sharded_centrality_simplest
        from cityseer_gb300.tools import graphs

        nsd = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
        r = sharded_centrality_simplest(nsd, distances=[300, 1200], sample_probability=0.6, random_seed=2,
                                        rows_fn=_oracle_rows_simplest)
        q.put((rank, "simplest", r._data, r.reachability_totals, r.sampled_source_count))
        from cityseer_gb300.replicas import sharded_segment_centrality

        r = sharded_segment_centrality(ns, distances=[200, 600], rows_fn=_oracle_rows_segment)
        q.put((rank, "segment", r._data, [], 0))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_sharded_single_graph_equals_one_process():
    """Two gloo ranks, each running half of the sources through the oracle, then one sum all-reduce,
    equal the whole job run in one process (plain, sampled, source-indexed)."""
    import numpy as np

    from cityseer_gb300.replicas import sharded_centrality_shortest
    from cityseer_gb300.tools import io
    from helpers import mock_graph

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = [q.get(timeout=150) for _ in range(2 * (len(_SHARD_CASES) + 2))]
    for pr in procs:
        pr.join(60)
        assert pr.exitcode == 0
    from cityseer_gb300.replicas import sharded_centrality_simplest
    from cityseer_gb300.tools import graphs

    nsd = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    want_s = sharded_centrality_simplest(nsd, distances=[300, 1200], sample_probability=0.6, random_seed=2,
                                         rows_fn=_oracle_rows_simplest)
    import oracle
    from cityseer_gb300.common import pair_distances_betas_time

    ns_p = io.network_structure_from_nx(mock_graph())[2]
    d, b, s = pair_distances_betas_time(1.33333, distances=[200, 600])
    want_seg = oracle.segment_centrality(oracle.OracleGraph(ns_p), d, b, s, ns=ns_p)
    for rank, jj, data, reach, sampled in got:
        if jj == "segment":
            np.testing.assert_allclose(data, want_seg, rtol=1e-9, atol=1e-9)
        if jj == "simplest":
            np.testing.assert_allclose(data, want_s._data, rtol=1e-12, atol=1e-12)
            assert reach == want_s.reachability_totals and sampled == want_s.sampled_source_count
    ns = io.network_structure_from_nx(mock_graph())[2]
    for j, kw in enumerate(_SHARD_CASES):
        want = sharded_centrality_shortest(ns, rows_fn=_oracle_rows, **kw)  # no process group: one rank
        for rank, jj, data, reach, sampled in got:
            if jj != j:
                continue
            np.testing.assert_allclose(data, want._data, rtol=1e-12, atol=1e-12)
            assert reach == want.reachability_totals and sampled == want.sampled_source_count


def test_sharded_form_without_a_group_equals_the_oracle_call():
    import numpy as np

    import oracle
    from cityseer_gb300.centrality import prepare_source_sampling, validate_tolerance
    from cityseer_gb300.common import pair_distances_betas_time
    from cityseer_gb300.replicas import sharded_centrality_shortest
    from cityseer_gb300.tools import io
    from helpers import mock_graph

    ns = io.network_structure_from_nx(mock_graph())[2]
    for kw in _SHARD_CASES:
        got = sharded_centrality_shortest(ns, rows_fn=_oracle_rows, **kw)
        sp = prepare_source_sampling(ns, kw.get("sample_probability"), None, kw.get("random_seed"),
                                     kw.get("source_indices"))
        d, b, s = pair_distances_betas_time(1.33333, distances=kw["distances"])
        want, _ = oracle.centrality_shortest(oracle.OracleGraph(ns), d, b, s, tol=validate_tolerance(None),
                                             closeness=kw.get("compute_closeness", True),
                                             plan=oracle.plan_from(sp, ns.node_bound()))
        np.testing.assert_array_equal(got._data, want)
