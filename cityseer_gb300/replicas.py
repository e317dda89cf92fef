"""Multi-GPU forms.  Sources are independent units:

* replicas: N ranks (one process per GPU) each run a whole workload with no collective on the data
  path; the only exchange is the timing reduction (`job_throughput`: the slowest rank's time), which
  turns per-rank work into the whole job's throughput;
* one graph sharded by sources (`sharded_centrality_shortest`): every rank holds the graph, runs a
  strided slice of the sources, and one f64 sum all-reduce of the accumulator rows gives every rank
  the whole result.
"""
from __future__ import annotations

import os

import numpy as np
import torch


def job_throughput(units_per_rank: float, seconds: float, device: torch.device | None = None) -> tuple[float, float]:
    """(units of all ranks / slowest rank's seconds, slowest seconds).  Works on one process (no
    process group) and under torch.distributed with any backend (nccl on GPUs, gloo on CPU)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units_per_rank / seconds, seconds
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units_per_rank)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    t_max = float(t.item())
    return float(u.item()) / t_max, t_max


def _sharded(ns, kind, distances, betas, minutes, compute_closeness, compute_betweenness, min_threshold_wt,
             speed_m_s, tolerance, sample_probability, sampling_weights, random_seed, source_indices, group,
             rows_fn, extra):
    import torch.distributed as dist

    from . import centrality as c
    from .common import WALKING_SPEED, pair_distances_betas_time

    closeness = True if compute_closeness is None else bool(compute_closeness)
    betweenness = True if compute_betweenness is None else bool(compute_betweenness)
    if not closeness and not betweenness:
        raise ValueError(
            "Either or both closeness and betweenness flags is required, but both parameters are False.")
    speed = WALKING_SPEED if speed_m_s is None else float(speed_m_s)
    tol = c.validate_tolerance(tolerance)
    dists, bets, secs = pair_distances_betas_time(speed, distances, betas, minutes, min_threshold_wt)
    on = dist.is_available() and dist.is_initialized()
    world = dist.get_world_size(group) if on else 1
    rank = dist.get_rank(group) if on else 0
    seed = random_seed
    if world > 1 and sample_probability is not None and seed is None:
        box = [int.from_bytes(os.urandom(8), "little") if rank == 0 else None]
        dist.broadcast_object_list(box, src=dist.get_global_rank(group, 0) if group is not None else 0, group=group)
        seed = box[0]
    sp = c.prepare_source_sampling(ns, sample_probability, sampling_weights, seed, source_indices)
    track = sp.sample_probability is not None or sp.is_source_indexed
    mine = np.ascontiguousarray(sp.process[rank::world])
    if kind == "shortest":
        fn = rows_fn if rows_fn is not None else c.shortest_rows
        rows, reach = fn(ns, sp, mine, dists, bets, secs, speed, tol, closeness, betweenness, track)
    else:
        from . import dual

        fn = rows_fn if rows_fn is not None else dual.simplest_rows
        rows, reach = fn(ns, sp, mine, dists, bets, secs, speed, tol, extra[0], extra[1], closeness, betweenness,
                         track)
    if world > 1:
        dist.all_reduce(rows, op=dist.ReduceOp.SUM, group=group)
        dist.all_reduce(reach, op=dist.ReduceOp.SUM, group=group)
    data, reach_tot = rows.cpu().numpy(), reach.cpu().numpy()
    if kind == "shortest":
        return c.finish_shortest(ns, dists, sp, data, reach_tot, betweenness, track)
    from . import dual

    return dual.finish_simplest(ns, dists, sp, data, reach_tot, betweenness, track)


def sharded_centrality_shortest(ns, distances=None, betas=None, minutes=None, compute_closeness=None,
                                compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, tolerance=None,
                                sample_probability=None, sampling_weights=None, random_seed=None,
                                source_indices=None, group=None, rows_fn=None):
    """centrality_shortest (rust/src/centrality.rs:1624-1874) for one graph over the ranks of a process
    group: the same source plan on every rank (a sampled plan without a seed takes rank 0's seed),
    rank r runs the plan's sources r, r + N, ..., and the rows and reach counts are summed over the
    ranks (NCCL on GPUs; any backend for `rows_fn` results on the CPU).  Every rank returns the whole
    result.  Without a process group it is centrality_shortest.  rows_fn(ns, plan, sources, distances,
    betas, seconds, speed, tolerance, closeness, betweenness, track) -> (rows, reach) computes one
    rank's share; the default runs it on the GPU (centrality.shortest_rows)."""
    return _sharded(ns, "shortest", distances, betas, minutes, compute_closeness, compute_betweenness,
                    min_threshold_wt, speed_m_s, tolerance, sample_probability, sampling_weights, random_seed,
                    source_indices, group, rows_fn, None)


def sharded_centrality_simplest(ns, distances=None, betas=None, minutes=None, compute_closeness=None,
                                compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, tolerance=None,
                                angular_scaling_unit=None, farness_scaling_offset=None, sample_probability=None,
                                sampling_weights=None, random_seed=None, source_indices=None, group=None,
                                rows_fn=None):
    """centrality_simplest (rust/src/centrality.rs:1880-2132) sharded like sharded_centrality_shortest;
    rows_fn(ns, plan, sources, distances, betas, seconds, speed, tolerance, angular_scaling_unit,
    farness_scaling_offset, closeness, betweenness, track) defaults to dual.simplest_rows."""
    ns.validate_dual_for_angular("centrality_simplest")
    asu = 180.0 if angular_scaling_unit is None else float(angular_scaling_unit)
    fso = 1.0 if farness_scaling_offset is None else float(farness_scaling_offset)
    return _sharded(ns, "simplest", distances, betas, minutes, compute_closeness, compute_betweenness,
                    min_threshold_wt, speed_m_s, tolerance, sample_probability, sampling_weights, random_seed,
                    source_indices, group, rows_fn, (asu, fso))


def sharded_segment_centrality(ns, distances=None, betas=None, minutes=None, compute_closeness=None,
                               compute_betweenness=None, min_threshold_wt=None, speed_m_s=None, group=None,
                               rows_fn=None):
    """segment_centrality (rust/src/centrality.rs:2134-2407) sharded like sharded_centrality_shortest:
    rank r runs the live sources r, r + N, ... and the rows are summed over the ranks.
    rows_fn(ns, sources, distances, betas, seconds, speed, closeness, betweenness) -> rows defaults to
    centrality.segment_rows."""
    import torch.distributed as dist

    from . import centrality as c
    from .common import WALKING_SPEED, pair_distances_betas_time

    speed = WALKING_SPEED if speed_m_s is None else float(speed_m_s)
    dists, bets, secs = pair_distances_betas_time(speed, distances, betas, minutes, min_threshold_wt)
    closeness = True if compute_closeness is None else bool(compute_closeness)
    betweenness = True if compute_betweenness is None else bool(compute_betweenness)
    if not closeness and not betweenness:
        raise ValueError(
            "Either or both closeness and betweenness flags is required, but both parameters are False.")
    on = dist.is_available() and dist.is_initialized()
    world = dist.get_world_size(group) if on else 1
    rank = dist.get_rank(group) if on else 0
    mine = np.ascontiguousarray(c.segment_sources(ns)[rank::world])
    fn = rows_fn if rows_fn is not None else c.segment_rows
    rows = fn(ns, mine, dists, bets, secs, speed, closeness, betweenness)
    if world > 1:
        dist.all_reduce(rows, op=dist.ReduceOp.SUM, group=group)
    return c.finish_segment(ns, dists, rows.cpu().numpy())
