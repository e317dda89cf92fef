"""Schedule autotuner for the persistent kernels.

Tunes the label-correcting search's band width (multiples of the median edge travel time) and the
register budget (3 or 2 resident blocks per SM) by timing a sample of sources with CUDA events.
Results are cached in a JSON file (CS_AUTOTUNE_CACHE, default ~/.cache/cityseer_gb300/autotune.json)
keyed on (mode, graph size, mean out-degree, max threshold, threshold count).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from pathlib import Path

import numpy as np
import torch

from . import _native, centrality, device
from .common import pair_distances_betas_time

DELTA_MULTS = (1.0, 2.0, 4.0)
VARIANTS = (4, 3, 2)


def cache_path() -> Path:
    return Path(os.environ.get("CS_AUTOTUNE_CACHE", Path.home() / ".cache" / "cityseer_gb300" / "autotune.json"))


_memo: dict = {}


def _load() -> dict:
    p = cache_path()
    try:
        mt = p.stat().st_mtime_ns
    except OSError:
        return {}
    hit = _memo.get(str(p))
    if hit is not None and hit[0] == mt:
        return hit[1]
    try:
        db = json.loads(p.read_text())
    except (OSError, ValueError):
        return {}
    _memo[str(p)] = (mt, db)
    return db


def _store(db: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(db, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass


def key_of(csr, mode: str, secs, k: int) -> str:
    n = max(1, csr.n_bound)
    deg = csr.m / n
    return f"{mode}|n2^{round(math.log2(n))}|deg{round(deg * 2) / 2}|t{int(max(secs))}|k{k}"


def default(csr, speed: float) -> dict:
    # variant 0: the library's register budget per mode (3 blocks per SM for shortest paths, 4 for
    # segments)
    return {"delta": 2.0 * csr.median_edge_seconds(speed), "variant": 0, "tuned": False}


def lookup(ns, csr, mode: str, d, s, speed: float) -> dict:
    hit = _load().get(key_of(csr, mode, s, len(d)))
    if hit is None:
        return default(csr, speed)
    med = csr.median_edge_seconds(speed)
    return {"delta": hit["delta_mult"] * med, "variant": hit["variant"], "tuned": True}


def _time_sample(ns, csr, mode_i: int, d, b, s, speed, src, delta, variant, reps=2) -> float:
    lib = _native.load()
    plan = device.plan_primal(csr, mode_i, len(d), speed, cap=int(min(csr.n_bound, max(1024, 1.3 *
                              centrality.estimate_reach(ns, csr, speed, max(s))))), delta=delta, variant=variant,
                              mem_budget=centrality._mem_budget(csr.device))
    ws = device.Workspace(plan, csr.n_bound, csr.device)
    dev = csr.device
    sp = centrality.prepare_source_sampling(ns, None, None, None, None)
    proc = torch.from_numpy(src.astype(np.int32)).to(dev)
    q = centrality._make_query(d, b, s, speed, 1e-4, True, True, False, proc, torch.from_numpy(sp.src_wt).to(dev),
                               torch.from_numpy(sp.eligible).to(dev))
    out = torch.zeros((7 if mode_i == 0 else 4, len(d), csr.n_bound), dtype=torch.float64, device=dev)
    g = csr.struct(speed)
    fn = lib.cs_centrality_shortest if mode_i == 0 else lib.cs_segment_centrality
    best = float("inf")
    stream = torch.cuda.current_stream()
    for r in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _native.check(fn(C.byref(g), C.byref(q), C.byref(plan), ws.ptr, ws.nbytes,
                         _native.Outputs(out.data_ptr(), None), stream.cuda_stream), "autotune sample")
        e1.record(stream)
        e1.synchronize()
        if r > 0:
            best = min(best, e0.elapsed_time(e1))
    del ws
    return best


def tune(ns, mode: str, distances, speed: float = 1.33333, sample: int = 2048) -> dict:
    """Times every candidate schedule on an even sample of sources and caches the fastest."""
    csr = centrality._primal_csr(ns)
    d, b, s = pair_distances_betas_time(speed, distances=distances)
    key = key_of(csr, mode, s, len(d))
    idx = np.asarray(ns.node_indices(), np.int64)
    src = idx[np.linspace(0, len(idx) - 1, min(sample, len(idx))).astype(np.int64)]
    med = csr.median_edge_seconds(speed)
    mode_i = 0 if mode == "shortest" else 1
    trials = []
    for v in VARIANTS:
        for m in DELTA_MULTS:
            trials.append((_time_sample(ns, csr, mode_i, d, b, s, speed, src, m * med, v), m, v))
    t, m, v = min(trials)
    db = _load()
    db[key] = {"delta_mult": m, "variant": v, "ms_per_sample": t, "sample": len(src),
               "trials": [[tt, mm, vv] for tt, mm, vv in trials]}
    _store(db)
    return {"delta": m * med, "variant": v, "tuned": True, "trials": trials}
