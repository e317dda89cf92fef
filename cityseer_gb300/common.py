"""Threshold conversions: distances <-> betas <-> seconds.

Same names, arguments and ValueError messages as the reference's ``rustalgos`` functions
(rust/src/common.rs:99-270).  The arithmetic runs in f32 inside libcsgpu.so's host code
(cs_pair_distances_betas_time) so that results are bit-identical to the reference's f32 maths.
"""
from __future__ import annotations

import ctypes as C
from collections.abc import Sequence

import numpy as np

from . import _native

MIN_THRESH_WT = 0.01831563888873418  # rust/src/common.rs:10
WALKING_SPEED = 1.33333  # rust/src/common.rs:12


def _call(speed_m_s: float, mode: int, values: Sequence, min_threshold_wt: float | None):
    lib = _native.load()
    k = len(values)
    if k == 0:
        name = ("distances", "betas", "minutes")[mode]
        if mode == 2:
            raise ValueError("Input 'seconds' cannot be empty.")
        raise ValueError(f"Input '{name}' cannot be empty.")
    dist_in = np.zeros(k, np.uint32)
    beta_in = np.zeros(k, np.float32)
    min_in = np.zeros(k, np.float32)
    if mode == 0:
        arr = np.asarray(values)
        if np.any(arr < 0):
            raise ValueError("Distances must be positive integers.")
        dist_in[:] = arr.astype(np.int64)
    elif mode == 1:
        beta_in[:] = np.asarray(values, dtype=np.float32)
    else:
        min_in[:] = np.asarray(values, dtype=np.float32)
    od = np.zeros(k, np.uint32)
    ob = np.zeros(k, np.float32)
    os_ = np.zeros(k, np.uint32)
    mtw = -1.0 if min_threshold_wt is None else float(np.float32(min_threshold_wt))
    rc = lib.cs_pair_distances_betas_time(
        C.c_float(speed_m_s),
        mode,
        k,
        dist_in.ctypes.data,
        beta_in.ctypes.data,
        min_in.ctypes.data,
        C.c_float(mtw),
        od.ctypes.data,
        ob.ctypes.data,
        os_.ctypes.data,
    )
    _native.check(rc)
    return [int(x) for x in od], [float(x) for x in ob], [int(x) for x in os_]


def pair_distances_betas_time(
    speed_m_s: float,
    distances: Sequence[int] | None = None,
    betas: Sequence[float] | None = None,
    minutes: Sequence[float] | None = None,
    min_threshold_wt: float | None = None,
) -> tuple[list[int], list[float], list[int]]:
    """Resolves exactly one of distances / betas / minutes into (distances, betas, seconds)."""
    given = [x is not None for x in (distances, betas, minutes)]
    if sum(given) != 1:
        raise ValueError(
            "Please provide exactly one of the following arguments: 'distances', 'betas', or 'minutes'."
        )
    if distances is not None:
        return _call(speed_m_s, 0, list(distances), min_threshold_wt)
    if betas is not None:
        return _call(speed_m_s, 1, list(betas), min_threshold_wt)
    return _call(speed_m_s, 2, list(minutes), min_threshold_wt)


def betas_from_distances(distances: Sequence[int], min_threshold_wt: float | None = None) -> list[float]:
    return _call(WALKING_SPEED, 0, list(distances), min_threshold_wt)[1]


def distances_from_betas(betas: Sequence[float], min_threshold_wt: float | None = None) -> list[int]:
    return _call(WALKING_SPEED, 1, list(betas), min_threshold_wt)[0]


def seconds_from_distances(distances: Sequence[int], speed_m_s: float) -> list[int]:
    if speed_m_s <= 0:
        raise ValueError("Speed must be positive.")
    return _call(speed_m_s, 0, list(distances), None)[2]


# ---------------------------------------------------------------------------------------------
# The remaining top-level helpers of rustalgos (rust/src/common.rs:74-89, 167-201, 273-347), in f32.
# The data-aggregation modules use them; centrality does not.
# ---------------------------------------------------------------------------------------------
def _f32(x) -> np.float32:
    return np.float32(x)


def _round_half_away(v: np.float32) -> float:
    """f32::round: halves away from zero (exact in f64 for every f32 value)."""
    import math

    x = float(v)
    return float(math.floor(x + 0.5)) if x >= 0 else -float(math.floor(-x + 0.5))


def check_numerical_data(data_arr) -> None:
    """Every element of a 2D f32 array must be finite (rust/src/common.rs:74-89)."""
    a = np.asarray(data_arr, dtype=np.float32)
    if a.ndim != 2:
        raise TypeError("check_numerical_data expects a 2D array")
    if not np.all(np.isfinite(a)):
        raise ValueError("The numeric data values must be finite.")


def distances_from_seconds(seconds: Sequence[int], speed_m_s: float) -> list[int]:
    """rust/src/common.rs:167-201."""
    secs = list(seconds)
    if not secs:
        raise ValueError("Input 'seconds' cannot be empty.")
    if _f32(speed_m_s) <= 0.0:
        raise ValueError("Speed must be positive.")
    if any(b <= a for a, b in zip(secs, secs[1:])):
        raise ValueError("Times must be unique and sorted in strictly increasing order.")
    out = []
    for t in secs:
        if t == 0:
            raise ValueError("Time values must be positive integers.")
        d = _round_half_away(_f32(_f32(t) * _f32(speed_m_s)))
        if d <= 0.0:
            raise ValueError("Derived distance must be positive. Check time and speed values.")
        out.append(int(d))
    return out


def avg_distances_for_betas(betas: Sequence[float], min_threshold_wt: float | None = None) -> list[float]:
    """Mean distance under each beta's decay curve up to its threshold distance
    (rust/src/common.rs:273-308)."""
    bs = list(betas)
    if not bs:
        raise ValueError("Input 'betas' cannot be empty.")
    mtw = MIN_THRESH_WT if min_threshold_wt is None else min_threshold_wt
    dists = distances_from_betas(bs, mtw)
    out = []
    for b, d in zip(bs, dists):
        beta = _f32(b)
        if abs(beta) < np.finfo(np.float32).eps:
            raise ValueError(f"Beta ({b}) must not be zero during average distance calculation.")
        with np.errstate(all="ignore"):
            auc = _f32(_f32(np.exp(_f32(-beta * _f32(d))) - _f32(1.0)) / -beta)
            wt = _f32(auc / _f32(d))
        if not wt > 0.0:
            raise ValueError(f"Invalid weight ({wt}) encountered during average distance calculation.")
        out.append(float(_f32(-np.log(wt) / beta)))
    return out


def clip_wts_curve(distances: Sequence[int], betas: Sequence[float], spatial_tolerance: int) -> list[float]:
    """exp(-beta * spatial_tolerance) per threshold (rust/src/common.rs:311-336)."""
    ds, bs = list(distances), list(betas)
    if len(ds) != len(bs):
        raise ValueError("Input 'distances' and 'betas' must have the same length.")
    out = []
    for d, b in zip(ds, bs):
        if spatial_tolerance > d:
            raise ValueError(f"Clipping distance ({spatial_tolerance}) cannot be greater than the distance "
                             f"threshold ({d}).")
        out.append(float(_f32(np.exp(_f32(-_f32(b) * _f32(spatial_tolerance))))))
    return out


def clipped_beta_wt(beta: float, max_curve_wt: float, data_dist: float) -> float:
    """min(exp(-beta d), max_curve_wt) / max_curve_wt (rust/src/common.rs:339-347)."""
    mcw = _f32(max_curve_wt)
    if not (0.0 <= mcw <= 1.0):
        raise ValueError("Max curve weight must be in the range [0, 1].")
    raw = _f32(np.exp(_f32(-_f32(beta) * _f32(data_dist))))
    with np.errstate(all="ignore"):
        return float(_f32(min(raw, mcw) / mcw))
