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
