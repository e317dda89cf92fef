"""Constants and helpers of pysrc/cityseer/config.py (column keys, thresholds, progress)."""
from __future__ import annotations

import os
import threading
import time
from collections.abc import Callable
from queue import Queue

MIN_THRESH_WT: float = 0.01831563888873418
SPEED_M_S = 1.33333
ATOL: float = 0.01
RTOL: float = 0.0001


def prep_gdf_key(key: str, dist: int, angular: bool = False, weighted: bool | None = None) -> str:
    """Column label, pysrc/cityseer/config.py:21-32."""
    key = key.replace(".0", "")
    key = key.replace(".0_", "_")
    key = f"cc_{key}_{dist}"
    if angular is True:
        key += "_ang"
    if weighted is True:
        key += "_wt"
    elif weighted is False:
        key += "_nw"
    return key


def check_quiet() -> bool:
    if "GCP_PROJECT" in os.environ:
        return True
    return os.environ.get("CITYSEER_QUIET_MODE", "").lower() in ("true", "1")


QUIET_MODE = check_quiet()


def check_debug() -> bool:
    """CITYSEER_DEBUG_MODE set to true or 1 (pysrc/cityseer/config.py:48-53)."""
    return os.environ.get("CITYSEER_DEBUG_MODE", "").lower() in ("true", "1")


DEBUG_MODE: bool = check_debug()
SKIP_VALIDATION: bool = False


def log_thresholds(distances=None, betas=None, minutes=None, min_threshold_wt: float = MIN_THRESH_WT,
                   speed_m_s: float = SPEED_M_S) -> list[int]:
    """Resolves and logs the thresholds, returning the distances (pysrc/cityseer/config.py:67-83)."""
    import logging

    from .common import pair_distances_betas_time

    dists, betas_, secs = pair_distances_betas_time(speed_m_s, distances, betas, minutes,
                                                    min_threshold_wt=min_threshold_wt)
    log = logging.getLogger(__name__)
    log.info("Metrics computed for:")
    for d, b, t in zip(dists, betas_, secs):
        log.info(f"Distance: {d}m, Beta: {round(b, 5)}, Walking Time: {t / 60} minutes.")
    return dists


def wrap_progress(total: int, rust_struct, partial_func: Callable, desc: str | None = None):
    """Runs partial_func on a worker thread and polls rust_struct.progress() meanwhile (live for
    NetworkStructure calls: the kernels count completed sources on the device), re-raising worker
    exceptions (pysrc/cityseer/config.py:96-130)."""
    q: Queue = Queue()

    def worker():
        try:
            q.put(partial_func())
        except Exception as e:  # noqa: BLE001
            q.put(e)

    th = threading.Thread(target=worker)
    th.start()
    while th.is_alive():
        time.sleep(0.05)
    th.join()
    res = q.get()
    if isinstance(res, Exception):
        raise res
    return res
