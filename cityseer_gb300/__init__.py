"""cityseer_gb300: GB300-native (sm_103a) localised network centrality.

A drop-in for cityseer's NetworkStructure.centrality_shortest / centrality_simplest /
segment_centrality (rust/src/centrality.rs in cityseer-api v4.24.0) and the
cityseer.metrics.networks wrappers, computed by hand-written CUDA kernels in libcsgpu.so.
"""
from . import common, config
from .common import (
    betas_from_distances,
    distances_from_betas,
    pair_distances_betas_time,
    seconds_from_distances,
)
from .graph import EdgeVisit, NetworkStructure, NodeVisit

__all__ = [
    "NetworkStructure",
    "NodeVisit",
    "EdgeVisit",
    "pair_distances_betas_time",
    "betas_from_distances",
    "distances_from_betas",
    "seconds_from_distances",
    "common",
    "config",
]
__version__ = "0.1.0"
