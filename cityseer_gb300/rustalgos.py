"""Namespace mirror of the reference's compiled module `cityseer.rustalgos` (rust/src/lib.rs:37-164)
for the parts this package implements: `rustalgos.graph.NetworkStructure`, the centrality result
classes and the threshold conversions."""
from types import SimpleNamespace

from . import centrality as _c
from . import graph as _g
from .common import (
    avg_distances_for_betas,
    betas_from_distances,
    check_numerical_data,
    clip_wts_curve,
    clipped_beta_wt,
    distances_from_betas,
    distances_from_seconds,
    pair_distances_betas_time,
    seconds_from_distances,
)

graph = SimpleNamespace(NetworkStructure=_g.NetworkStructure, NodeVisit=_g.NodeVisit, EdgeVisit=_g.EdgeVisit,
                        NodePayload=_g.NodePayload, EdgePayload=_g.EdgePayload)
centrality = SimpleNamespace(
    CentralityShortestResult=_c.CentralityShortestResult,
    CentralitySimplestResult=_c.CentralitySimplestResult,
    CentralitySegmentResult=_c.CentralitySegmentResult,
    BetweennessShortestResult=_c.BetweennessShortestResult,
    OdMatrix=_c.OdMatrix,
)

__all__ = ["graph", "centrality", "pair_distances_betas_time", "betas_from_distances", "distances_from_betas",
           "seconds_from_distances", "distances_from_seconds", "avg_distances_for_betas", "clip_wts_curve",
           "clipped_beta_wt", "check_numerical_data"]
