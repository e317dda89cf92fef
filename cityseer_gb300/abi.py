"""Public helpers for calling libcsgpu.so's C-ABI (include/cityseer_gb300.h) directly, as a binding in
another host package would: the device CSR of a graph, a planned workspace, the query struct and the
output rows of one centrality call, all owned by the returned object (keep it alive while the call
runs).  `NetworkStructure.centrality_shortest` / `centrality_simplest` do the same and then post-scale
and compact the rows; the raw rows here are [metric][threshold][node_bound], before any post-scale.
Calls built for the same graph share that graph's workspace (as the public API's calls do): issue
them one after another on one stream, never concurrently.

    call = abi.shortest_call(ns, distances=[500, 2000])
    rc = abi.library().cs_centrality_shortest(*call.args())
    abi.check(rc)                     # CS_ERR_* -> ValueError / RuntimeError, the reference's messages
    rows = call.out.cpu().numpy()     # rows: density, farness, cycles, harmonic, beta, betweenness,
                                      #       betweenness_beta (rust/src/centrality.rs:1624-1874)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native, centrality, dual
from .common import pair_distances_betas_time
from .config import SPEED_M_S

__all__ = ["library", "check", "Call", "shortest_call", "simplest_call"]


def library() -> C.CDLL:
    """libcsgpu.so with every entry point's ctypes signature declared."""
    return _native.load()


def check(rc: int, what: str = "") -> None:
    """Raises the error a non-zero status stands for (ValueError for argument errors, with the
    library's message)."""
    _native.check(rc, what)


@dataclass
class Call:
    """Everything one centrality call takes: C structs, the workspace and the zeroed output rows."""
    graph: C.Structure
    query: _native.Query
    plan: _native.Plan
    workspace: object
    out: torch.Tensor
    reach: torch.Tensor
    stream: int
    keep: list = field(default_factory=list)

    def args(self) -> tuple:
        """The argument tuple of cs_centrality_shortest / cs_centrality_simplest."""
        return (C.byref(self.graph), C.byref(self.query), C.byref(self.plan), self.workspace.ptr,
                self.workspace.nbytes, _native.Outputs(self.out.data_ptr(), self.reach.data_ptr()), self.stream)


def _plan_tensors(ns, source_indices, dev):
    sp = centrality.prepare_source_sampling(ns, None, None, None, source_indices)
    keep = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (sp.process, sp.src_wt, sp.eligible)]
    return sp, keep


def shortest_call(ns, distances, speed_m_s: float = SPEED_M_S, tolerance: float | None = None,
                  compute_closeness: bool = True, compute_betweenness: bool = True,
                  source_indices=None) -> Call:
    """The arguments of one cs_centrality_shortest call over a primal graph (at most 16 thresholds;
    every source, or `source_indices`)."""
    d, b, s = pair_distances_betas_time(speed_m_s, distances=list(distances))
    if len(d) > _native.MAX_K:
        raise ValueError("a call takes at most 16 thresholds")
    csr = centrality._primal_csr(ns)
    dev = csr.device
    ws = centrality._workspace(ns, csr, 0, len(d), speed_m_s, max(s))
    _, keep = _plan_tensors(ns, source_indices, dev)
    q = centrality._make_query(d, b, s, speed_m_s, centrality.validate_tolerance(tolerance), compute_closeness,
                               compute_betweenness, True, *keep)
    out = torch.zeros((7, len(d), csr.n_bound), dtype=torch.float64, device=dev)
    reach = torch.zeros(len(d), dtype=torch.int32, device=dev)
    return Call(csr.struct(speed_m_s), q, ws.plan, ws, out, reach, torch.cuda.current_stream(dev).cuda_stream, keep)


def simplest_call(ns_dual, distances, speed_m_s: float = SPEED_M_S, tolerance: float | None = None,
                  compute_closeness: bool = True, compute_betweenness: bool = True, source_indices=None,
                  angular_scaling_unit: float = 180.0, farness_scaling_offset: float = 1.0) -> Call:
    """The arguments of one cs_centrality_simplest call over a dual graph (rows: density, farness,
    harmonic, betweenness; every call searches to its largest threshold)."""
    d, b, s = pair_distances_betas_time(speed_m_s, distances=list(distances))
    if len(d) > _native.MAX_K:
        raise ValueError("a call takes at most 16 thresholds")
    csr = dual.dual_csr(ns_dual)
    dev = csr.device
    ws = dual.dual_workspace(ns_dual, csr, len(d), speed_m_s, cap=dual.estimate_states(ns_dual, speed_m_s, max(s)))
    _, keep = _plan_tensors(ns_dual, source_indices, dev)
    q = centrality._make_query(d, b, s, speed_m_s, centrality.validate_tolerance(tolerance), compute_closeness,
                               compute_betweenness, True, *keep, angular_scaling_unit, farness_scaling_offset)
    out = torch.zeros((4, len(d), csr.n_bound), dtype=torch.float64, device=dev)
    reach = torch.zeros(len(d), dtype=torch.int32, device=dev)
    return Call(csr.struct(speed_m_s), q, ws.plan, ws, out, reach, torch.cuda.current_stream(dev).cuda_stream, keep)
