"""Accessibility on the GPU (DataMap.accessibility with angular = False, rust/src/data.rs:605-740):
the data map's tables go to the device once per call and cs_accessibility runs one search per live
source, summing its reachable entries per land-use class and threshold."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native, centrality


def accessibility_rows(ns, t: dict, sources, d, b, s, mcw, speed: float, n_classes: int):
    """Per class: unweighted and weighted rows [n_classes][K][n_bound] (f64) and the nearest
    distance within the largest threshold [n_classes][n_bound] (NaN when none), for `sources`."""
    nb = ns.node_bound()
    K = len(d)
    u = np.zeros((n_classes, K, nb))
    w = np.zeros((n_classes, K, nb))
    n = np.full((n_classes, nb), np.nan)
    if n_classes == 0 or len(sources) == 0:
        return u, w, n
    csr = centrality._primal_csr(ns)
    dev = csr.device
    ws = centrality._workspace(ns, csr, 0, 1, speed, int(max(s)))

    def i32(x):
        return torch.from_numpy(np.ascontiguousarray(x, np.int32)).to(dev)

    keep = {
        "node_ptr": i32(t["ptr"]), "assign_entry": i32(t["a_entry"]),
        "assign_dist": torch.from_numpy(np.ascontiguousarray(t["a_dist"], np.float32)).to(dev),
        "assign_node": i32(t["a_node"]), "assign_rank": i32(t["a_rank"]), "entry_group": i32(t["entry_group"]),
        "entry_class": i32(t["entry_class"]), "group_ptr": i32(t["g_ptr"]), "group_assign": i32(t["g_assign"]),
    }
    dm = _native.DataMapArrays()
    dm.n_entries = len(t["keys"])
    dm.n_assign = len(t["a_entry"])
    dm.n_groups = int(t["n_groups"])
    for name, tensor in keep.items():
        setattr(dm, name, tensor.data_ptr() if tensor.numel() else None)
    src_t = torch.from_numpy(np.ascontiguousarray(sources, np.int32)).to(dev)
    zf = torch.zeros(nb, dtype=torch.float32, device=dev)
    zu = torch.zeros(nb, dtype=torch.uint8, device=dev)
    q = centrality._make_query(d, b, s, speed, float(centrality.TIE_EPSILON), False, False, False, src_t, zf, zu)
    unw = torch.zeros((n_classes, K, nb), dtype=torch.float64, device=dev)
    wt = torch.zeros((n_classes, K, nb), dtype=torch.float64, device=dev)
    near = torch.full((n_classes, nb), float("inf"), dtype=torch.float32, device=dev)
    mcw_arr = (C.c_float * K)(*[float(x) for x in mcw])
    lib = _native.load()
    rc = lib.cs_accessibility(C.byref(csr.struct(speed)), C.byref(dm), C.byref(q), mcw_arr, int(n_classes),
                              C.byref(ws.plan), ws.ptr, ws.nbytes, unw.data_ptr(), wt.data_ptr(), near.data_ptr(),
                              centrality._stream_ptr())
    if rc != _native.CS_OK:
        ws.init(centrality._stream_ptr())
    _native.check(rc, "cs_accessibility")
    near_h = near.cpu().numpy().astype(np.float64)
    near_h[np.isinf(near_h)] = np.nan
    return unw.cpu().numpy(), wt.cpu().numpy(), near_h
