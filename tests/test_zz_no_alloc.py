"""The allocation-free entry point, cs_centrality_shortest_noalloc, called through the C-ABI.

It serves callers that cannot allocate device memory when they call (their host application owns
every allocation through its own pool, or the call must not block or fail on an allocation): its
scratch is a static device array reserved when the library loads.  This file is collected last so
that a failure here cannot hide the other tests; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from cityseer_gb300 import _native, centrality, common, synth

ROWS = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
        "node_betweenness_beta")


def _lib():
    lib = _native.load()
    fn = lib.cs_centrality_shortest_noalloc
    fn.restype = C.c_int32
    fn.argtypes = [C.POINTER(_native.PrimalGraph), C.POINTER(_native.Query), _native.Outputs, C.c_void_p]
    return lib


def _call_noalloc(lib, g, q, k, nb, dev):
    out = torch.zeros((7, k, nb), dtype=torch.float64, device=dev)
    reach = torch.zeros(k, dtype=torch.int32, device=dev)
    rc = lib.cs_centrality_shortest_noalloc(C.byref(g), C.byref(q), _native.Outputs(out.data_ptr(), reach.data_ptr()),
                                            torch.cuda.current_stream().cuda_stream)
    _native.check(rc, "cs_centrality_shortest_noalloc")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _case(side, dists, closeness=True):
    """A lattice, its query for every source, and the existing entry point's result rows."""
    p, _ = synth.lattice_config("c1", side=side)
    ns = synth.primal_structure(p)
    want = ns.centrality_shortest(distances=dists, compute_closeness=closeness)  # caller-owned workspace
    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    csr = centrality._primal_csr(ns)
    dev = csr.device
    sp = centrality.prepare_source_sampling(ns, None, None, None, None)
    keep = (torch.from_numpy(sp.process).to(dev), torch.from_numpy(sp.src_wt).to(dev),
            torch.from_numpy(sp.eligible).to(dev))
    q = centrality._make_query(d, b, s, 1.33333, float(centrality.TIE_EPSILON), closeness, True, False, *keep)
    return dict(ns=ns, want=want, d=d, csr=csr, q=q, g=csr.struct(1.33333), keep=keep, closeness=closeness)


def _check(lib, c, label):
    got = _call_noalloc(lib, c["g"], c["q"], len(c["d"]), c["csr"].n_bound, c["csr"].device)
    idx = np.asarray(c["ns"].node_indices())
    for m, name in enumerate(ROWS):
        if m < 5 and not c["closeness"]:
            assert not got[m].any(), f"{label}: closeness row {name} written with closeness off"
            continue
        ref = getattr(c["want"], name)
        for i, dist in enumerate(c["d"]):
            if name in ("node_density", "node_cycles"):
                np.testing.assert_array_equal(got[m, i][idx], ref[dist], err_msg=f"{label} {name}[{dist}]")
            else:
                rtol = 1e-6 if name == "node_betweenness" else 1e-5
                np.testing.assert_allclose(got[m, i][idx], ref[dist], rtol=rtol, atol=1e-9,
                                           err_msg=f"{label} {name}[{dist}]")


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point_twice():
    lib = _lib()
    a = _case(24, [500, 1000, 2000])
    for call in range(2):  # the static scratch keeps the previous call's contents
        _check(lib, a, f"call {call}")


@pytest.mark.gpu
def test_noalloc_graphs_of_other_sizes_in_turn():
    """Each call places its header, closeness bucket, dense state and per-source arrays at offsets
    set by its own node bound and threshold count, over bytes the previous call used for something
    else: A (24x24, 3 thresholds), B (16x16, 4 thresholds), B without closeness, then A again, and
    a 40x40 graph whose searches fill the array with fewer slots than the GPU could run."""
    lib = _lib()
    a = _case(24, [500, 1000, 2000])
    b = _case(16, [300, 600, 900, 1500])
    b_nc = _case(16, [400], closeness=False)
    big = _case(40, [500, 1000, 2000, 5000])
    for label, c in (("A", a), ("B", b), ("B without closeness", b_nc), ("A again", a), ("40x40", big),
                     ("A after 40x40", a)):
        _check(lib, c, label)


@pytest.mark.gpu
def test_noalloc_call_after_a_rejected_call():
    lib = _lib()
    a = _case(24, [500, 1000, 2000])
    _check(lib, a, "before")
    g = _native.PrimalGraph()
    g.n_bound = 10_000_000
    g.max_out_degree = 4
    rc = lib.cs_centrality_shortest_noalloc(C.byref(g), C.byref(a["q"]), _native.Outputs(None, None), None)
    assert rc == _native.CS_ERR_ARG
    _check(lib, a, "after the rejected call")


@pytest.mark.gpu
def test_noalloc_rejects_graphs_beyond_the_static_scratch():
    lib = _lib()
    g = _native.PrimalGraph()
    g.n_bound = 10_000_000  # one search would need far more than the 64 MiB array
    g.max_out_degree = 4
    q = _native.Query()
    q.k = 1
    rc = lib.cs_centrality_shortest_noalloc(C.byref(g), C.byref(q), _native.Outputs(None, None), None)
    assert rc == _native.CS_ERR_ARG
    assert "too large for the allocation-free path" in _native.last_error()
