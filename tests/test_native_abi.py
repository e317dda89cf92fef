"""libcsgpu.so: loads without a GPU, exports every symbol include/*.h declares, and its host-side
f32 arithmetic (thresholds, edge travel seconds) matches the oracle bit for bit."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from cityseer_gb300 import _native, common, synth

HEADER = Path(__file__).resolve().parents[1] / "include" / "cityseer_gb300.h"


def declared_functions():
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cs_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = _native.load()
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    # every declared function has a ctypes signature in the binding (except test-only lookups)
    missing = [n for n in names if n not in _native.SIGNATURES]
    assert missing == [], missing


def test_thresholds_match_oracle_bitwise():
    rng = np.random.default_rng(0)
    for _ in range(50):
        k = int(rng.integers(1, 8))
        dists = np.sort(rng.choice(np.arange(1, 20000), size=k, replace=False)).tolist()
        speed = float(np.float32(rng.uniform(0.5, 3.0)))
        d, b, s = common.pair_distances_betas_time(speed, distances=dists)
        assert d == dists
        np.testing.assert_array_equal(np.float32(b), oracle.betas_from_distances(dists))
        np.testing.assert_array_equal(np.uint32(s), oracle.seconds_from_distances(dists, speed))
        if all(b[i + 1] < b[i] for i in range(len(b) - 1)):  # 5-dp rounding can merge close distances
            d2 = common.distances_from_betas(b)
            np.testing.assert_array_equal(np.uint32(d2), oracle.distances_from_betas(b))


def test_threshold_known_values():
    d, b, s = common.pair_distances_betas_time(1.33333, distances=[500, 1000, 2000, 5000])
    assert s == [375, 750, 1500, 3750]
    assert [round(x, 5) for x in b] == [0.008, 0.004, 0.002, 0.0008]
    _, b2, _ = common.pair_distances_betas_time(1.33333, distances=[4800])
    assert np.float32(b2[0]) == np.float32(0.00083)
    d3, _, s3 = common.pair_distances_betas_time(1.33333, minutes=[5, 10])
    assert s3 == [300, 600] and d3 == [400, 800]


@pytest.mark.parametrize("kw,msg", [
    (dict(distances=[100, 50]), "strictly increasing"),
    (dict(distances=[0, 50]), "positive integers"),
    (dict(betas=[0.01, 0.02]), "strictly decreasing"),
    (dict(betas=[-0.01]), "greater than zero"),
    (dict(), "exactly one"),
    (dict(distances=[100], betas=[0.04]), "exactly one"),
])
def test_threshold_errors(kw, msg):
    with pytest.raises(ValueError, match=msg):
        common.pair_distances_betas_time(1.33333, **kw)


def test_edge_seconds_match_oracle_with_slopes():
    p, _ = synth.lattice_config("c1", side=8)
    ns = synth.primal_structure(p)
    a = ns.arrays()
    rng = np.random.default_rng(3)
    a["z"][:] = rng.uniform(0, 30, len(a["z"]))
    a["has_z"][:] = 1
    a["has_z"][::5] = 0
    a["e_imp"][:] = rng.uniform(0.5, 2.0, len(a["e_imp"])).astype(np.float32)
    from cityseer_gb300 import device

    og = oracle.OracleGraph(ns)
    for use_imp in (True, False):
        got = device.edge_seconds(a, 1.33333, use_imp)
        want = np.array([oracle.lib().og_edge_travel_seconds(og.h, e, C.c_float(1.33333), int(use_imp))
                         for e in range(len(got))], np.float32)
        np.testing.assert_array_equal(got, want)


def test_gpu_entry_points_fail_cleanly_without_device():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _native.load()
    plan = _native.Plan()
    g = _native.PrimalGraph()
    g.n_bound = 10
    g.max_out_degree = 4
    rc = lib.cs_plan_primal(C.byref(g), 0, 1, 0, 0, 0, C.byref(plan))
    assert rc == _native.CS_ERR_CUDA
    assert _native.last_error()
