"""Lane-by-lane model of the settle-order sort `warp_bucket_sort` (cityseer_gb300/csrc/cs_sort.cuh),
run on inputs the GPU parity graphs rarely produce: heavy exact ties, buckets of 33-64 keys (the
two-keys-per-lane branch) and buckets of more than 64 keys (the radix fallback).  The model follows
the kernel's steps with 32 lanes as numpy vectors (ballot, shuffle, match) and must equal a stable
sort by key; `dist_bucket` must be monotone in the key in f32 arithmetic."""
import numpy as np
import pytest

LANES = 32
F32 = np.float32


def dist_bucket(keys: np.ndarray, inv: np.float32) -> np.ndarray:
    d = keys.view(np.float32) if keys.dtype == np.uint32 else keys
    t = np.minimum((d * inv).astype(F32), F32(1.0))
    return np.minimum(511, ((t * t).astype(F32) * F32(512.0)).astype(F32).astype(np.int64))


def bucket_sort_model(keys: np.ndarray, dmax: float):
    """Returns (sorted keys, original positions, path taken)."""
    R = len(keys)
    vals = np.arange(R)
    inv = F32(1.0) / F32(dmax) if dmax > 0 else F32(0.0)
    b_all = dist_bucket(keys, inv)
    counts = np.bincount(b_all, minlength=512)
    if counts.max() > 64:
        o = np.argsort(keys, kind="stable")
        return keys[o], vals[o], "radix"
    start = np.concatenate([[0], np.cumsum(counts)[:-1]])
    kout = np.empty(R, np.uint32)
    vout = np.empty(R, np.int64)
    # stable scatter, 32 keys per step: rank among earlier lanes of the same bucket
    for base in range(0, R, LANES):
        kk, vv, bb = keys[base:base + LANES], vals[base:base + LANES], b_all[base:base + LANES]
        for lane in range(len(kk)):
            rank = int(np.sum(bb[:lane] == bb[lane]))
            kout[start[bb[lane]] + rank] = kk[lane]
            vout[start[bb[lane]] + rank] = vv[lane]
        for b in np.unique(bb):
            start[b] += int(np.sum(bb == b))
    end = start  # each bucket's counter now holds its end offset
    path = "runs"
    w0 = 0
    lane = np.arange(LANES)
    while w0 < R:
        i = w0 + lane
        ok = i < R
        k = np.where(ok, kout[np.minimum(i, R - 1)], np.uint32(0xFFFFFFFF))
        v = np.where(ok, vout[np.minimum(i, R - 1)], 0)
        bnext = int(dist_bucket(kout[w0 + 32:w0 + 33], inv)[0]) if w0 + 32 < R else (1 << 20)
        b = np.where(ok, dist_bucket(np.where(ok, k, np.uint32(0)), inv), 1 << 21)
        n = int(np.sum(b < bnext))
        assert np.all((b < bnext)[:n]) and not np.any((b < bnext)[n:]), "window is not a lane prefix"
        if n > 0:
            r = np.zeros(LANES, np.int64)
            for j in range(n):
                a = k[j]
                r += (a < k) | ((a == k) & (j < lane))
            kout[w0 + r[:n]] = k[:n]
            vout[w0 + r[:n]] = v[:n]
            w0 += n
        else:
            path = "runs+pairs"
            e = int(end[b[0]])
            assert 33 <= e - w0 <= 64
            i1 = i + 32
            k1 = np.where(i1 < e, kout[np.minimum(i1, R - 1)], np.uint32(0xFFFFFFFF))
            v1 = np.where(i1 < e, vout[np.minimum(i1, R - 1)], 0)
            r0 = np.zeros(LANES, np.int64)
            r1 = np.zeros(LANES, np.int64)
            for j in range(32):
                a = k[j]
                r0 += (a < k) | ((a == k) & (j < lane))
                r1 += a <= k1
            for j in range(e - w0 - 32):
                a = k1[j]
                r0 += a < k
                r1 += (a < k1) | ((a == k1) & (j < lane))
            kout[w0 + r0] = k
            vout[w0 + r0] = v
            m = i1 < e
            kout[w0 + r1[m]] = k1[m]
            vout[w0 + r1[m]] = v1[m]
            w0 = e
    return kout, vout, path


def _case(dists):
    keys = np.asarray(dists, np.float32).view(np.uint32)
    dmax = float(np.max(dists)) if len(dists) else 0.0
    got_k, got_v, path = bucket_sort_model(keys, dmax * 1.01)
    o = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(got_k, keys[o])
    np.testing.assert_array_equal(got_v, o)
    return path


def test_disk_like_reach_uses_runs():
    rng = np.random.default_rng(0)
    d = np.sqrt(rng.random(8000)) * 3750.0  # a search disk: reach grows with the square of distance
    d[0] = 0.0
    assert _case(d) == "runs"


def test_ties_and_buckets_of_33_to_64_keys():
    rng = np.random.default_rng(1)
    for n_tied in (33, 40, 63, 64):
        d = np.concatenate([[0.0], np.sqrt(rng.random(500)) * 3000.0, np.full(n_tied, 1234.5)])
        rng.shuffle(d)
        assert _case(d) == "runs+pairs"
        # near-ties inside one bucket, not exact
        d2 = np.concatenate([[0.0], 1234.5 + rng.random(n_tied) * 1e-3, rng.random(200) * 3000.0])
        assert _case(d2) in ("runs", "runs+pairs")


def test_overfull_bucket_falls_back():
    d = np.concatenate([[0.0], np.full(65, 700.0), np.linspace(1, 3000, 300)])
    assert _case(d) == "radix"


@pytest.mark.parametrize("dmax", [1.0, 122.0, 3750.0, 1e6])
def test_bucket_is_monotone_in_the_key(dmax):
    inv = F32(1.0) / F32(dmax)
    lo, hi = np.float32(0.0).view(np.uint32), np.float32(dmax).view(np.uint32)
    keys = np.unique(np.linspace(int(lo), int(hi), 2_000_000).astype(np.uint32))
    b = dist_bucket(keys, inv)
    assert np.all(np.diff(b) >= 0) and b[0] == 0 and b[-1] <= 511
