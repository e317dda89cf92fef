"""The sampling random stream (rust/src/centrality.rs:1082-1091): rand 0.10 StdRng restated.

Pinned two ways: the ChaCha block function against RFC 7539 section 2.3.2 (20 rounds), and the
12-round generator with its key / counter / stream layout and u32 consumption order against the
value-stability targets of rand's own StdRng test (`test_stdrng_construction`, src/rngs/std.rs of the
rand crate: a fixed 32-byte seed; next_u64, then next_u64 of a StdRng seeded from the first)."""
import numpy as np
import pytest

from cityseer_gb300.centrality import prepare_source_sampling
from cityseer_gb300.stdrng import _CONST, StdRng, chacha_blocks, pcg32_seed
from helpers import mock_graph, structure


def test_chacha_block_rfc7539():
    st = np.zeros((16, 1), np.uint32)
    st[0:4, 0] = _CONST
    st[4:12, 0] = np.frombuffer(bytes(range(32)), "<u4")
    st[12, 0] = 1
    st[13:16, 0] = np.frombuffer(bytes.fromhex("000000090000004a00000000"), "<u4")
    out = chacha_blocks(st, 20)[:, 0].astype("<u4").tobytes().hex()
    assert out == ("10f1e7e4d13b5915500fdd1fa32071c4c7d1f4c733c068030422aa9ac3d46c4e"
                   "d2826446079faa0914c2d705d98b02a2b5129cd1de164eb9cbd083e8a2503c4e")


def _u64(rng):
    w = rng.next_u32(2)
    return int(w[0]) | (int(w[1]) << 32)


def test_stdrng_value_stability():
    seed = bytes([1, 0, 0, 0, 23, 0, 0, 0, 200, 1, 0, 0, 210, 30, 0, 0] + [0] * 16)
    rng0 = StdRng(seed)
    x0 = _u64(rng0)
    rng1 = StdRng(rng0.next_u32(8).astype("<u4").tobytes())  # StdRng::from_rng(&mut rng0)
    assert [x0, _u64(rng1)] == [10719222850664546238, 14064965282130556830]


def test_stream_is_independent_of_chunking():
    a = StdRng.seed_from_u64(42).next_u32(1000)
    r = StdRng.seed_from_u64(42)
    b = np.concatenate([r.next_u32(n) for n in (1, 15, 16, 17, 100, 851)])
    np.testing.assert_array_equal(a, b)


def test_seed_expansion_and_f32_draws():
    assert len(pcg32_seed(0)) == 32 and pcg32_seed(7) != pcg32_seed(8)
    x = StdRng.seed_from_u64(3).random_f32(100000)
    assert x.dtype == np.float32 and x.min() >= 0.0 and x.max() < 1.0
    assert abs(float(x.mean()) - 0.5) < 0.01
    # 24-bit draws: every value is a multiple of 2^-24
    assert np.all((x * np.float32(1 << 24)) == np.floor(x * np.float32(1 << 24)))
    with pytest.raises(OverflowError):
        StdRng.seed_from_u64(-1)


def test_seeded_sampling_plan_is_reproducible():
    _, _, ns = structure(mock_graph())
    a = prepare_source_sampling(ns, 0.5, None, 11, None)
    b = prepare_source_sampling(ns, 0.5, None, 11, None)
    c = prepare_source_sampling(ns, 0.5, None, 12, None)
    assert a.process.tolist() == b.process.tolist()
    assert a.process.tolist() != c.process.tolist()
    # the plan keeps exactly the nodes whose draw is below p (one draw per node index)
    draws = StdRng.seed_from_u64(11).random_f32(ns.node_bound())
    live = ns.arrays()["live"][: ns.node_bound()] == 1
    want = [i for i in ns.node_indices() if live[i] and draws[i] < np.float32(0.5)]
    assert a.process.tolist() == want
