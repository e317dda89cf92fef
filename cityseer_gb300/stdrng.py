"""The reference's source-sampling random stream: rand 0.10 `StdRng` (ChaCha with 12 rounds).

`prepare_source_sampling` (rust/src/centrality.rs:1082-1091) draws one `f32` per node index from
`StdRng::seed_from_u64(seed)`.  Restated here from the published algorithms of the crates pinned in
rust/Cargo.lock (rand 0.10.0, rand_core 0.10.0, chacha20 0.10.0), so that a seeded sampled run picks
the same sources as the reference:

* seed expansion (`SeedableRng::seed_from_u64`): a PCG32 (XSH-RR) generator, advanced before each
  output, fills the 32-byte seed 4 little-endian bytes at a time;
* the generator: the ChaCha block function (D. J. Bernstein) with 12 rounds, key = the seed, a 64-bit
  block counter from 0 in words 12-13 and stream 0 in words 14-15; the keystream is consumed as
  little-endian u32 words, block after block;
* `rng.random::<f32>()` (`StandardUniform`): the top 24 bits of one u32, times 2^-24.

The ChaCha block function is checked against the RFC 7539 section 2.3.2 test vector (20 rounds).
"""
from __future__ import annotations

import numpy as np

_CONST = np.array([0x61707865, 0x3320646E, 0x79622D32, 0x6B206574], dtype=np.uint32)
_PCG_MUL = 6364136223846793005
_PCG_INC = 11634580027462260723
_M64 = (1 << 64) - 1


def _rotl(x: np.ndarray, n: int) -> np.ndarray:
    return (x << np.uint32(n)) | (x >> np.uint32(32 - n))


def _quarter(s, a, b, c, d):
    s[a] += s[b]
    s[d] = _rotl(s[d] ^ s[a], 16)
    s[c] += s[d]
    s[b] = _rotl(s[b] ^ s[c], 12)
    s[a] += s[b]
    s[d] = _rotl(s[d] ^ s[a], 8)
    s[c] += s[d]
    s[b] = _rotl(s[b] ^ s[c], 7)


def chacha_blocks(state: np.ndarray, rounds: int) -> np.ndarray:
    """ChaCha block function over many input states at once: state [16, n] u32 -> output [16, n]."""
    x = state.copy()
    with np.errstate(over="ignore"):
        for _ in range(rounds // 2):
            _quarter(x, 0, 4, 8, 12)
            _quarter(x, 1, 5, 9, 13)
            _quarter(x, 2, 6, 10, 14)
            _quarter(x, 3, 7, 11, 15)
            _quarter(x, 0, 5, 10, 15)
            _quarter(x, 1, 6, 11, 12)
            _quarter(x, 2, 7, 8, 13)
            _quarter(x, 3, 4, 9, 14)
        return x + state


def pcg32_seed(state: int, n_bytes: int = 32) -> bytes:
    """rand_core's seed_from_u64 expansion: PCG32 (XSH-RR) words, little-endian."""
    state &= _M64
    out = bytearray()
    for _ in range(n_bytes // 4):
        state = (state * _PCG_MUL + _PCG_INC) & _M64
        xorshifted = (((state >> 18) ^ state) >> 27) & 0xFFFFFFFF
        rot = state >> 59
        x = ((xorshifted >> rot) | (xorshifted << ((32 - rot) & 31))) & 0xFFFFFFFF
        out += x.to_bytes(4, "little")
    return bytes(out)


class StdRng:
    """ChaCha12 keystream generator with rand's StdRng seeding and f32 conversion."""

    ROUNDS = 12

    def __init__(self, seed: bytes):
        if len(seed) != 32:
            raise ValueError("StdRng takes a 32-byte seed")
        self._key = np.frombuffer(seed, dtype="<u4").astype(np.uint32)
        self._block = 0  # next block counter
        self._buf = np.zeros(0, np.uint32)

    @classmethod
    def seed_from_u64(cls, seed: int) -> "StdRng":
        if seed < 0:
            raise OverflowError("can't convert negative int to unsigned")
        if seed > _M64:
            raise OverflowError("int too big to convert")
        return cls(pcg32_seed(int(seed)))

    def _blocks(self, n: int) -> np.ndarray:
        ctr = np.arange(self._block, self._block + n, dtype=np.uint64)
        st = np.empty((16, n), np.uint32)
        st[0:4] = _CONST[:, None]
        st[4:12] = self._key[:, None]
        st[12] = (ctr & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        st[13] = (ctr >> np.uint64(32)).astype(np.uint32)
        st[14] = 0
        st[15] = 0
        self._block += n
        return chacha_blocks(st, self.ROUNDS).T.reshape(-1)  # block after block, word after word

    def next_u32(self, n: int) -> np.ndarray:
        """The next n u32 outputs of the keystream."""
        need = n - len(self._buf)
        if need > 0:
            self._buf = np.concatenate([self._buf, self._blocks(-(-need // 16))])
        out, self._buf = self._buf[:n], self._buf[n:]
        return out

    def random_f32(self, n: int) -> np.ndarray:
        """n draws of rng.random::<f32>(): (u32 >> 8) * 2^-24, in [0, 1)."""
        return (self.next_u32(n) >> np.uint32(8)).astype(np.float32) * np.float32(1.0 / (1 << 24))
