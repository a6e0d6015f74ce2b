"""The engine's own draw generator (used when callers pass no draws): rand's
StdRng as the reference's QubitManager seeds it, StdRng::seed_from_u64(
KBW_SEED) (kbw src/quantum_execution.rs:181-191), each draw the
UniformFloat<f64> sample WeightedIndex consumes (src/convert.rs:60-64).

The ChaCha core is pinned to RFC 7539's known answers (20 rounds).  The
composition -- PCG32 seed expansion, 12 rounds, word order of next_u64 -- is
restated again here in plain Python from the published algorithms and the
engine must agree with it; against the rand crates themselves (absent here)
the stream is unpinned."""
import struct

import numpy as np
import pytest

from kbw_gb300 import _native as N

M32 = 0xFFFFFFFF
M64 = 0xFFFFFFFFFFFFFFFF


@pytest.fixture(scope="module")
def lib():
    return N.load()


def test_chacha20_rfc7539_block_vector(lib):
    # RFC 7539 section 2.3.2: key 00..1f, counter 1, nonce 00000009 0000004a 00000000
    key = [struct.unpack("<I", bytes(range(4 * i, 4 * i + 4)))[0] for i in range(8)]
    counter = 1 | (0x09000000 << 32)  # state words 12, 13
    stream = 0x4A000000  # state words 14, 15
    out = N.chacha_block(key, counter, stream, 20)
    want = [0xE4E7F110, 0x15593BD1, 0x1FDD0F50, 0xC47120A3, 0xC7F4D1C7, 0x0368C033, 0x9AAA2204, 0x4E6CD4C3,
            0x466482D2, 0x09AA9F07, 0x05D7C214, 0xA2028BD9, 0xD19C12B5, 0xB94E16DE, 0xE883D0CB, 0x4E3C50A2]
    assert out == want


def test_chacha20_rfc7539_zero_key_keystream(lib):
    # RFC 7539 appendix A.1, test vector 1: all-zero key and nonce, counter 0
    out = N.chacha_block([0] * 8, 0, 0, 20)
    ks = b"".join(struct.pack("<I", w) for w in out)
    assert ks[:16].hex() == "76b8e0ada0f13d90405d6ae55386bd28"


def _pcg32_seed(state):
    words = []
    for _ in range(8):
        state = (state * 6364136223846793005 + 11634580027462260723) & M64
        x = ((((state >> 18) ^ state) >> 27) & M32)
        rot = state >> 59
        words.append(((x >> rot) | (x << ((32 - rot) & 31))) & M32)
    return words


def _rotl(x, r):
    return ((x << r) | (x >> (32 - r))) & M32


def _block(key, counter, rounds):
    s = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574] + key + [counter & M32, counter >> 32, 0, 0]
    x = list(s)

    def qr(a, b, c, d):
        x[a] = (x[a] + x[b]) & M32; x[d] = _rotl(x[d] ^ x[a], 16)
        x[c] = (x[c] + x[d]) & M32; x[b] = _rotl(x[b] ^ x[c], 12)
        x[a] = (x[a] + x[b]) & M32; x[d] = _rotl(x[d] ^ x[a], 8)
        x[c] = (x[c] + x[d]) & M32; x[b] = _rotl(x[b] ^ x[c], 7)
    for _ in range(rounds // 2):
        qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
        qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
    return [(x[i] + s[i]) & M32 for i in range(16)]


def _stdrng_draws(seed, count):
    key = _pcg32_seed(seed)
    words, counter = [], 0
    out = []
    while len(out) < count:
        if len(words) < 2:
            words += _block(key, counter, 12)
            counter += 1
        lo, hi = words[0], words[1]
        del words[:2]
        u = (hi << 32) | lo
        out.append(struct.unpack("<d", struct.pack("<Q", (u >> 12) | 0x3FF0000000000000))[0] - 1.0)
    return out


@pytest.mark.parametrize("seed", [0, 1, 42, 2 ** 63 + 12345, M64])
def test_engine_draws_follow_stdrng(lib, seed):
    got = N.draws(seed, 70)  # crosses ChaCha block boundaries (8 draws per block)
    want = np.array(_stdrng_draws(seed, 70))
    assert np.array_equal(got, want)
    assert np.all((got >= 0.0) & (got < 1.0))


def test_draws_are_52_bit_uniformfloat_values(lib):
    d = N.draws(7, 1000)
    # every draw is k * 2^-52: the UniformFloat construction, not the 53-bit one
    k = d * 2.0 ** 52
    assert np.array_equal(k, np.floor(k))
    assert 0.4 < d.mean() < 0.6
