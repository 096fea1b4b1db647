"""Philox-4x32-10 known-answer tests.

The reference draws from one global mt19937 (Random.hh:10-12, Random.cc:3-4);
both GPU forms and the oracle's Philox mode use counter-based Philox-4x32-10
(Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
SC'11) instead. A mistake in its round constants or key schedule would pass
every replay test, because the oracle and the GPU would share it; so both are
held to the published known-answer vectors of the Random123 distribution
(kat_vectors, philox4x32 with 10 rounds), and the GPU's conversions of words
to uniforms are checked bit for bit against their definition.
"""
import numpy as np
import pytest

# (counter, key, output) of Random123's philox4x32_10 known-answer vectors
KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def philox_py(c, k):
    """Philox-4x32-10 as published: 10 rounds of the two 32x32->64 products
    with multipliers 0xD2511F53 and 0xCD9E8D57, key bumped by the Weyl
    constants 0x9E3779B9 and 0xBB67AE85 between rounds."""
    c = [int(x) for x in c]
    k0, k1 = int(k[0]), int(k[1])
    m = 0xFFFFFFFF
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & m, p1 & m, ((p0 >> 32) ^ c[3] ^ k1) & m, p0 & m]
        k0 = (k0 + 0x9E3779B9) & m
        k1 = (k1 + 0xBB67AE85) & m
    return c


def kat_arrays():
    c = np.array([v[0] for v in KAT], dtype=np.uint32)
    k = np.array([v[1] for v in KAT], dtype=np.uint32)
    o = np.array([v[2] for v in KAT], dtype=np.uint32)
    return c, k, o


def random_counters(n, seed=2024):
    r = np.random.default_rng(seed)
    return (r.integers(0, 2 ** 32, (n, 4), dtype=np.uint64).astype(np.uint32),
            r.integers(0, 2 ** 32, (n, 2), dtype=np.uint64).astype(np.uint32))


def uniform_f32(words):
    """UniformF32 by its definition: (w | 1) converted to float with rounding
    toward zero (keep the 24 leading significant bits), times 2^-32."""
    out = np.empty(words.shape, dtype=np.float32)
    flat = out.reshape(-1)
    for i, w in enumerate(words.reshape(-1)):
        v = int(w) | 1
        sh = max(0, v.bit_length() - 24)
        flat[i] = np.float32(((v >> sh) << sh) * 2.0 ** -32)   # exact in float32
    return out


def uniform_f64(words):
    """UniformF64 by its definition: the 53 high bits of (hi << 32 | lo), the
    lowest forced to 1, times 2^-53."""
    w = words.astype(np.uint64)
    out = np.empty((len(w), 2))
    for j in range(2):
        bits = (w[:, 2 * j + 1] << np.uint64(32)) | w[:, 2 * j]
        out[:, j] = ((bits >> np.uint64(11)) | np.uint64(1)).astype(np.float64) * 2.0 ** -53
    return out


def test_published_vectors_python():
    for c, k, o in KAT:
        assert philox_py(c, k) == list(o)


def test_oracle_philox_known_answers(orc):
    c, k, o = kat_arrays()
    np.testing.assert_array_equal(orc.philox(c, k), o)
    c, k = random_counters(512)
    got = orc.philox(c, k)
    for i in range(len(c)):
        assert list(got[i]) == philox_py(c[i], k[i])


@pytest.mark.gpu
def test_gpu_philox_known_answers(dpm, gpu_lib, orc):
    c, k, o = kat_arrays()
    w, _, _ = dpm.rng_eval(c, k)
    np.testing.assert_array_equal(w, o)
    c, k = random_counters(4096)
    w, f, d = dpm.rng_eval(c, k)
    np.testing.assert_array_equal(w, orc.philox(c, k))
    # the transport's uniforms, bit for bit, and strictly inside (0, 1)
    np.testing.assert_array_equal(f, uniform_f32(w))
    np.testing.assert_array_equal(d, uniform_f64(w))
    assert f.min() > 0.0 and f.max() < 1.0 and d.min() > 0.0 and d.max() < 1.0
