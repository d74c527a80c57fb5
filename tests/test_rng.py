"""Counter-based RNG contract shared by the kernels and the oracle."""
import numpy as np

import oracle

# Known-answer vectors of Philox4x32-10 published with the algorithm
# (Salmon et al., SC'11; Random123 kat_vectors).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers():
    for ctr, key, want in KAT:
        assert tuple(int(x) for x in oracle.philox(ctr, key)) == want


def test_bounce_words_layout():
    seed = 0x0123456789ABCDEF
    w = oracle.bounce_words(seed, 7, 1234, 56, 3)
    for call in range(3):
        blk = oracle.philox((1234, 56, 3 * 4 + call, 7), (seed & 0xFFFFFFFF, seed >> 32))
        assert np.array_equal(w[4 * call:4 * call + 4], blk)


def test_uniform_conversions_edges():
    words = np.array([0, 0xFFFFFFFF, 0x80000000, 0x100, 0xFF], np.uint32)
    u01, upm1 = oracle.uniforms(words)
    # rand 0.8.5 Standard f32: (u >> 8) * 2^-24, in [0, 1)
    assert u01.tolist() == [0.0, np.float32(1 - 2 ** -24), 0.5, np.float32(2 ** -24), 0.0]
    # gen_range(-1.0..=1.0): both ends reachable
    assert upm1[0] == -1.0 and upm1[1] == 1.0
    assert upm1[4] == -1.0


def test_uniform_distributions():
    rng = np.random.default_rng(0)
    words = rng.integers(0, 2 ** 32, 1 << 20, dtype=np.uint64).astype(np.uint32)
    u01, upm1 = oracle.uniforms(words)
    assert 0.0 <= u01.min() and u01.max() < 1.0
    assert -1.0 <= upm1.min() and upm1.max() <= 1.0
    assert abs(u01.mean() - 0.5) < 2e-3 and abs(upm1.mean()) < 4e-3
    assert abs(u01.var() - 1 / 12) < 2e-3


def test_philox_stream_statistics():
    # Consecutive counters give uncorrelated, uniform words.
    ws = np.array([oracle.bounce_words(1, 0, p, 0, 0) for p in range(4096)], np.uint32).ravel()
    u01, _ = oracle.uniforms(ws)
    hist, _ = np.histogram(u01, bins=16, range=(0, 1))
    expected = len(u01) / 16
    chi2 = ((hist - expected) ** 2 / expected).sum()
    assert chi2 < 40  # 15 dof, p ~ 5e-4
    assert abs(np.corrcoef(u01[:-1], u01[1:])[0, 1]) < 0.02
