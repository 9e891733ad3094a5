"""Known-answer checks of the uniform sources the oracle and the GPU share."""
import numpy as np

import oracle


def test_mt19937_matches_numpy_legacy_seeding(built):
    # cpp/3d/mt_rng.hpp:119-179 is mt19937ar; numpy's RandomState(int) seeds it the same way
    for seed in (0, 1, 5489, 12345, 2 ** 32 - 1):
        ref = np.random.RandomState(seed)._bit_generator.random_raw(2000).astype(np.uint32)
        np.testing.assert_array_equal(oracle.mt_words(seed, 2000), ref)


def test_mt_seed_truncates_to_32_bits(built):
    # Seed(unsigned long s) keeps s & 0xffffffff (cpp/3d/mt_rng.hpp:120)
    np.testing.assert_array_equal(oracle.mt_words(2 ** 32 + 7, 50), oracle.mt_words(7, 50))


def test_philox4x64_round_structure_matches_numpy(built):
    # numpy.random.Philox is Philox4x64-10; our 4x64 and 4x32 share one round structure
    for key in ([0, 0], [1, 2], [0xDEADBEEF, 0x12345678]):
        for ctr in ([0, 0, 0, 0], [5, 0, 0, 0], [2 ** 63, 7, 1, 9]):
            bg = np.random.Philox(key=np.array(key, np.uint64), counter=np.array(ctr, np.uint64))
            # numpy increments the counter before producing a block
            c = np.array(ctr, np.uint64)
            c[0] = c[0] + np.uint64(1)
            ours = oracle.philox4x64(c, key)
            np.testing.assert_array_equal(bg.random_raw(4).astype(np.uint64), ours)


def test_philox_stream_layout(built):
    # photon p of stream s with seed k: blocks counter = (p lo, p hi, block, s), key = (k lo, k hi)
    seed, stream, photon = 0x0123456789ABCDEF, 3, 2 ** 33 + 5
    w = oracle.philox_words(seed, stream, photon, 12)
    for b in range(3):
        blk = oracle.philox4x32([photon & 0xffffffff, photon >> 32, b, stream], [seed & 0xffffffff, seed >> 32])
        np.testing.assert_array_equal(w[4 * b: 4 * b + 4], blk)


def test_philox_uniformity(built):
    w = np.concatenate([oracle.philox_words(99, 0, p, 64) for p in range(2000)])
    u = w.astype(np.float64) / 2 ** 32
    hist, _ = np.histogram(u, bins=64, range=(0, 1))
    expected = len(u) / 64
    chi2 = ((hist - expected) ** 2 / expected).sum()
    assert chi2 < 120  # 63 dof: p ~ 1e-5 cut
    assert abs(u.mean() - 0.5) < 5e-3
    # distinct photons give distinct streams
    assert not np.array_equal(oracle.philox_words(99, 0, 1, 8), oracle.philox_words(99, 0, 2, 8))
    assert not np.array_equal(oracle.philox_words(99, 0, 1, 8), oracle.philox_words(99, 1, 1, 8))
