"""Philox4x32-10 (Salmon et al., SC'11) known-answer vectors from the Random123 distribution,
checked against the host restatement that the GPU tests use to rebuild the engine's
test matrices."""
import numpy as np

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85


def philox(ctr, key):
    x, y, z, w = [np.uint64(c) for c in ctr]
    k0, k1 = key
    for _ in range(10):
        p0 = x * np.uint64(M0)
        p1 = z * np.uint64(M1)
        x, y, z, w = ((p1 >> np.uint64(32)) ^ y ^ np.uint64(k0), p1 & np.uint64(0xFFFFFFFF),
                      (p0 >> np.uint64(32)) ^ w ^ np.uint64(k1), p0 & np.uint64(0xFFFFFFFF))
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return [int(v) for v in (x, y, z, w)]


def test_philox4x32_10_known_answers():
    assert philox((0, 0, 0, 0), (0, 0)) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    f = 0xFFFFFFFF
    assert philox((f, f, f, f), (f, f)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]


def test_batch_test_generator_uses_the_same_rounds():
    from test_gpu_batch import philox_gaussians
    v = philox_gaussians(8, 0, 0)
    assert v.shape == (8,) and np.all(np.isfinite(v))
