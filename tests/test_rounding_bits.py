"""The stochastic-rounding bits of the BF16 write-backs (host copy of the kernels' sr_bits4,
no device): the restated formula, and each 16-bit field uniform over [0, 2^16) so the
rounding is unbiased."""
import numpy as np

import sgns

M32 = (1 << 32) - 1


def fmix32(h):
    h ^= h >> 16
    h = (h * 0x7FEB352D) & M32
    h ^= h >> 15
    h = (h * 0x846CA68B) & M32
    return h ^ (h >> 16)


def sr_bits4_py(ev, row, col4):
    h = fmix32((ev & M32) ^ ((row * 0x9E3779B1 + col4 * 0x85EBCA77) & M32))
    t = ((h ^ (ev >> 32)) * 0x9E3779B1) & M32
    return ((t ^ (t >> 16)) << 32) | h


def test_library_bits_follow_the_formula(sgns_lib):
    rng = np.random.default_rng(1)
    ev = rng.integers(0, 2**63, 2000, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, 2000, dtype=np.uint64)
    row = rng.integers(0, 2**32, 2000, dtype=np.uint64).astype(np.uint32)
    col4 = rng.integers(0, 64, 2000).astype(np.uint32)
    got = sgns.sr_bits4(ev, row, col4)
    want = [sr_bits4_py(int(a), int(b), int(c)) for a, b, c in zip(ev, row, col4)]
    assert [int(x) for x in got] == want


def test_fields_are_uniform_and_independent(sgns_lib):
    rng = np.random.default_rng(2)
    n = 1 << 20
    # one event key per 256 (row, chunk) draws, rows and chunks as a write-back sees them
    ev = np.repeat(rng.integers(0, 2**63, n // 256, dtype=np.uint64), 256)
    row = rng.integers(0, 2_500_000, n).astype(np.uint32)
    col4 = rng.integers(0, 32, n).astype(np.uint32)
    bits = sgns.sr_bits4(ev, row, col4)
    fields = [((bits >> np.uint64(16 * j)) & np.uint64(0xFFFF)).astype(np.float64) for j in range(4)]
    for f in fields:
        # mean of a uniform 16-bit field: 32767.5, standard error 18918 / sqrt(n) = 18.5
        assert abs(f.mean() - 32767.5) < 6 * 18.5, f.mean()
        assert f.max() >= 65500 and f.min() <= 35
        counts = np.bincount((f.astype(np.int64) >> 8), minlength=256)
        chi2 = (((counts - n / 256) ** 2) / (n / 256)).sum()
        assert chi2 < 400, chi2  # 255 degrees of freedom: 255 +- 23
    for a in range(4):
        for b in range(a + 1, 4):
            r = np.corrcoef(fields[a], fields[b])[0, 1]
            assert abs(r) < 0.01, (a, b, r)
