"""The multiply-shift division the kernels use for run-time divisors
(FastDiv in csrc/mmc_internal.h): n / d == (umulhi(m, n) + n) >> l with
l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, for 0 <= n < 2^31.
Checked here with exact integers for every divisor the lattices can produce
up to 4096 and for the extremes of n."""
import numpy as np


def magic(d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    assert 0 < m < (1 << 32) or d == 1
    return m & 0xFFFFFFFF, l


def fastdiv(n, d):
    m, l = magic(d)
    return (((m * n) >> 32) + n) >> l


def test_fastdiv_exact():
    rng = np.random.default_rng(1)
    ns = [0, 1, 2, 3, (1 << 31) - 1, (1 << 31) - 2, (1 << 30), 65535, 65536]
    ns += [int(v) for v in rng.integers(0, 1 << 31, size=300)]
    for d in list(range(1, 4097)) + [65537, 1 << 20, (1 << 31) - 1]:
        cases = ns + [k * d + r for k in (1, 7, 1000) for r in (0, d - 1) if k * d + r < (1 << 31)]
        for n in cases:
            assert fastdiv(n, d) == n // d, (n, d)
