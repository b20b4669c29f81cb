"""The index math's division by a high multiply (nqes_internal.h FastDiv):
x / d = floor(x m / 2^32) with m = ceil(2^32 / d) is exact for x < 2^32 / d.
Checked here on the formula itself for every divisor the kernels use (row and
column counts up to 1024, rows per sample up to 10) over the index ranges
they pass (plus the largest x the bound allows)."""
import numpy as np


def magic(d):
    return 0 if d <= 1 else (2 ** 32 + d - 1) // d


def fdiv(x, d):
    m = magic(d)
    return x if d <= 1 else (x * m) >> 32


def test_fast_div_is_exact_below_its_bound():
    rng = np.random.default_rng(0)
    for d in list(range(1, 1025)) + [2145, 4097, 66176]:
        bound = (2 ** 32) // d
        xs = np.unique(np.concatenate([np.arange(0, min(bound, 12000)), rng.integers(0, bound, 500),
                                       [bound - 1]])).astype(object)
        for x in xs:
            assert fdiv(int(x), d) == int(x) // d, (x, d)


def test_fast_div_magic_fits_32_bits():
    for d in range(2, 5000):
        assert 0 < magic(d) < 2 ** 32
