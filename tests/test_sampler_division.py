"""The batched sampler's digit division (planner_device.cuh, DivTable):
floor(i / b) = (i * m31[b]) >> (31 + ceil(log2 b)) for every i < 2^31 and
every divisor 2..64.

With m * b = 2^(31 + l) + e, i = q b + r: i m / 2^(31 + l) = i / b +
i e / (b 2^(31 + l)), whose floor is q as long as r + i e / 2^(31 + l) < b,
i.e. for every i < 2^31 when 0 <= e and (2^31 - 1) e < 2^(31 + l).  That
condition is checked for every divisor, and the formula numerically on the
indices where the error term is largest (the top 2^20 below 2^31), the
first 2^16 and a random sample."""
import numpy as np


def magic31(b: int):
    ell = (b - 1).bit_length()
    return ((1 << (31 + ell)) + b - 1) // b, ell - 1


def q31(i: np.ndarray, m: int, s: int) -> np.ndarray:
    return ((i * np.uint64(m)) >> np.uint64(32)) >> np.uint64(s)   # umulhi, then the shift


def test_magic_fits_32_bits_and_is_exact():
    for b in range(2, 65):
        m, s = magic31(b)
        ell = s + 1
        assert 0 < m < 1 << 32 and 0 <= s <= 5
        e = m * b - (1 << (31 + ell))
        assert 0 <= e < b and ((1 << 31) - 1) * e < 1 << (31 + ell)


def test_division_numeric():
    top = 1 << 31
    rng = np.random.default_rng(0)
    idx = np.concatenate([np.arange(top - (1 << 20), top, dtype=np.uint64), np.arange(1 << 16, dtype=np.uint64),
                          rng.integers(0, top, 1 << 20, dtype=np.uint64)])
    for b in range(2, 65):
        m, s = magic31(b)
        np.testing.assert_array_equal(q31(idx, m, s), idx // np.uint64(b))
