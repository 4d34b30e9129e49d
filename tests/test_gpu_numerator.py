"""The float64 step's integer numerator against IEEE arithmetic.

The float64 streamline step computes the numerator fma(2, 0.5 - f, f) of
time_to_next_pixel (src/lib.rs:168-179, a velocity component whose sign bit
is clear) with integer instructions for 0 <= f <= 1, keeping GB300's FP64
pipe for the arithmetic that needs it (rlic_check_numerators_f64 exposes it).
Its bits must equal the IEEE result, which numpy gives as
2 * (0.5 - f) + f (the product by 2 is exact, so the sum rounds once, as
the FMA does): random bit patterns over every exponent of [0, 1],
fractions drawn uniformly, operands built to sit on the rounding ties of
either rounding, powers of two and their neighbours, and values outside
[0, 1], which it must refuse.
"""

from __future__ import annotations

import numpy as np
import pytest

from rlic_gb300 import _native

pytestmark = pytest.mark.gpu

MANT = (1 << 52) - 1


def _run(f: np.ndarray):
    import torch

    tf = torch.from_numpy(np.ascontiguousarray(f, dtype=np.float64)).cuda()
    g = torch.empty_like(tf)
    ok = torch.empty(tf.shape, dtype=torch.int32, device="cuda")
    _native.check(_native.lib().rlic_check_numerators_f64(tf.data_ptr(), tf.numel(), g.data_ptr(),
                                                          ok.data_ptr(), None))
    torch.cuda.synchronize()
    return g.cpu().numpy(), ok.cpu().numpy().astype(bool)


def _want(f: np.ndarray) -> np.ndarray:
    return 2.0 * (0.5 - f) + f


def _from_bits(b: np.ndarray) -> np.ndarray:
    return np.asarray(b, dtype=np.uint64).view(np.float64)


def _assert_exact(f):
    g, ok = _run(f)
    assert ok.all()
    want = _want(f)
    bad = g.view(np.int64) != want.view(np.int64)
    assert not bad.any(), (f[bad][:5], g[bad][:5], want[bad][:5])


def test_random_bit_patterns_over_every_exponent() -> None:
    rng = np.random.default_rng(0)
    n = 4_000_000
    e = rng.integers(0, 1023, n, dtype=np.uint64)  # subnormals to [0.5, 1)
    m = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    _assert_exact(_from_bits((e << np.uint64(52)) | m))


def test_uniform_fractions() -> None:
    rng = np.random.default_rng(1)
    _assert_exact(rng.random(4_000_000))


def test_rounding_ties_of_both_roundings() -> None:
    """For f in [2^-55, 0.25) the step rounds twice: 0.5 - f to a multiple of
    2^-54, then the sum to a multiple of 2^-53; build f whose remainders sit
    exactly on half a unit of each, and one bit either side."""
    rng = np.random.default_rng(2)
    rows = []
    for E in range(968, 1022):
        s1 = 1021 - E
        for s in (s1, s1 + 1):
            if s == 0:
                continue
            m = (np.uint64(1) << np.uint64(52)) | rng.integers(0, 1 << 52, 4000, dtype=np.uint64)
            low = np.uint64((1 << s) - 1)
            tie = (m & ~low) | np.uint64(1 << (s - 1))
            for mm in (tie, tie + np.uint64(1), tie - np.uint64(1)):
                rows.append((np.uint64(E) << np.uint64(52)) | (mm & np.uint64(MANT)))
    _assert_exact(_from_bits(np.concatenate(rows)))


def test_powers_of_two_and_neighbours() -> None:
    p = np.ldexp(1.0, np.arange(-1074, 1))
    f = np.concatenate([[0.0], p, np.nextafter(p, 0.0), np.nextafter(p, 2.0)])
    f = f[(f >= 0.0) & (f <= 1.0)]
    _assert_exact(f)


def test_values_outside_zero_one_are_refused() -> None:
    f = np.array([-0.0, -1e-300, -0.5, np.nextafter(1.0, 2.0), 1.5, 2.0, np.inf, np.nan, -np.inf])
    g, ok = _run(f)
    assert not ok.any()
