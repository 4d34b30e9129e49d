"""The derivation behind the float64 step's integer numerator, on the CPU.

The float64 streamline step computes fma(2, RN(0.5 - f), f) (the numerator
of time_to_next_pixel, src/lib.rs:168-179, for a velocity component whose
sign bit is clear) with integer instructions (numerator_two_int in
rlic_gb300/csrc/lic_device.cuh; tests/test_gpu_numerator.py checks that
code against IEEE arithmetic on the GPU).  This test restates the same
integer steps in numpy and checks them against IEEE float64 arithmetic,
where 2 * (0.5 - f) + f rounds exactly like the FMA (the product by 2 is
exact): every exponent from the subnormals to [0.5, 1), and operands on the
rounding ties of both roundings.
"""

from __future__ import annotations

import numpy as np

MANT = np.uint64((1 << 52) - 1)
ONE = np.uint64(0x3FF0000000000000)
U = np.uint64


def _model(b: np.ndarray) -> np.ndarray:
    """The integer restatement, vectorised: bit patterns of f in [0, 1] ->
    bit patterns of fma(2, RN(0.5 - f), f)."""
    E = (b >> U(52)).astype(np.int64)
    m = (b & MANT) | U(1 << 52)
    # f in [0.5, 1): 1 - f exactly, normalised by its leading zeros
    r1 = U(1 << 53) - m
    # leading zeros of the 64-bit r1 (exact: r1 < 2^53 converts to float64 exactly)
    lz = 64 - np.frexp(np.maximum(r1, U(1)).astype(np.float64))[1].astype(np.int64)
    sh = np.maximum(lz - 11, 0).astype(np.uint64)
    g_half = (((1033 - lz) & 0x7FF).astype(np.uint64) << U(52)) | ((r1 << sh) & MANT)
    # f in [2^-55, 0.5): both roundings on the significand
    s1 = np.clip(1021 - E, 0, 53).astype(np.uint64)
    K = m >> s1
    lo1 = m & ((U(1) << s1) - U(1))
    h1 = (U(1) << s1) >> U(1)
    c1 = ((s1 > 0) & ((lo1 > h1) | ((lo1 == h1) & ((K & U(1)) == 1)))).astype(np.uint64)
    G0 = U(1 << 53) - ((K + U(1)) >> U(1)) - c1
    c2 = (((K & U(1)) == 1) & ((lo1 != 0) | ((G0 & U(1)) == 1))).astype(np.uint64)
    G = G0 + c2
    g_low = np.where(G >= U(1 << 53), ONE, (U(1022) << U(52)) | (G & MANT))
    r = np.where(E < 968, ONE, np.where(E <= 1021, g_low, g_half))
    return np.where(b == ONE, U(0), r)


def _check(f: np.ndarray) -> None:
    f = f[(f >= 0.0) & (f <= 1.0) & ~np.signbit(f)]
    want = (2.0 * (0.5 - f) + f).view(np.uint64)
    got = _model(f.view(np.uint64))
    bad = got != want
    assert not bad.any(), (f[bad][:5], got[bad][:5], want[bad][:5])


def test_every_exponent_random_bit_patterns() -> None:
    rng = np.random.default_rng(0)
    e = rng.integers(0, 1023, 2_000_000, dtype=np.uint64)
    m = rng.integers(0, 1 << 52, 2_000_000, dtype=np.uint64)
    _check(((e << U(52)) | m).view(np.float64))


def test_uniform_fractions_and_powers_of_two() -> None:
    rng = np.random.default_rng(1)
    p = np.ldexp(1.0, np.arange(-1074, 1))
    _check(np.concatenate([rng.random(1_000_000), [0.0, 1.0], p, np.nextafter(p, 0.0),
                           np.nextafter(p, 2.0)]))


def test_rounding_ties_of_both_roundings() -> None:
    rng = np.random.default_rng(2)
    rows = []
    for E in range(968, 1022):
        s1 = 1021 - E
        for s in (s1, s1 + 1):
            if s == 0:
                continue
            m = U(1 << 52) | rng.integers(0, 1 << 52, 2000, dtype=np.uint64)
            low = U((1 << s) - 1)
            tie = (m & ~low) | U(1 << (s - 1))
            for mm in (tie, tie + U(1), tie - U(1)):
                rows.append((U(E) << U(52)) | (mm & MANT))
    _check(np.concatenate(rows).view(np.float64))
