"""Pure-Python restatement of rLIC's convolution, for tiny images only.

TEST INFRASTRUCTURE ONLY.  A second, independent restatement of the
reference's native core (neutrinoceros/rlic src/lib.rs:157-443) used to
cross-check the C oracle (lic_oracle.c) on small cases: scalar numpy
arithmetic in the input dtype, with ``mul_add`` evaluated exactly on
rationals and rounded once (Python 3.12 has no math.fma).  ``variant``
selects the reference's Cargo feature set as the C oracle does: bit 0 =
``fma`` (``mul_add`` fused; otherwise a rounded product, then a rounded
sum), bit 1 = ``branchless`` (src/lib.rs:157-180); 3, both on, is the
reference's default build.
"""

from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

VARIANT_FMA = 1
VARIANT_BRANCHLESS = 2
DEFAULT_VARIANT = VARIANT_FMA | VARIANT_BRANCHLESS


def _round_fraction(x: Fraction, dtype) -> float:
    """Round an exact rational to the nearest float of `dtype` (ties to even)."""
    if x == 0:
        return dtype(0.0)
    if dtype is np.float64:
        try:
            return np.float64(x.numerator / x.denominator)  # int/int rounds correctly
        except OverflowError:
            return np.float64(math.copysign(math.inf, x))
    # float32: 24-bit significand, exponent range [-126, 127], subnormal quantum 2^-149
    sign = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    e = max(e, -126)
    quantum = Fraction(2) ** (e - 23)
    q = a / quantum
    n = q.numerator // q.denominator
    rem = q - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n % 2 == 1):
        n += 1
    val = n * quantum
    if val >= Fraction(2) ** 128:
        return np.float32(sign * math.inf)
    return np.float32(sign * float(val))


def fma(a, b, c, dtype):
    """Single-rounding a*b + c in `dtype`."""
    a, b, c = dtype(a), dtype(b), dtype(c)
    if not (np.isfinite(a) and np.isfinite(b) and np.isfinite(c)):
        with np.errstate(all="ignore"):
            return dtype(np.float64(a) * np.float64(b) + np.float64(c))
    exact = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    if exact == 0:
        # sign of an exact zero result follows IEEE: -0 only if both terms are -0
        prod_neg = (math.copysign(1, a) * math.copysign(1, b)) < 0
        if prod_neg and math.copysign(1, c) < 0:
            return dtype(-0.0)
        return dtype(0.0)
    return _round_fraction(exact, dtype)


def signum(x, dtype):
    if np.isnan(x):
        return x
    return dtype(-1.0) if np.signbit(x) else dtype(1.0)


def mul_add(a, b, c, dtype, variant=DEFAULT_VARIANT):
    """``a.mul_add(b, c)`` with the ``fma`` feature, ``c += a * b`` without it
    (src/lib.rs:174-177, 226-232, 353-360, 376-383)."""
    if variant & VARIANT_FMA:
        return fma(a, b, c, dtype)
    with np.errstate(all="ignore"):
        return dtype(dtype(c) + dtype(dtype(a) * dtype(b)))


def time_to_next_pixel(vel, frac, dtype, variant=DEFAULT_VARIANT):
    """src/lib.rs:157-180, all four feature builds."""
    one, half = dtype(1.0), dtype(0.5)
    with np.errstate(all="ignore"):
        if not variant & VARIANT_BRANCHLESS:
            if vel > 0:
                return dtype((one - frac) / vel)
            if vel < 0:
                return dtype(-(frac / vel))
            return dtype(np.inf)
        rem = mul_add(one + signum(vel, dtype), dtype(half - frac), frac, dtype, variant)
        return dtype(abs(rem / vel))


def advance(u, v, i, j, fx, fy, bounds, dtype, variant=DEFAULT_VARIANT):
    """src/lib.rs:236-273; bounds = ((xl, xr), (yl, yr), nx, ny), names as str."""
    if u == 0 and v == 0:
        return i, j, fx, fy
    tx = time_to_next_pixel(u, fx, dtype, variant)
    ty = time_to_next_pixel(v, fy, dtype, variant)
    if tx < ty:
        if u >= 0:
            j, fx = j + 1, dtype(0.0)
        else:
            j, fx = j - 1, dtype(1.0)
        fy = mul_add(tx, v, fy, dtype, variant)
    else:
        if v >= 0:
            i, fy = i + 1, dtype(0.0)
        else:
            i, fy = i - 1, dtype(1.0)
        fx = mul_add(ty, u, fx, dtype, variant)
    (xl, xr), (yl, yr), nx, ny = bounds
    j = _apply(j, xl, xr, nx)
    i = _apply(i, yl, yr, ny)
    return i, j, fx, fy


def _apply(c, left, right, size):
    """src/lib.rs:83-96 with -1 standing for usize::MAX."""
    if c == -1:
        return 0 if left == "closed" else size - 1
    if c == size:
        return size - 1 if right == "closed" else 0
    return c


def convolve(texture, u, v, kernel, uv_mode="velocity", boundaries=(("closed",) * 2,) * 2,
             iterations=1, variant=DEFAULT_VARIANT):
    """src/lib.rs:305-443 on tiny arrays; boundaries as ((xl, xr), (yl, yr))."""
    dtype = texture.dtype.type
    ny, nx = texture.shape
    bounds = (tuple(boundaries[0]), tuple(boundaries[1]), nx, ny)
    K = len(kernel)
    kmid = K // 2
    inp = texture.astype(dtype).copy()
    out = np.zeros_like(inp)
    for it in range(iterations):
        out = np.zeros_like(inp)
        for i0 in range(ny):
            for j0 in range(nx):
                acc = mul_add(kernel[kmid], inp[i0, j0], dtype(0.0), dtype, variant)
                for backward in (False, True):
                    i, j = i0, j0
                    fx = fy = dtype(0.5)
                    lu = lv = dtype(0.0)
                    ks = range(kmid - 1, -1, -1) if backward else range(kmid + 1, K)
                    for k in ks:
                        pu, pv = u[i, j], v[i, j]
                        if np.isnan(pu) or np.isnan(pv):
                            break
                        if uv_mode == "polarization":
                            with np.errstate(all="ignore"):
                                if dtype(pu * lu) + dtype(pv * lv) < 0:
                                    pu, pv = -pu, -pv
                            lu, lv = pu, pv
                        if backward:
                            pu, pv = -pu, -pv
                        i, j, fx, fy = advance(pu, pv, i, j, fx, fy, bounds, dtype, variant)
                        acc = mul_add(kernel[k], inp[i, j], acc, dtype, variant)
                out[i0, j0] = acc
        inp = out
    return out
