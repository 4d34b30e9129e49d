"""Pins the CPU oracle to the reference before anything is checked against it.

Three sources, none of which needs a GPU:

* the reference's Rust known-answer tests (src/lib.rs:139-151, 182-206,
  275-297);
* the exact identities its Python suite asserts on outputs
  (tests/test_convolution.py:42-206), evaluated here on the oracle;
* an independent pure-Python restatement (oracle/pyoracle.py) on tiny
  images, which must agree bit for bit in all four Cargo feature builds;
* committed golden vectors (tests/golden/), which must reproduce exactly on
  every host the oracle is built on.
"""

from __future__ import annotations

from itertools import combinations
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle

GOLDEN = Path(__file__).resolve().parent / "golden"


# ------------------------------------------------------------------ KATs --

@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_time_to_next_pixel_kats(oracle, dtype) -> None:
    # src/lib.rs:186-205
    assert oracle.time_to_next_pixel(1.0, 0.0, dtype) == 1.0
    assert oracle.time_to_next_pixel(-1.0, 1.0, dtype) == 1.0
    assert oracle.time_to_next_pixel(0.0, 0.5, dtype) == np.inf


def test_time_to_next_pixel_signed_zero_and_variants(oracle) -> None:
    # branchless: |fma(1 + signum(v), 0.5 - f, f) / v|, signum(-0.0) = -1
    assert oracle.time_to_next_pixel(-0.0, 0.5) == np.inf
    assert np.isnan(oracle.time_to_next_pixel(0.0, 1.0))  # 0/0
    assert np.isnan(oracle.time_to_next_pixel(-0.0, 0.0))  # 0/-0
    # branchy variant returns +inf for any zero velocity
    for var in (0, 1):
        assert oracle.time_to_next_pixel(0.0, 1.0, variant=var) == np.inf
        assert oracle.time_to_next_pixel(-0.0, 0.0, variant=var) == np.inf
    # rounding: fma(2, 0.5 - f, f) vs (1 - f) differ for some f < 0.25
    f = np.float32(0.1)
    a = oracle.time_to_next_pixel(3.0, float(f), np.float32, variant=3)
    b = oracle.time_to_next_pixel(3.0, float(f), np.float32, variant=1)
    assert a == pytest.approx(b, rel=1e-6)


def test_advance_zero_velocity_kat(oracle) -> None:
    # src/lib.rs:279-296
    assert oracle.advance(0.0, 0.0, 5, 5, 0.5, 0.5, (10, 10)) == (5, 5, 0.5, 0.5)


def test_advance_steps_and_boundaries(oracle) -> None:
    # +x step from the pixel centre: tx = 0.5 < ty = inf
    assert oracle.advance(1.0, 0.0, 5, 5, 0.5, 0.5, (10, 10)) == (5, 6, 0.0, 0.5)
    # tie (tx == ty) takes the y branch
    assert oracle.advance(1.0, 1.0, 5, 5, 0.5, 0.5, (10, 10)) == (6, 5, 1.0, 0.0)
    # -0.0 velocity counts as >= 0: y step upward
    i, j, fx, fy = oracle.advance(-0.0, -1.0, 5, 5, 0.5, 0.5, (10, 10))
    assert (i, j) == (4, 5)
    # closed boundary clamps, periodic wraps; the fraction is not reset
    assert oracle.advance(-1.0, 0.0, 3, 0, 0.5, 0.5, (10, 10), "closed")[:3] == (3, 0, 1.0)
    assert oracle.advance(-1.0, 0.0, 3, 0, 0.5, 0.5, (10, 10), "periodic")[:3] == (3, 9, 1.0)
    assert oracle.advance(0.0, 1.0, 9, 2, 0.5, 0.5, (10, 10), "closed")[:2] == (9, 2)
    assert oracle.advance(0.0, 1.0, 9, 2, 0.5, 0.5, (10, 10), "periodic")[:2] == (0, 2)
    # mixed sides (computed by the native core even though Python rejects them)
    b = {"x": ("closed", "periodic"), "y": "closed"}
    assert oracle.advance(1.0, 0.0, 0, 9, 0.5, 0.5, (10, 10), b)[:2] == (0, 0)
    assert oracle.advance(-1.0, 0.0, 0, 0, 0.5, 0.5, (10, 10), b)[:2] == (0, 0)


# ------------------------------------------------------------ identities --

prng = np.random.default_rng(0)
NX = 64


def _args(nx=NX, klen=11, dtype=np.float64):
    return (
        prng.random((nx, nx), dtype=dtype),
        prng.random((nx, nx), dtype=dtype),
        prng.random((nx, nx), dtype=dtype),
        np.linspace(0, 1, klen, dtype=dtype),
    )


def test_iterations_all_differ(oracle) -> None:
    img, u, v, k = _args()
    outs = [img] + [oracle.convolve(img, u, v, k, iterations=n) for n in (1, 2)]
    for a, b in combinations(outs, 2):
        assert np.all(a != b)


def test_iterations_compose(oracle) -> None:
    img, u, v, k = _args()
    two = oracle.convolve(img, u, v, k, iterations=2)
    once = oracle.convolve(oracle.convolve(img, u, v, k), u, v, k)
    np.testing.assert_array_equal(two, once)


def test_uv_transpose_symmetry(oracle) -> None:
    # tests/test_convolution.py:69-82: bitwise
    img, u, v, k = _args()
    a = oracle.convolve(img, u, v, k)
    b = oracle.convolve(img.T, v.T, u.T, k).T
    np.testing.assert_array_equal(a, b)


def test_uv_modes_diff(oracle) -> None:
    # tests/test_convolution.py:93-110
    img = _args()[0]
    kernel = np.ones(5)
    ones = np.ones((NX, NX))
    ii = np.broadcast_to(np.arange(NX), (NX, NX))
    u1 = np.where(ii < NX / 2, ones, -ones)
    u2 = -u1
    v = np.zeros((NX, NX))
    vel1 = oracle.convolve(img, u1, v, kernel, uv_mode="velocity")
    vel2 = oracle.convolve(img, u2, v, kernel, uv_mode="velocity")
    np.testing.assert_allclose(vel2, vel1, atol=1e-14)
    pol1 = oracle.convolve(img, u1, v, kernel, uv_mode="polarization")
    pol2 = oracle.convolve(img, u2, v, kernel, uv_mode="polarization")
    np.testing.assert_allclose(pol2, pol1, atol=1e-14)
    assert np.ptp(vel2 - pol2) > 1


@pytest.mark.parametrize("klen", [3, 4])
def test_short_kernel_polarization_is_velocity(oracle, klen) -> None:
    # tests/test_convolution.py:113-122
    img, u, v, _ = _args()
    k = np.ones(klen)
    np.testing.assert_array_equal(
        oracle.convolve(img, u, v, k, uv_mode="polarization"),
        oracle.convolve(img, u, v, k, uv_mode="velocity"),
    )


def test_polarization_sign_symmetry(oracle) -> None:
    # tests/test_convolution.py:125-162
    img = np.eye(5)
    k = np.ones(5)
    zero, one = np.zeros((5, 5)), np.ones((5, 5))
    for a, b in (((one, zero), (-one, zero)), ((zero, one), (zero, -one))):
        np.testing.assert_allclose(
            oracle.convolve(img, *a, k, uv_mode="polarization"),
            oracle.convolve(img, *b, k, uv_mode="polarization"),
        )


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 5])
def test_nan_field_scales_texture(oracle, dtype, n) -> None:
    # tests/test_convolution.py:165-177: exact
    img, _, _, k = _args(dtype=dtype)
    nan = np.full_like(img, np.nan)
    out = oracle.convolve(img, nan, nan, k, iterations=n)
    scale = out / img
    assert np.ptp(scale) == 0.0
    assert scale[0, 0] == k[len(k) // 2] ** n


def test_boundary_kinds_differ(oracle) -> None:
    # tests/test_convolution.py:180-206
    img, _, _, k = _args(nx=64, klen=128)
    ones = np.ones_like(img)
    x = np.linspace(0, np.pi, 64)
    ii = np.broadcast_to(np.arange(64), img.shape)
    U = np.where(ii < 32, -ones, ones)
    V = np.broadcast_to(np.sin(x).T, img.shape)
    closed = oracle.convolve(img, U, V, k, boundaries="closed")
    periodic = oracle.convolve(img, U, V, k, boundaries="periodic")
    xc_yp = oracle.convolve(img, U, V, k, boundaries={"x": "closed", "y": "periodic"})
    xp_yc = oracle.convolve(img, U, V, k, boundaries={"x": "periodic", "y": "closed"})
    assert np.all(np.abs(closed - periodic) > 0)
    assert np.all(np.abs(xc_yp - periodic) > 0)
    assert np.all(np.abs(xp_yc - closed) > 0)
    assert np.all(np.abs(xc_yp - xp_yc) > 0)


def test_iterations_zero_gives_zeros(oracle) -> None:
    # the native core returns its zeroed output buffer (src/lib.rs:425, 433)
    img, u, v, k = _args(nx=8)
    assert not oracle.convolve(img, u, v, k, iterations=0).any()


def test_openmp_rows_bit_identical(oracle) -> None:
    img, u, v, k = _args(nx=96, klen=33)
    a = oracle.convolve(img, u, v, k, uv_mode="polarization", nthreads=1)
    b = oracle.convolve(img, u, v, k, uv_mode="polarization", nthreads=4)
    np.testing.assert_array_equal(a, b)


def test_sweep_rows_matches_full(oracle) -> None:
    img, u, v, k = _args(nx=48, klen=21)
    full = oracle.convolve(img, u, v, k, boundaries="periodic")
    band = oracle.sweep_rows(img, u, v, k, 10, 30, boundaries="periodic")
    np.testing.assert_array_equal(band, full[10:30])


def test_paths_consistent_with_convolution(oracle) -> None:
    # Summing kernel-weighted texture along the oracle's recorded cells gives
    # back its convolution output (default build accumulates with fma).
    img, u, v, k = _args(nx=24, klen=9)
    u = u - 0.5
    v = v - 0.5
    pix = np.arange(24 * 24)
    cells = oracle.paths(u, v, len(k), pix, uv_mode="polarization")
    out = oracle.convolve(img, u, v, k, uv_mode="polarization")
    kmid = len(k) // 2
    nf = len(k) - kmid - 1
    flat = img.ravel()
    for p in (0, 17, 300, 575):
        acc = pyoracle.fma(k[kmid], flat[p], 0.0, np.float64)
        for s in range(nf):
            acc = pyoracle.fma(k[kmid + 1 + s], flat[cells[p, s]], acc, np.float64)
        for s in range(kmid):
            acc = pyoracle.fma(k[kmid - 1 - s], flat[cells[p, nf + s]], acc, np.float64)
        assert acc == out.ravel()[p]


# ------------------------------------------ independent Python restatement --

def _tiny_cases():
    rng = np.random.default_rng(7)
    for dtype in (np.float32, np.float64):
        for mode in ("velocity", "polarization"):
            for bnd in ((("closed",) * 2, ("closed",) * 2), (("periodic",) * 2, ("closed",) * 2),
                        (("periodic",) * 2, ("periodic",) * 2)):
                ny, nx = 6, 7
                tex = rng.random((ny, nx)).astype(dtype)
                u = (rng.random((ny, nx)) - 0.5).astype(dtype)
                v = (rng.random((ny, nx)) - 0.5).astype(dtype)
                u[1, 2] = v[1, 2] = 0.0
                u[3, 3] = -0.0
                v[2, 5] = np.nan
                k = rng.random(9).astype(dtype)
                yield tex, u, v, k, mode, bnd


@pytest.mark.parametrize("variant", [3, 2, 1, 0], ids=["fma-branchless", "branchless",
                                                      "fma", "plain"])
@pytest.mark.parametrize("case", list(_tiny_cases()))
def test_oracle_matches_python_restatement(oracle, case, variant) -> None:
    # every Cargo feature build of the reference (Cargo.toml:27-30)
    tex, u, v, k, mode, bnd = case
    want = pyoracle.convolve(tex, u, v, k, mode, bnd, iterations=2, variant=variant)
    got = oracle.convolve(tex, u, v, k, uv_mode=mode, boundaries=bnd, iterations=2,
                          variant=variant)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_time_to_next_pixel_variants_match_python_restatement(oracle, dtype) -> None:
    # src/lib.rs:157-180 in all four builds, bit for bit, on random velocities
    # over twelve decades (signed zeros included) and fractions in [0, 1]
    rng = np.random.default_rng(12)
    n = 1200
    vel = ((rng.random(n) - 0.5) * 10.0 ** rng.integers(-6, 6, n)).astype(dtype)
    vel[:4] = (0.0, -0.0, 1e-30, -1e30)
    frac = rng.random(n).astype(dtype)
    frac[4:40], frac[40:76], frac[76:96] = 0.0, 1.0, 0.5
    frac[96:900] *= dtype(0.3)  # f < 1/4 with a full significand: 0.5 - f inexact
    differs = 0
    for x, f in zip(vel, frac):
        got = [oracle.time_to_next_pixel(float(x), float(f), dtype, variant=var)
               for var in range(4)]
        for var in range(4):
            want = pyoracle.time_to_next_pixel(x, f, dtype, var)
            assert np.asarray(got[var], dtype).tobytes() == np.asarray(want, dtype).tobytes(), (
                x, f, var)
        differs += got[0] != got[3]
    # the branchy and branchless forms round differently on some inputs
    assert differs > 0


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_fma_feature_changes_outputs(oracle, dtype) -> None:
    # with and without `fma` the accumulation rounds differently (src/lib.rs:353-360)
    rng = np.random.default_rng(11)
    n = 24
    tex = rng.random((n, n)).astype(dtype)
    u = (rng.random((n, n)) - 0.5).astype(dtype)
    v = (rng.random((n, n)) - 0.5).astype(dtype)
    k = rng.random(15).astype(dtype)
    outs = [oracle.convolve(tex, u, v, k, variant=var) for var in range(4)]
    assert not np.array_equal(outs[3], outs[2])
    assert not np.array_equal(outs[1], outs[0])


def test_python_fma_single_rounding() -> None:
    # 1 + 2^-24 is not a float32; (1 + 2^-12)^2 - 1 needs one rounding
    a = np.float32(1 + 2.0**-12)
    got = pyoracle.fma(a, a, np.float32(-1), np.float32)
    assert got == np.float32(2.0**-11 + 2.0**-24)
    assert np.float32(a * a) - np.float32(1) == np.float32(2.0**-11)


# ---------------------------------------------------------- row bands --

@pytest.mark.parametrize("bnd", ["closed", "periodic", {"x": "closed", "y": "periodic"},
                                 {"x": "periodic", "y": "closed"}], ids=str)
def test_convolve_rows_equals_full_convolution(oracle, bnd) -> None:
    """The band evaluation that checks the GPU at full image sizes gives the
    rows of the full n-pass convolution exactly, at edges and in the middle,
    for kernels of odd and even length."""
    rng = np.random.default_rng(31)
    n = 90
    tex = rng.random((n, n))
    u = rng.random((n, n)) - 0.5
    v = rng.random((n, n)) - 0.5
    u[rng.random((n, n)) < 0.02] = 0.0
    v[u == 0.0] = 0.0
    for klen in (9, 12):
        k = np.hanning(klen + 2)[1:-1]
        full = oracle.convolve(tex, u, v, k, uv_mode="polarization", boundaries=bnd,
                               iterations=4)
        for r0, r1 in ((0, 3), (40, 47), (87, 90), (12, 13)):
            band = oracle.convolve_rows(tex, u, v, k, r0, r1, uv_mode="polarization",
                                        boundaries=bnd, iterations=4)
            np.testing.assert_array_equal(band, full[r0:r1])


# ------------------------------------------------------------- golden --

def _golden_files():
    return sorted(GOLDEN.glob("*.npz"))


@pytest.mark.parametrize("path", _golden_files(), ids=lambda p: p.stem)
def test_oracle_reproduces_golden(oracle, path) -> None:
    g = np.load(path, allow_pickle=False)
    bnd = ((str(g["bx"][0]), str(g["bx"][1])), (str(g["by"][0]), str(g["by"][1])))
    out = oracle.convolve(
        g["texture"], g["u"], g["v"], g["kernel"], uv_mode=str(g["uv_mode"]),
        boundaries=bnd, iterations=int(g["iterations"]), variant=int(g["variant"]),
    )
    np.testing.assert_array_equal(out, g["out"])
    if "cells" in g.files:
        cells = oracle.paths(g["u"], g["v"], g["kernel"].size, g["pix"],
                             uv_mode=str(g["uv_mode"]), boundaries=bnd,
                             variant=int(g["variant"]))
        np.testing.assert_array_equal(cells, g["cells"])


def test_oracle_matches_python_restatement_on_random_cases(oracle) -> None:
    """Property: the C oracle and the Python restatement agree bit for bit
    (signed zeros and NaN payloads included) on random tiny cases: shapes
    down to one row or column, kernels of 1 to 9 taps (even lengths too),
    fields holding ±0, NaN, ±inf, subnormals and huge values, every side's
    boundary drawn on its own, both uv modes, 1 to 3 iterations, all four
    feature builds."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    specials = [0.0, -0.0, np.nan, np.inf, -np.inf, 1e-310, -1e-310, 1e30, -1e30, 0.5, -0.5]

    @hyp.settings(max_examples=120, deadline=None, derandomize=True)
    @hyp.given(
        ny=st.integers(1, 6), nx=st.integers(1, 6), klen=st.integers(1, 9),
        dtype=st.sampled_from([np.float32, np.float64]),
        mode=st.sampled_from(["velocity", "polarization"]),
        sides=st.tuples(*[st.sampled_from(["closed", "periodic"])] * 4),
        iterations=st.integers(1, 3), variant=st.integers(0, 3),
        seed=st.integers(0, 2**31 - 1), special_rate=st.sampled_from([0.0, 0.2, 0.5]),
    )
    def check(ny, nx, klen, dtype, mode, sides, iterations, variant, seed, special_rate):
        rng = np.random.default_rng(seed)
        tex = rng.random((ny, nx)).astype(dtype)
        u = (rng.random((ny, nx)) - 0.5).astype(dtype)
        v = (rng.random((ny, nx)) - 0.5).astype(dtype)
        for a in (u, v):
            mask = rng.random((ny, nx)) < special_rate
            a[mask] = rng.choice(specials, int(mask.sum())).astype(dtype)
        k = (rng.random(klen) - 0.25).astype(dtype)
        bnd = ((sides[0], sides[1]), (sides[2], sides[3]))
        want = pyoracle.convolve(tex, u, v, k, mode, bnd, iterations=iterations, variant=variant)
        got = oracle.convolve(tex, u, v, k, uv_mode=mode, boundaries=bnd,
                              iterations=iterations, variant=variant)
        assert got.dtype == want.dtype and got.tobytes() == want.tobytes()

    check()
