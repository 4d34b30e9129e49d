"""The reference's behavioural suite (tests/test_convolution.py of
neutrinoceros/rlic), restated and run on the GPU through ``import rlic``.

Each test asserts the same identity as its namesake, with the same inputs
and tolerances (most are bitwise).
"""

from __future__ import annotations

from itertools import combinations

import numpy as np
import pytest
from numpy.testing import assert_allclose, assert_array_equal, assert_array_less

import rlic

pytestmark = pytest.mark.gpu

prng = np.random.default_rng(0)
NX = 128


def get_args(nx=NX, klen=11, dtype=np.dtype("float64")):
    return dict(
        img=prng.random((nx, nx), dtype=dtype),
        u=prng.random((nx, nx), dtype=dtype),
        v=prng.random((nx, nx), dtype=dtype),
        kernel=np.linspace(0, 1, klen, dtype=dtype),
    )


ARGS = get_args()


def test_no_iterations() -> None:
    out = rlic.convolve(ARGS["img"], ARGS["u"], ARGS["v"], kernel=ARGS["kernel"], iterations=0)
    assert_array_equal(out, ARGS["img"])


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_single_iteration(dtype) -> None:
    a = get_args(dtype=np.dtype(dtype))
    implicit = rlic.convolve(a["img"], a["u"], a["v"], kernel=a["kernel"])
    explicit = rlic.convolve(a["img"], a["u"], a["v"], kernel=a["kernel"], iterations=1)
    assert implicit.dtype == np.dtype(dtype)
    assert_array_equal(implicit, explicit)


def test_multiple_iterations() -> None:
    outs = [
        rlic.convolve(ARGS["img"], ARGS["u"], ARGS["v"], kernel=ARGS["kernel"], iterations=n)
        for n in range(3)
    ]
    for o1, o2 in combinations(outs, 2):
        assert np.all(o2 != o1)


def test_uv_symmetry() -> None:
    out1 = rlic.convolve(ARGS["img"], ARGS["u"], ARGS["v"], kernel=ARGS["kernel"])
    out2 = rlic.convolve(ARGS["img"].T, ARGS["v"].T, ARGS["u"].T, kernel=ARGS["kernel"]).T
    assert_array_equal(out2, out1)


def test_uv_mode_default() -> None:
    a = rlic.convolve(ARGS["img"], ARGS["u"], ARGS["v"], kernel=ARGS["kernel"])
    b = rlic.convolve(ARGS["img"], ARGS["u"], ARGS["v"], kernel=ARGS["kernel"],
                      uv_mode="velocity")
    assert_array_equal(a, b)


def test_uv_modes_diff() -> None:
    kernel = np.ones(5, dtype="float64")
    u0 = np.ones((NX, NX))
    ii = np.broadcast_to(np.arange(NX), (NX, NX))
    u1 = np.where(ii < NX / 2, u0, -u0)
    u2 = np.where(ii < NX / 2, -u0, u0)
    v = np.zeros((NX, NX))
    vel1 = rlic.convolve(ARGS["img"], u1, v, kernel=kernel, uv_mode="velocity")
    vel2 = rlic.convolve(ARGS["img"], u2, v, kernel=kernel, uv_mode="velocity")
    assert_allclose(vel2, vel1, atol=1e-14)
    pol1 = rlic.convolve(ARGS["img"], u1, v, kernel=kernel, uv_mode="polarization")
    pol2 = rlic.convolve(ARGS["img"], u2, v, kernel=kernel, uv_mode="polarization")
    assert_allclose(pol2, pol1, atol=1e-14)
    assert np.ptp(vel2 - pol2) > 1


@pytest.mark.parametrize("kernel_size", [3, 4])
def test_uv_modes_equiv(kernel_size) -> None:
    kernel = np.ones(kernel_size, dtype="float64")
    vel = rlic.convolve(ARGS["img"], ARGS["u"], ARGS["v"], kernel=kernel, uv_mode="velocity")
    pol = rlic.convolve(ARGS["img"], ARGS["u"], ARGS["v"], kernel=kernel,
                        uv_mode="polarization")
    assert_array_equal(pol, vel)


def test_uv_mode_polarization_sym() -> None:
    kernel = np.ones(5)
    img = np.eye(5)
    zero, one = np.zeros((5, 5)), np.ones((5, 5))
    assert_allclose(
        rlic.convolve(img, u=-one, v=zero, kernel=kernel, uv_mode="polarization"),
        rlic.convolve(img, u=one, v=zero, kernel=kernel, uv_mode="polarization"),
    )
    assert_allclose(
        rlic.convolve(img, u=zero, v=-one, kernel=kernel, uv_mode="polarization"),
        rlic.convolve(img, u=zero, v=one, kernel=kernel, uv_mode="polarization"),
    )


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("niterations", [0, 1, 5])
def test_nan_vectors(dtype, niterations) -> None:
    a = get_args(dtype=np.dtype(dtype))
    nan = np.full_like(a["img"], np.nan)
    out = rlic.convolve(a["img"], nan, nan, kernel=a["kernel"], iterations=niterations)
    scale = out / a["img"]
    assert np.ptp(scale) == 0.0
    assert scale[0, 0] == a["kernel"][len(a["kernel"]) // 2] ** niterations


def test_boundaries() -> None:
    a = get_args(dtype=np.dtype("float64"), nx=64, klen=128)
    one = np.ones_like(a["img"])
    zero = np.zeros_like(a["img"])
    x = np.linspace(0, np.pi, 64)
    ii = np.broadcast_to(np.arange(64), a["img"].shape)
    U = np.where(ii < 32, -one, one)
    V = np.broadcast_to(np.sin(x).T, a["img"].shape)
    closed = rlic.convolve(a["img"], U, V, kernel=a["kernel"], boundaries="closed")
    periodic = rlic.convolve(a["img"], U, V, kernel=a["kernel"], boundaries="periodic")
    assert_array_less(zero, np.abs(closed - periodic))
    xc_yp = rlic.convolve(a["img"], U, V, kernel=a["kernel"],
                          boundaries={"x": "closed", "y": "periodic"})
    yc_xp = rlic.convolve(a["img"], U, V, kernel=a["kernel"],
                          boundaries={"y": "closed", "x": "periodic"})
    assert_array_less(zero, np.abs(xc_yp - periodic))
    assert_array_less(zero, np.abs(yc_xp - closed))
    assert_array_less(zero, np.abs(xc_yp - yc_xp))


def test_inputs_not_mutated() -> None:
    a = get_args(nx=32)
    copies = {k: x.copy() for k, x in a.items()}
    rlic.convolve(a["img"], a["u"], a["v"], kernel=a["kernel"], iterations=3)
    for k in a:
        assert_array_equal(a[k], copies[k])
