"""``rlic._core``: the reference's native-module names over this library.

The CPU tests check the argument handling, which never reaches a GPU
(zero passes and images without pixels return before any launch); the GPU
test checks that the module computes what ``rlic.convolve`` and the oracle
compute, and that, like the native module, it does not validate values.
"""

from __future__ import annotations

import numpy as np
import pytest

import rlic._core as core
from rlic_gb300 import equalize

CLOSED = (("closed", "closed"), ("closed", "closed"))


def _arrays(dtype, shape=(6, 7), klen=5, seed=0):
    rng = np.random.default_rng(seed)
    t, u, v = (rng.random(shape).astype(dtype) for _ in range(3))
    return t, u - dtype(0.5), v - dtype(0.5), np.hanning(klen).astype(dtype)


def test_stub_names() -> None:
    # the functions src/rlic/_core.pyi declares
    for name in ("convolve_f32", "convolve_f64", "equalize_histogram_f32",
                 "equalize_histogram_f64", "equalize_histogram_sliding_tile_f32",
                 "equalize_histogram_sliding_tile_f64",
                 "equalize_histogram_tile_interpolation_f32",
                 "equalize_histogram_tile_interpolation_f64"):
        assert callable(getattr(core, name)), name
        assert name in core.__all__
    assert core.equalize_histogram_f32 is equalize.equalize_histogram_f32


@pytest.mark.parametrize("fn, dtype", [(core.convolve_f32, np.float32),
                                       (core.convolve_f64, np.float64)])
def test_zero_or_negative_iterations_give_zeros(fn, dtype) -> None:
    t, u, v, k = _arrays(dtype)
    for n in (0, -3):
        out = fn(t, (u, v, "velocity"), k, CLOSED, n)
        assert out.dtype == np.dtype(dtype) and out.shape == t.shape
        assert not out.any()
    # the native core validates no values: a negative texture is not an error
    out = fn(-t, (u, v, "polarization"), k, CLOSED, 0)
    assert not out.any()


def test_image_without_pixels() -> None:
    t = np.zeros((0, 4))
    out = core.convolve_f64(t, (t, t, "velocity"), np.ones(3), CLOSED, 2)
    assert out.shape == (0, 4) and out.dtype == np.float64


def test_types_are_checked() -> None:
    t, u, v, k = _arrays(np.float64)
    with pytest.raises(TypeError, match="argument 'texture'"):
        core.convolve_f32(t, (u, v, "velocity"), k, CLOSED, 1)
    with pytest.raises(TypeError, match="argument 'kernel'"):
        core.convolve_f64(t, (u, v, "velocity"), k[None, :], CLOSED, 1)
    with pytest.raises(TypeError, match="argument 'v'"):
        core.convolve_f64(t, (u, v.astype(np.float32), "velocity"), k, CLOSED, 1)
    with pytest.raises(TypeError, match="argument 'uv'"):
        core.convolve_f64(t, (u, v), k, CLOSED, 1)


def test_values_the_native_module_aborts_on_raise_instead() -> None:
    t, u, v, k = _arrays(np.float64)
    with pytest.raises(ValueError, match="uv_mode"):
        core.convolve_f64(t, (u, v, "vorticity"), k, CLOSED, 1)
    with pytest.raises(ValueError, match="boundaries"):
        core.convolve_f64(t, (u, v, "velocity"), k, (("closed", "wall"), ("closed", "closed")), 1)
    with pytest.raises(ValueError, match="boundaries"):
        core.convolve_f64(t, (u, v, "velocity"), k, "closed", 1)
    with pytest.raises(ValueError, match="shape mismatch"):
        core.convolve_f64(t, (u[:, :-1], v, "velocity"), k, CLOSED, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("fn, dtype", [(core.convolve_f32, np.float32),
                                       (core.convolve_f64, np.float64)])
def test_matches_convolve_and_oracle(oracle, fn, dtype) -> None:
    import rlic

    t, u, v, k = _arrays(dtype, shape=(96, 80), klen=21, seed=4)
    bnd = (("periodic", "periodic"), ("closed", "closed"))
    got = fn(t, (u, v, "polarization"), k, bnd, 3)
    want = rlic.convolve(t, u, v, kernel=k, uv_mode="polarization",
                         boundaries={"x": "periodic", "y": "closed"}, iterations=3)
    assert got.tobytes() == want.tobytes()
    # no value validation: a negative texture is convolved like any other
    got = fn(-t, (u, v, "velocity"), k, bnd, 2)
    want = oracle.convolve(-t, u, v, k, uv_mode="velocity", boundaries=bnd, iterations=2)
    assert got.tobytes() == want.tobytes()
