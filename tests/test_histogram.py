"""Histogram equalization: the numpy definition's properties and the Python
API's argument checks (CPU; the GPU results are compared with the definition
in test_gpu_histogram.py).

The reference only declares these functions (src/rlic/_core.pyi:30-57); the
definition in oracle/histogram.py is this repository's, so these tests pin
its basic properties: the global form is the empirical CDF of the finite
pixels, a window or a tile covering the whole image reduces the adaptive
forms to the global one, and non-finite pixels pass through.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import histogram as H


@pytest.fixture(params=[np.float32, np.float64])
def image(request):
    rng = np.random.default_rng(5)
    x = rng.normal(size=(23, 31)).astype(request.param)
    x[3, 4] = np.nan
    x[7, 1] = np.inf
    x[9, 9] = -np.inf
    return x


def test_global_is_the_empirical_cdf(image) -> None:
    out = H.equalize_global(image, 64)
    fin = np.isfinite(image)
    assert out.dtype == image.dtype
    np.testing.assert_array_equal(out[~fin], image[~fin])
    v, o = image[fin], out[fin]
    order = np.argsort(v, kind="stable")
    assert np.all(np.diff(o[order]) >= 0)  # monotone in the input
    assert o.max() == 1 and o.min() > 0
    # with as many bins as distinct values, it is the exact rank fraction
    rank = H.equalize_global(image, 1 << 20)[fin]
    want = (np.searchsorted(np.sort(v), v, side="right") / v.size).astype(image.dtype)
    assert np.max(np.abs(rank - want)) <= 2 / v.size


def test_whole_image_window_and_tile_reduce_to_global(image) -> None:
    ny, nx = image.shape
    g = H.equalize_global(image, 32)
    np.testing.assert_array_equal(H.equalize_sliding_tile(image, 32, (2 * ny + 1, 2 * nx + 1)), g)
    np.testing.assert_array_equal(H.equalize_tile_interpolation(image, 32, (ny, nx)), g)


def test_tile_interpolation_blends_between_centres(image) -> None:
    out = H.equalize_tile_interpolation(image, 16, (8, 8))
    fin = np.isfinite(image)
    assert np.all((out[fin] >= 0) & (out[fin] <= 1))
    np.testing.assert_array_equal(out[~fin], image[~fin])


def test_constant_and_empty_images() -> None:
    c = np.full((5, 6), 3.5, dtype=np.float32)
    np.testing.assert_array_equal(H.equalize_global(c, 8), np.ones_like(c))
    nan = np.full((4, 4), np.nan)
    np.testing.assert_array_equal(H.equalize_global(nan, 8), nan)


def test_python_api_checks_arguments() -> None:
    from rlic_gb300 import equalize as E

    x = np.zeros((4, 4), dtype=np.float32)
    with pytest.raises(ValueError, match="nbins"):
        E.equalize_histogram(x, 0)
    with pytest.raises(TypeError, match="nbins"):
        E.equalize_histogram(x, 2.5)
    with pytest.raises(ValueError, match="nbins"):
        E.equalize_histogram_tile_interpolation(x, E.MAX_TILE_BINS + 1, (2, 2))
    with pytest.raises(ValueError, match="tile_shape"):
        E.equalize_histogram_sliding_tile(x, 8, (0, 3))
    with pytest.raises(TypeError, match="tile_shape"):
        E.equalize_histogram_sliding_tile(x, 8, 3)
    with pytest.raises(TypeError, match="float32"):
        E.equalize_histogram_f32(x.astype(np.float64), 8)
