"""``rlic._core``: the reference's native-module surface, served by rlic_gb300.

neutrinoceros/rlic builds ``rlic._core`` from Rust with PyO3
(src/lib.rs:448-485; signatures in src/rlic/_core.pyi:8-57).  This module
gives the same names and arguments over the C ABI of ``librlic_gb300.so``,
so that code written against the native module, the reference's own
``src/rlic/_lib.py`` included (it imports ``convolve_f32`` and
``convolve_f64`` from here), runs unchanged on the GPU.

Like the native functions, these check types, not values: the caller
validates first, as ``rlic.convolve`` does.  Inputs are read, never
written, and each call returns a new array.  Where the native module aborts
the process (an unknown mode or boundary string, src/lib.rs:24, 65;
mismatched shapes, which index out of bounds) these raise ValueError; a
wrong dtype or rank raises TypeError, as PyO3's argument extraction does.
A negative iteration count runs no pass and returns zeros, as the native
loop does (src/lib.rs:432-441).

The histogram-equalization names of the stubs are this library's GPU
implementations (``rlic_gb300.equalize``); the reference declares them
without implementing them.
"""

from __future__ import annotations

import operator
from typing import Any

import numpy as np

from rlic_gb300 import _native
from rlic_gb300._boundaries import BOUNDARY_CODES
from rlic_gb300._lib import _convolve_numpy
from rlic_gb300.equalize import (
    equalize_histogram_f32,
    equalize_histogram_f64,
    equalize_histogram_sliding_tile_f32,
    equalize_histogram_sliding_tile_f64,
    equalize_histogram_tile_interpolation_f32,
    equalize_histogram_tile_interpolation_f64,
)

__all__ = [
    "convolve_f32",
    "convolve_f64",
    "equalize_histogram_f32",
    "equalize_histogram_f64",
    "equalize_histogram_sliding_tile_f32",
    "equalize_histogram_sliding_tile_f64",
    "equalize_histogram_tile_interpolation_f32",
    "equalize_histogram_tile_interpolation_f64",
]


def _native_call(dtype: np.dtype, texture: Any, uv: Any, kernel: Any, boundaries: Any,
                 iterations: Any) -> np.ndarray:
    try:
        u, v, uv_mode = uv
    except (TypeError, ValueError):
        raise TypeError("argument 'uv': expected a tuple (u, v, uv_mode)") from None
    for name, a, ndim in (("texture", texture, 2), ("u", u, 2), ("v", v, 2),
                          ("kernel", kernel, 1)):
        if not isinstance(a, np.ndarray) or a.dtype != dtype or a.ndim != ndim:
            raise TypeError(f"argument '{name}': expected a {ndim}-D numpy array of {dtype}")
    if not isinstance(uv_mode, str) or uv_mode not in _native.UV_MODE_CODES:
        raise ValueError(f"unknown uv_mode {uv_mode!r}")
    try:
        (xl, xr), (yl, yr) = boundaries
        bcodes = tuple(BOUNDARY_CODES[s] for s in (xl, xr, yl, yr))
    except (KeyError, TypeError, ValueError):
        raise ValueError(f"invalid boundaries {boundaries!r}: expected "
                         "((x_left, x_right), (y_left, y_right)) of 'closed'/'periodic'") from None
    if u.shape != texture.shape or v.shape != texture.shape:
        raise ValueError(f"shape mismatch: texture {texture.shape}, u {u.shape}, v {v.shape}")
    n = max(0, operator.index(iterations))
    return _convolve_numpy(texture, u, v, kernel, _native.UV_MODE_CODES[uv_mode], bcodes, n,
                           check_texture=False)


def convolve_f32(texture: Any, uv: Any, kernel: Any, boundaries: Any,
                 iterations: int = 1) -> np.ndarray:
    """float32 line integral convolution (rlic._core.convolve_f32, src/lib.rs:451-465)."""
    return _native_call(np.dtype("float32"), texture, uv, kernel, boundaries, iterations)


def convolve_f64(texture: Any, uv: Any, kernel: Any, boundaries: Any,
                 iterations: int = 1) -> np.ndarray:
    """float64 line integral convolution (rlic._core.convolve_f64, src/lib.rs:467-482)."""
    return _native_call(np.dtype("float64"), texture, uv, kernel, boundaries, iterations)
