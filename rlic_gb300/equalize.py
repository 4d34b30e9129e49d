"""Histogram equalization on the GPU: the post-processing step of LIC images.

The reference declares these operations in its native-module stubs
(neutrinoceros/rlic src/rlic/_core.pyi:30-57) without implementing them (its
README, README.md:19-23, points to the separate ``ahe`` package); the
definitions below are this library's own, stated in numpy by the test
oracle and matched bit for bit by the kernels (lic_equalize.cu):

* nbins equal bins over [min, max] of the image's finite pixels;
* ``equalize_histogram``: each pixel becomes the cumulative histogram at its
  bin divided by the number of finite pixels;
* ``equalize_histogram_sliding_tile``: each pixel becomes its rank among the
  finite pixels of the ``tile_shape`` window around it (clipped to the
  image): the fraction whose bin is not above its own;
* ``equalize_histogram_tile_interpolation``: the image is cut into tiles of
  ``tile_shape``; each tile maps bins through its own cumulative histogram,
  and each pixel blends the mappings of the four nearest tile centres
  bilinearly.

Non-finite pixels are returned unchanged.  Images are float32 or float64
numpy arrays (the result is a new numpy array) or CUDA tensors (the result
is a CUDA tensor, computed on the current stream).  The per-dtype names of
the reference's stubs (``equalize_histogram_f32`` and so on) are provided
too.
"""

from __future__ import annotations

__all__ = [
    "equalize_histogram",
    "equalize_histogram_sliding_tile",
    "equalize_histogram_tile_interpolation",
    "equalize_histogram_f32",
    "equalize_histogram_f64",
    "equalize_histogram_sliding_tile_f32",
    "equalize_histogram_sliding_tile_f64",
    "equalize_histogram_tile_interpolation_f32",
    "equalize_histogram_tile_interpolation_f64",
]

import ctypes
import operator
from typing import Any

import numpy as np

from rlic_gb300 import _native

GLOBAL, SLIDING_TILE, TILE_INTERPOLATION = 0, 1, 2
MAX_BINS = 1 << 24
MAX_TILE_BINS = 49152


def _check_nbins(nbins: Any, strategy: int) -> int:
    try:
        n = operator.index(nbins)
    except TypeError:
        raise TypeError(f"nbins must be an integer, got {nbins!r}") from None
    limit = MAX_TILE_BINS if strategy == TILE_INTERPOLATION else MAX_BINS
    if not 1 <= n <= limit:
        raise ValueError(f"nbins must be in [1, {limit}], got {n}")
    return n


def _check_tile(tile_shape: Any) -> tuple[int, int]:
    try:
        th, tw = (operator.index(t) for t in tile_shape)
    except (TypeError, ValueError):
        raise TypeError(f"tile_shape must be a pair of integers, got {tile_shape!r}") from None
    if th < 1 or tw < 1:
        raise ValueError(f"tile_shape must be positive, got {(th, tw)}")
    return th, tw


def _run(image: Any, nbins: int, strategy: int, tile: tuple[int, int]) -> Any:
    lib = _native.lib()
    try:
        import torch
    except ImportError:  # pragma: no cover - torch is a dependency of the package
        torch = None
    if torch is not None and isinstance(image, torch.Tensor):
        if not image.is_cuda:
            raise TypeError("torch tensors must be on a CUDA device")
        if image.dtype not in (torch.float32, torch.float64):
            raise TypeError(f"Found unsupported data type: {image.dtype}")
        if image.ndim != 2:
            raise ValueError(f"Expected a 2D image, got {image.ndim} dimensions")
        x = image.contiguous()
        out = torch.empty_like(x)
        fn = (lib.rlic_equalize_histogram_f32 if x.dtype == torch.float32
              else lib.rlic_equalize_histogram_f64)
        stream = ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
        with torch.cuda.device(x.device):
            _native.check(fn(x.data_ptr(), x.shape[0], x.shape[1], nbins, strategy, tile[0],
                             tile[1], out.data_ptr(), stream, 0))
        return out
    x = np.asarray(image)
    if x.dtype not in (np.dtype("float32"), np.dtype("float64")):
        raise TypeError(f"Found unsupported data type: {x.dtype}")
    if x.ndim != 2:
        raise ValueError(f"Expected a 2D image, got {x.ndim} dimensions")
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    fn = (lib.rlic_equalize_histogram_f32 if x.dtype == np.dtype("float32")
          else lib.rlic_equalize_histogram_f64)
    _native.check(fn(x.ctypes.data, x.shape[0], x.shape[1], nbins, strategy, tile[0], tile[1],
                     out.ctypes.data, None, _native.RLIC_FLAG_HOST_MEMORY))
    return out


def equalize_histogram(image: Any, nbins: int) -> Any:
    """Global histogram equalization (see the module docstring)."""
    return _run(image, _check_nbins(nbins, GLOBAL), GLOBAL, (1, 1))


def equalize_histogram_sliding_tile(image: Any, nbins: int, tile_shape: Any) -> Any:
    """Adaptive equalization: rank of each pixel within its sliding window."""
    return _run(image, _check_nbins(nbins, SLIDING_TILE), SLIDING_TILE, _check_tile(tile_shape))


def equalize_histogram_tile_interpolation(image: Any, nbins: int, tile_shape: Any) -> Any:
    """Adaptive equalization: per-tile mappings blended between tile centres."""
    return _run(image, _check_nbins(nbins, TILE_INTERPOLATION), TILE_INTERPOLATION,
                _check_tile(tile_shape))


def _typed(fn, dtype):
    def call(image, nbins, *args):
        got = (str(image.dtype).replace("torch.", "") if hasattr(image, "is_cuda")
               else str(np.asarray(image).dtype))
        if got != dtype:
            raise TypeError(f"expected a {dtype} image, got {got}")
        return fn(image, nbins, *args)

    call.__name__ = f"{fn.__name__}_{'f32' if dtype == 'float32' else 'f64'}"
    call.__doc__ = f"{fn.__doc__} ({dtype} images only; the reference's stub name.)"
    return call


equalize_histogram_f32 = _typed(equalize_histogram, "float32")
equalize_histogram_f64 = _typed(equalize_histogram, "float64")
equalize_histogram_sliding_tile_f32 = _typed(equalize_histogram_sliding_tile, "float32")
equalize_histogram_sliding_tile_f64 = _typed(equalize_histogram_sliding_tile, "float64")
equalize_histogram_tile_interpolation_f32 = _typed(equalize_histogram_tile_interpolation,
                                                   "float32")
equalize_histogram_tile_interpolation_f64 = _typed(equalize_histogram_tile_interpolation,
                                                   "float64")
