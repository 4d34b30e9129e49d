"""ctypes binding of ``librlic_gb300.so`` (C ABI in ``include/rlic_gb300.h``).

The shared library is built in-tree by ``rlic_gb300._build`` (or
``__graft_entry__.build()``).  There is no fallback: when the library is
missing or cannot be loaded, every call that needs it raises
``NativeLibraryError``.
"""

from __future__ import annotations

import ctypes
import math
import os
import threading
import weakref
from pathlib import Path

# the in-tree build, or another build of the same sources named by
# RLIC_GB300_LIBRARY (for example one compiled with different tuning macros)
LIB_PATH = Path(os.environ.get("RLIC_GB300_LIBRARY") or
                Path(__file__).resolve().with_name("librlic_gb300.so"))

RLIC_OK = 0
RLIC_ERR_INVALID_ARGUMENT = 1
RLIC_ERR_CUDA = 2
RLIC_ERR_OUT_OF_MEMORY = 3
RLIC_ERR_WORKSPACE_TOO_SMALL = 4
RLIC_ERR_NEGATIVE_TEXTURE = 5
RLIC_ERR_UNSUPPORTED = 6

RLIC_UV_VELOCITY = 0
RLIC_UV_POLARIZATION = 1

RLIC_FLAG_HOST_MEMORY = 0x1
RLIC_FLAG_NO_FMA = 0x2
RLIC_FLAG_NO_BRANCHLESS = 0x4
RLIC_FLAG_NO_PATH_CACHE = 0x8
RLIC_FLAG_CHECK_TEXTURE = 0x20
RLIC_FLAG_FIELD_NAN_FREE = 0x40
RLIC_FLAG_BATCH_QUEUE = 0x80

RLIC_STORAGE_FP16 = 0
RLIC_STORAGE_BF16 = 1

RLIC_REPLAY_AUTO = 0
RLIC_REPLAY_L1 = 1
RLIC_REPLAY_STAGED = 2

# size of the static scratch of rlic_convolve_f32_noalloc (RLIC_NOALLOC_SCRATCH_BYTES)
NOALLOC_SCRATCH_BYTES = 64 << 20

UV_MODE_CODES: dict[str, int] = {
    "velocity": RLIC_UV_VELOCITY,
    "polarization": RLIC_UV_POLARIZATION,
}

# Every symbol the header declares, with its ctypes signature.
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_INT = ctypes.c_int
_SZ = ctypes.c_size_t
_U = ctypes.c_uint
_CONVOLVE_ARGS = [_P, _P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT, _INT, _I64, _P, _P,
                  _SZ, _P, _U]
_TRACE_ARGS = [_P, _P, _I64, _I64, _I64, _INT, _INT, _INT, _INT, _INT, _I64, _P, _P, _P, _U]
SIGNATURES: dict[str, tuple[list, object]] = {
    "rlic_version": ([], ctypes.c_char_p),
    "rlic_last_error": ([], ctypes.c_char_p),
    "rlic_workspace_bytes": ([_I64, _I64, _I64, _I64, _INT, _U], _SZ),
    "rlic_path_code_bytes": ([_I64, _I64, _I64], _SZ),
    "rlic_convolve_f32": (_CONVOLVE_ARGS, _INT),
    "rlic_convolve_f64": (_CONVOLVE_ARGS, _INT),
    "rlic_convolve_strided_f32": ([_P, _P, _P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT,
                                   _INT, _I64, _P, _P, _U], _INT),
    "rlic_convolve_strided_f64": ([_P, _P, _P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT,
                                   _INT, _I64, _P, _P, _U], _INT),
    "rlic_host_direct_access": ([], _INT),
    "rlic_trace_cells_f32": (_TRACE_ARGS, _INT),
    "rlic_trace_cells_f64": (_TRACE_ARGS, _INT),
    "rlic_pack_field_f32": ([_P, _P, _I64, _I64, _P, _P], _INT),
    "rlic_pack_field_f64": ([_P, _P, _I64, _I64, _P, _P], _INT),
    "rlic_sweep_f32": ([_P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT, _INT, _P, _P, _P,
                        _U], _INT),
    "rlic_sweep_f64": ([_P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT, _INT, _P, _P, _P,
                        _U], _INT),
    "rlic_replay_f32": ([_P, _P, _I64, _I64, _P, _I64, _P, _P, _U], _INT),
    "rlic_replay_f64": ([_P, _P, _I64, _I64, _P, _I64, _P, _P, _U], _INT),
    "rlic_lowp_workspace_bytes": ([_I64, _I64, _I64, _INT], _SZ),
    "rlic_convolve_lowp_f32": ([_P, _P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT, _INT,
                                _I64, _INT, _P, _P, _SZ, _P, _U], _INT),
    "rlic_convolve_lowp_f64": ([_P, _P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT, _INT,
                                _I64, _INT, _P, _P, _SZ, _P, _U], _INT),
    "rlic_adjoint_f32": ([_P, _P, _I64, _I64, _P, _I64, _P, _P, _U], _INT),
    "rlic_adjoint_f64": ([_P, _P, _I64, _I64, _P, _I64, _P, _P, _U], _INT),
    "rlic_kernel_grad_f32": ([_P, _P, _P, _I64, _I64, _I64, _P, _P, _U], _INT),
    "rlic_kernel_grad_f64": ([_P, _P, _P, _I64, _I64, _I64, _P, _P, _U], _INT),
    "rlic_batch_workspace_bytes_f32": ([_P, _INT], _SZ),
    "rlic_convolve_batch_f32": ([_P, _INT, _P, _SZ, _P, _U], _INT),
    "rlic_batch_status_f32": ([_P, _INT, _P], _INT),
    "rlic_convolve_f32_noalloc": ([_P, _P, _P, _I64, _I64, _P, _I64, _INT, _INT, _INT, _INT,
                                   _INT, _I64, _P, _P, _U], _INT),
    "rlic_check_quotients_f64": ([_P, _P, _I64, _P, _P, _P], _INT),
    "rlic_check_numerators_f64": ([_P, _I64, _P, _P, _P], _INT),
    "rlic_equalize_histogram_f32": ([_P, _I64, _I64, _I64, _INT, _I64, _I64, _P, _P, _U], _INT),
    "rlic_equalize_histogram_f64": ([_P, _I64, _I64, _I64, _INT, _I64, _I64, _P, _P, _U], _INT),
    "rlic_set_block_shape": ([_INT, _INT], _INT),
    "rlic_set_replay_mode": ([_INT, _INT], _INT),
    "rlic_set_split_pixels": ([_I64], _INT),
    "rlic_stage_timeouts": ([], _INT),
    "rlic_kernel_launch_count": ([], ctypes.c_uint64),
    "rlic_release_cached_memory": ([], _INT),
    "rlic_host_buffer_alloc": ([_SZ], _P),
    "rlic_host_buffer_free": ([_P], None),
}


class BatchItemF32(ctypes.Structure):
    """rlic_batch_item_f32 (include/rlic_gb300.h)."""

    _fields_ = [
        ("texture", ctypes.c_void_p), ("u", ctypes.c_void_p), ("v", ctypes.c_void_p),
        ("kernel", ctypes.c_void_p), ("out", ctypes.c_void_p),
        ("ny", ctypes.c_int64), ("nx", ctypes.c_int64), ("klen", ctypes.c_int64),
        ("iterations", ctypes.c_int64),
        ("uv_mode", ctypes.c_int), ("bx_left", ctypes.c_int), ("bx_right", ctypes.c_int),
        ("by_left", ctypes.c_int), ("by_right", ctypes.c_int), ("tile_x", ctypes.c_int),
        ("replay_tiles", ctypes.c_int),
    ]


RLIC_FLAG_BATCH_PREPARED = 0x10


class NativeLibraryError(RuntimeError):
    """The native library is missing, failed to load, or a call failed."""

    def __init__(self, message: str, code: int | None = None) -> None:
        super().__init__(message)
        self.code = code


_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def lib() -> ctypes.CDLL:
    """The loaded library (loaded on first use)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise NativeLibraryError(
                    f"{LIB_PATH.name} is not built: run `python -m rlic_gb300._build` "
                    "(needs nvcc) before using rlic_gb300"
                )
            try:
                handle = ctypes.CDLL(str(LIB_PATH))
            except OSError as exc:
                raise NativeLibraryError(f"cannot load {LIB_PATH}: {exc}") from exc
            for name, (argtypes, restype) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.argtypes = argtypes
                fn.restype = restype
            _lib = handle
    return _lib


def check(code: int) -> None:
    """Raise NativeLibraryError for a non-zero status code."""
    if code != RLIC_OK:
        msg = lib().rlic_last_error().decode(errors="replace")
        if code == RLIC_ERR_OUT_OF_MEMORY:
            raise MemoryError(f"rlic_gb300: {msg}")
        raise NativeLibraryError(f"rlic_gb300 error {code}: {msg}", code)


def pinned_empty(shape: tuple, dtype) -> "np.ndarray":
    """A new numpy array in a page-locked block from the library's host cache.

    The block returns to the cache when the array (and every view of it) is
    garbage-collected.  Falls back to np.empty when no block can be had.
    """
    import numpy as np

    dtype = np.dtype(dtype)
    count = math.prod(shape)
    nbytes = count * dtype.itemsize
    L = lib()
    ptr = L.rlic_host_buffer_alloc(max(nbytes, 1))
    if not ptr:
        return np.empty(shape, dtype=dtype)
    buf = (ctypes.c_char * max(nbytes, 1)).from_address(ptr)
    free = L.rlic_host_buffer_free
    weakref.finalize(buf, free, ctypes.c_void_p(ptr))
    arr = np.frombuffer(buf, dtype=dtype, count=count).reshape(shape)
    return arr


def launch_count() -> int:
    """Kernels this library has launched since it was loaded."""
    return int(lib().rlic_kernel_launch_count())


def set_block_shape(block_x: int, block_y: int) -> None:
    check(lib().rlic_set_block_shape(block_x, block_y))


def set_split_pixels(max_pixels: int) -> None:
    """Images of at most max_pixels trace each pixel's two half-streamlines on
    two threads (0: never; -1: the library's default threshold)."""
    check(lib().rlic_set_split_pixels(max_pixels))


def set_replay_mode(mode: int, stage_rows: int = 0) -> None:
    """RLIC_REPLAY_AUTO, _L1 or _STAGED for the replayed passes (bit-identical)."""
    check(lib().rlic_set_replay_mode(mode, stage_rows))
