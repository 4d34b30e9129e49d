"""``convolve``: the drop-in public entry point.

Same signature, dtype rules, validation order and error texts as the
reference's ``rlic.convolve`` (src/rlic/_lib.py:37-235).  Every input check
runs first and all failures are collected; one failure is raised as is,
several are raised together as ``ExceptionGroup("Invalid inputs were
received.", ...)``.  ``iterations=0`` returns a copy of the texture after
validation (src/rlic/_lib.py:208-209).  Everything else runs on the GPU
through the C ABI of ``librlic_gb300.so``; there is no CPU fallback.

Inputs may be numpy arrays (the reference's contract: the result is a new
numpy array) or torch CUDA tensors (the result is a new tensor on the same
device, computed on the current torch stream, with no host round trip).
"""

from __future__ import annotations

__all__ = ["convolve"]

import ctypes
from typing import TYPE_CHECKING, Any

import numpy as np

from rlic_gb300 import _native
from rlic_gb300._boundaries import BoundarySet

if TYPE_CHECKING:
    from rlic_gb300._boundaries import BoundarySpec
    from rlic_gb300._typing import FArray1D, FArray2D, UVMode

_KNOWN_UV_MODES = ["velocity", "polarization"]
_SUPPORTED_DTYPES: list[np.dtype[np.floating]] = [
    np.dtype("float32"),
    np.dtype("float64"),
]


def _is_torch(x: Any) -> bool:
    return type(x).__module__.split(".")[0] == "torch"


class _Ops:
    """The few array operations validation needs, for numpy or torch."""

    def __init__(self, use_torch: bool) -> None:
        self.torch = use_torch
        if use_torch:
            import torch

            self._t = torch
            self.supported = [torch.float32, torch.float64]
        else:
            self.supported = _SUPPORTED_DTYPES

    def shape(self, a: Any) -> tuple[int, ...]:
        return tuple(a.shape)

    def any_negative(self, a: Any) -> bool:
        if self.torch:
            return bool((a < 0).any())
        return bool((a < 0).any())

    def any_nonfinite(self, a: Any) -> bool:
        if self.torch:
            return bool((~self._t.isfinite(a)).any())
        return not np.isfinite(a).all()

    def scans(self, texture: Any, kernel: Any, check_negative: bool) -> tuple[bool, bool]:
        """(any texture element < 0, any kernel element non-finite).  For
        tensors on one device both reductions come back to the host in one
        transfer (one synchronisation instead of two)."""
        if not self.torch:
            neg = self.any_negative(texture) if check_negative else False
            return neg, self.any_nonfinite(kernel)
        parts = [(texture < 0).any()] if check_negative else []
        parts.append((~self._t.isfinite(kernel)).any())
        if len({p.device for p in parts}) == 1:
            vals = [bool(x) for x in self._t.stack(parts).tolist()]
        else:
            vals = [bool(p) for p in parts]
        return (vals[0] if check_negative else False), vals[-1]


_NEGATIVE_TEXTURE = "Found invalid texture element(s). Expected only positive values."


def _collect_problems(
    ops: _Ops,
    texture: Any,
    u: Any,
    v: Any,
    kernel: Any,
    uv_mode: Any,
    boundaries: Any,
    iterations: int,
    check_negative: bool = True,
) -> tuple[list[Exception], BoundarySet | None]:
    """All validation failures, in the reference's order (src/rlic/_lib.py:135-200).

    With check_negative=False the scan for negative texture elements is left
    out (the caller then has it done on the GPU).
    """
    problems: list[Exception] = []
    if iterations < 0:
        problems.append(
            ValueError(
                f"Invalid number of iterations: {iterations}\n"
                "Expected a strictly positive integer."
            )
        )
    if uv_mode not in _KNOWN_UV_MODES:
        problems.append(
            ValueError(f"Invalid uv_mode {uv_mode!r}. Expected one of {_KNOWN_UV_MODES}")
        )

    def expectation() -> str:  # built only when a dtype problem is reported
        return (
            "Expected texture, u, v and kernel with identical dtype, from "
            f"{ops.supported}. Got texture.dtype={texture.dtype!r}, u.dtype={u.dtype!r}, "
            f"v.dtype={v.dtype!r}, kernel.dtype={kernel.dtype!r}"
        )

    dtypes = {a.dtype for a in (texture, u, v, kernel)}
    unsupported = dtypes.difference(ops.supported)
    if unsupported:
        problems.append(
            TypeError(f"Found unsupported data type(s): {list(unsupported)}. {expectation()}")
        )
    if len(dtypes) != 1:
        problems.append(TypeError(f"Data types mismatch. {expectation()}"))

    if texture.ndim != 2:
        problems.append(
            ValueError(f"Expected a texture with exactly two dimensions. Got texture.ndim={texture.ndim!r}")
        )
    negative, nonfinite_kernel = ops.scans(texture, kernel, check_negative)
    if negative:
        problems.append(ValueError(_NEGATIVE_TEXTURE))
    tshape, ushape, vshape = ops.shape(texture), ops.shape(u), ops.shape(v)
    if ushape != tshape or vshape != tshape:
        problems.append(
            ValueError(
                "Shape mismatch: expected texture, u and v with identical shapes. "
                f"Got texture.shape={tshape!r}, u.shape={ushape!r}, v.shape={vshape!r}"
            )
        )
    if kernel.ndim != 1:
        problems.append(
            ValueError(f"Expected a kernel with exactly one dimension. Got kernel.ndim={kernel.ndim!r}")
        )
    if nonfinite_kernel:
        problems.append(ValueError("Found non-finite value(s) in kernel."))

    bs = BoundarySet.from_spec(boundaries)
    if bs is None:
        problems.append(TypeError(f"Invalid boundary specification {boundaries}"))
    else:
        problems.extend(bs.collect_exceptions())
    return problems, bs


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _element_strides(a: np.ndarray) -> tuple[int, int] | None:
    """(row, column) strides in elements, or None when not whole elements."""
    its = a.itemsize
    if any(st % its for st in a.strides):
        return None
    return a.strides[0] // its, a.strides[1] // its


def _empty_result(shape: tuple[int, ...], dtype: np.dtype) -> np.ndarray:
    """The result for an image without pixels (a zero-length axis).

    The native core allocates its zero-filled output and its pixel loops
    run zero times, so any kernel, even an empty one, gives a new empty
    array of the input's shape (src/lib.rs:364-375, 424-442).
    """
    return np.zeros(shape, dtype=dtype)


def _convolve_numpy(
    texture: np.ndarray,
    u: np.ndarray,
    v: np.ndarray,
    kernel: np.ndarray,
    uv_code: int,
    bcodes: tuple[int, int, int, int],
    iterations: int,
    check_texture: bool = True,
) -> np.ndarray:
    """One call of the C ABI on host arrays.  With check_texture the GPU
    also scans the texture for negative elements (the reference's
    validation), and a negative texture raises ValueError."""
    lib = _native.lib()
    dtype = texture.dtype
    if texture.size == 0:
        return _empty_result(texture.shape, dtype)
    k_c = np.ascontiguousarray(kernel)
    ny, nx = texture.shape
    # a page-locked result buffer, reused once the caller drops an earlier one
    out = _native.pinned_empty((ny, nx), dtype)
    flags = _native.RLIC_FLAG_HOST_MEMORY
    if check_texture:
        flags |= _native.RLIC_FLAG_CHECK_TEXTURE
    f32 = dtype == np.dtype("float32")
    views = (texture, u, v)
    strides = None
    if not all(a.flags.c_contiguous for a in views):
        strides = [_element_strides(a) for a in views]
        if any(s is None for s in strides) or not lib.rlic_host_direct_access():
            strides = None
    if strides is not None:
        # strided views (broadcasts, transposes, slices) are read in place
        st = (ctypes.c_int64 * 6)(*(x for s in strides for x in s))
        fn = lib.rlic_convolve_strided_f32 if f32 else lib.rlic_convolve_strided_f64
        rc = fn(
            _ptr(texture), _ptr(u), _ptr(v), st, ny, nx, _ptr(k_c), k_c.shape[0], uv_code,
            *bcodes, iterations, _ptr(out), None, flags,
        )
    else:
        tex_c = np.ascontiguousarray(texture)
        u_c = np.ascontiguousarray(u)
        v_c = np.ascontiguousarray(v)
        fn = lib.rlic_convolve_f32 if f32 else lib.rlic_convolve_f64
        rc = fn(
            _ptr(tex_c), _ptr(u_c), _ptr(v_c), ny, nx, _ptr(k_c), k_c.shape[0], uv_code,
            *bcodes, iterations, _ptr(out), None, 0, None, flags,
        )
    if rc == _native.RLIC_ERR_NEGATIVE_TEXTURE or (
        rc != _native.RLIC_OK and check_texture and np.any(texture < 0)
    ):
        # the only problem left (every other check passed on the host); it
        # takes precedence over a failure of the native call, as validation
        # does in the reference
        raise ValueError(_NEGATIVE_TEXTURE)
    _native.check(rc)
    return out


def _convolve_torch(
    texture: Any,
    u: Any,
    v: Any,
    kernel: Any,
    uv_code: int,
    bcodes: tuple[int, int, int, int],
    iterations: int,
) -> Any:
    import torch

    lib = _native.lib()
    dev = texture.device
    if dev.type != "cuda" or u.device != dev or v.device != dev:
        raise ValueError(
            "torch inputs must be CUDA tensors on one device. "
            f"Got texture.device={texture.device}, u.device={u.device}, v.device={v.device}"
        )
    if texture.numel() == 0:
        return torch.zeros(tuple(texture.shape), dtype=texture.dtype, device=dev)
    with torch.cuda.device(dev):
        tex_c = texture.contiguous()
        u_c = u.contiguous()
        v_c = v.contiguous()
        k_c = kernel.to(device=dev).contiguous()
        out = torch.empty_like(tex_c, memory_format=torch.contiguous_format)
        ny, nx = tex_c.shape
        elem = tex_c.element_size()
        nbytes = lib.rlic_workspace_bytes(ny, nx, k_c.shape[0], iterations, elem, 0)
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        fn = lib.rlic_convolve_f32 if tex_c.dtype == torch.float32 else lib.rlic_convolve_f64
        rc = fn(
            tex_c.data_ptr(), u_c.data_ptr(), v_c.data_ptr(), ny, nx, k_c.data_ptr(),
            k_c.shape[0], uv_code, *bcodes, iterations, out.data_ptr(), ws.data_ptr(), nbytes,
            ctypes.c_void_p(stream), 0,
        )
        _native.check(rc)
    return out


def convolve(
    texture: FArray2D,
    /,
    u: FArray2D,
    v: FArray2D,
    *,
    kernel: FArray1D,
    uv_mode: UVMode = "velocity",
    boundaries: BoundarySpec = "closed",
    iterations: int = 1,
) -> FArray2D:
    """2-dimensional line integral convolution, on the GPU.

    Convolves ``texture`` along the streamlines of the vector field
    ``(u, v)`` with the 1-D ``kernel``: each output pixel is the
    kernel-weighted sum of texture samples met while tracing the streamline
    through that pixel forward (second half of the kernel) and backward
    (first half of the kernel).

    texture: 2-D array of non-negative values (positional only).
    u, v: 2-D arrays, the x (column) and y (row) components of the field.
    kernel: 1-D array of finite weights (keyword only).
    uv_mode: "velocity" (direction matters) or "polarization" (each sample
        is flipped to agree with the previous one, so direction is ignored).
    boundaries: "closed", "periodic", or {"x": spec, "y": spec} with each
        spec a name or a (left, right) pair; a periodic side must face a
        periodic side.
    iterations: number of passes, each fed with the previous output; 0
        returns a copy of the texture.

    All four arrays share one dtype, float32 or float64.  The result is a
    new array of that dtype and the inputs are never modified.  numpy inputs
    give a numpy result; torch CUDA tensors give a tensor on their device.

    Raises TypeError for mismatched or unsupported dtypes, ValueError for
    other invalid inputs, and an ExceptionGroup when several problems are
    found at once.  The results, messages and edge cases follow the
    reference (src/rlic/_lib.py:37-235, src/lib.rs:305-443).
    """
    use_torch = _is_torch(texture)
    ops = _Ops(use_torch)
    # numpy inputs: the scan for negative texture elements runs on the GPU
    # with the convolution (one pass over the uploaded texture instead of a
    # host pass); it runs here only when the call fails anyway or never
    # reaches the GPU, so the raised errors are always those of the reference
    deferred = not use_torch and iterations != 0
    problems, bs = _collect_problems(
        ops, texture, u, v, kernel, uv_mode, boundaries, iterations,
        check_negative=not deferred,
    )
    if deferred and problems:
        problems, bs = _collect_problems(
            ops, texture, u, v, kernel, uv_mode, boundaries, iterations
        )
    if len(problems) == 1:
        raise problems[0]
    if problems:
        raise ExceptionGroup("Invalid inputs were received.", problems)
    assert bs is not None

    if iterations == 0:
        return texture.clone() if use_torch else texture.copy()

    uv_code = _native.UV_MODE_CODES[uv_mode]
    bcodes = bs.codes()
    if use_torch:
        if not all(_is_torch(a) for a in (u, v, kernel)):
            raise TypeError("texture is a torch tensor: u, v and kernel must be tensors too")
        return _convolve_torch(texture, u, v, kernel, uv_code, bcodes, iterations)
    if any(_is_torch(a) for a in (u, v, kernel)):
        raise TypeError("texture is a numpy array: u, v and kernel must be numpy arrays too")
    return _convolve_numpy(texture, u, v, kernel, uv_code, bcodes, iterations)
