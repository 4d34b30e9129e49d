"""Forms beyond the drop-in ``convolve``.

``convolve_lowp``: the reduced-precision form.  Streamline cells are traced
in the input dtype (float64 inputs keep a float64 advance), then the texture
and every buffer between passes are stored as FP16 or BF16 and each pass
accumulates in FP32 with compensated (Kahan) summation, storing its output
divided by sum(|kernel|); the scale is restored once at the end.  Results
approximate ``convolve`` (no counterpart in the reference).

Both take and return numpy arrays or torch CUDA tensors like ``convolve``
and validate their inputs with the same rules and messages.
"""

from __future__ import annotations

__all__ = ["convolve_lowp"]

import ctypes
from typing import Any

import numpy as np

from rlic_gb300 import _native
from rlic_gb300._lib import _collect_problems, _is_torch, _Ops

_STORAGES = {"fp16": _native.RLIC_STORAGE_FP16, "bf16": _native.RLIC_STORAGE_BF16}


def _validated(texture, u, v, kernel, uv_mode, boundaries, iterations):
    use_torch = _is_torch(texture)
    problems, bs = _collect_problems(
        _Ops(use_torch), texture, u, v, kernel, uv_mode, boundaries, iterations
    )
    if len(problems) == 1:
        raise problems[0]
    if problems:
        raise ExceptionGroup("Invalid inputs were received.", problems)
    return use_torch, bs


def _to_device(arrays, use_torch):
    import torch

    if use_torch:
        dev = arrays[0].device
        if dev.type != "cuda":
            raise ValueError("torch inputs must be CUDA tensors")
        return [a.to(device=dev).contiguous() for a in arrays]
    dev = torch.device("cuda", torch.cuda.current_device())
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrays]


def convolve_lowp(
    texture: Any,
    /,
    u: Any,
    v: Any,
    *,
    kernel: Any,
    uv_mode: str = "velocity",
    boundaries: Any = "closed",
    iterations: int = 1,
    storage: str = "fp16",
) -> Any:
    """Line integral convolution with 16-bit storage between passes.

    Same arguments and validation as ``convolve``, plus ``storage`` ("fp16"
    or "bf16").  Returns an array of the input dtype: numpy for numpy
    inputs, a CUDA tensor for tensor inputs.
    """
    import torch

    if storage not in _STORAGES:
        raise ValueError(f"Invalid storage {storage!r}. Expected one of {list(_STORAGES)}")
    use_torch, bs = _validated(texture, u, v, kernel, uv_mode, boundaries, iterations)
    if iterations == 0:
        return texture.clone() if use_torch else texture.copy()
    tex, uu, vv, k = _to_device([texture, u, v, kernel], use_torch)
    lib = _native.lib()
    ny, nx = tex.shape
    out = torch.empty_like(tex)
    elem = tex.element_size()
    nbytes = lib.rlic_lowp_workspace_bytes(ny, nx, k.shape[0], elem)
    with torch.cuda.device(tex.device):
        ws = torch.empty(nbytes, dtype=torch.uint8, device=tex.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(tex.device).cuda_stream)
        fn = lib.rlic_convolve_lowp_f32 if tex.dtype == torch.float32 else lib.rlic_convolve_lowp_f64
        _native.check(fn(
            tex.data_ptr(), uu.data_ptr(), vv.data_ptr(), ny, nx, k.data_ptr(), k.shape[0],
            _native.UV_MODE_CODES[uv_mode], *bs.codes(), iterations, _STORAGES[storage],
            out.data_ptr(), ws.data_ptr(), nbytes, stream, 0,
        ))
    if use_torch:
        return out
    return out.cpu().numpy()
