"""Forms beyond the drop-in ``convolve``.

``convolve_autograd``: the differentiable form, a ``torch.autograd.Function``
whose forward is bit-identical to ``convolve`` and whose backward runs the
adjoint on the GPU: the transpose of every pass scatters the incoming
gradient back along the same recorded streamlines (d loss / d texture), and
a per-tap reduction gives d loss / d kernel.  u and v are not
differentiable: the streamline cells are discrete choices.

``ConvolvePlan``: one ``convolve`` call on CUDA tensors recorded into a
CUDA graph: the field's packing and every pass (the traced first pass, the
replayed passes ping-ponging between the output and a workspace buffer) in
one graph launch, for callers that convolve new textures over a fixed
field and configuration repeatedly.

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

__all__ = ["ConvolvePlan", "convolve_autograd", "convolve_lowp"]

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


# ------------------------------------------------------------ differentiable --

def _launch(fn, *args) -> None:
    _native.check(fn(*args))


class _ConvolveFunction:
    """Namespace for the torch.autograd.Function (built lazily: torch import)."""

    cls = None

    @classmethod
    def get(cls):
        if cls.cls is not None:
            return cls.cls
        import torch

        class ConvolveFunction(torch.autograd.Function):
            @staticmethod
            def forward(ctx, texture, kernel, u, v, uv_code, bcodes, iterations):
                lib = _native.lib()
                f32 = texture.dtype == torch.float32
                sfx = "f32" if f32 else "f64"
                ny, nx = texture.shape
                klen = kernel.shape[0]
                dev = texture.device
                stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
                uv = torch.empty((ny, nx, 2), dtype=texture.dtype, device=dev)
                codes = torch.empty(max(lib.rlic_path_code_bytes(ny, nx, klen), 4),
                                    dtype=torch.uint8, device=dev)
                _launch(getattr(lib, f"rlic_pack_field_{sfx}"), u.data_ptr(), v.data_ptr(), ny,
                        nx, uv.data_ptr(), stream)
                xs = [texture]
                first = torch.empty_like(texture)
                _launch(getattr(lib, f"rlic_sweep_{sfx}"), texture.data_ptr(), uv.data_ptr(), ny,
                        nx, kernel.data_ptr(), klen, uv_code, *bcodes, first.data_ptr(),
                        codes.data_ptr(), stream, 0)
                xs.append(first)
                for _ in range(1, iterations):
                    nxt = torch.empty_like(texture)
                    _launch(getattr(lib, f"rlic_replay_{sfx}"), xs[-1].data_ptr(),
                            codes.data_ptr(), ny, nx, kernel.data_ptr(), klen, nxt.data_ptr(),
                            stream, 0)
                    xs.append(nxt)
                ctx.save_for_backward(kernel, codes, *xs[:-1])
                ctx.iterations = iterations
                return xs[-1]

            @staticmethod
            def backward(ctx, grad_out):
                lib = _native.lib()
                kernel, codes, *xs = ctx.saved_tensors
                n = ctx.iterations
                f32 = grad_out.dtype == torch.float32
                sfx = "f32" if f32 else "f64"
                ny, nx = grad_out.shape
                klen = kernel.shape[0]
                dev = grad_out.device
                stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
                need_tex, need_k = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
                g = grad_out.contiguous()
                dw = torch.zeros(klen, dtype=torch.float64, device=dev)
                for m in range(n):
                    if need_k:
                        _launch(getattr(lib, f"rlic_kernel_grad_{sfx}"), g.data_ptr(),
                                xs[n - 1 - m].data_ptr(), codes.data_ptr(), ny, nx, klen,
                                dw.data_ptr(), stream, 0)
                    if need_tex or m < n - 1:
                        y = torch.empty_like(g)
                        _launch(getattr(lib, f"rlic_adjoint_{sfx}"), g.data_ptr(),
                                codes.data_ptr(), ny, nx, kernel.data_ptr(), klen, y.data_ptr(),
                                stream, 0)
                        g = y
                grad_tex = g if need_tex else None
                grad_k = dw.to(kernel.dtype) if need_k else None
                return grad_tex, grad_k, None, None, None, None, None

        cls.cls = ConvolveFunction
        return ConvolveFunction


def convolve_autograd(
    texture: Any,
    /,
    u: Any,
    v: Any,
    *,
    kernel: Any,
    uv_mode: str = "velocity",
    boundaries: Any = "closed",
    iterations: int = 1,
) -> Any:
    """Differentiable ``convolve`` on torch CUDA tensors.

    Same arguments, validation and (bit-identical) result as ``convolve``;
    gradients flow to ``texture`` and ``kernel``.  d loss / d texture
    accumulates with atomics, so its last bits vary from run to run.
    """
    import torch

    if not _is_torch(texture):
        raise TypeError("convolve_autograd takes torch CUDA tensors")
    _, bs = _validated(texture, u, v, kernel, uv_mode, boundaries, iterations)
    if iterations == 0:
        return texture.clone()
    dev = texture.device
    if dev.type != "cuda":
        raise ValueError("convolve_autograd takes CUDA tensors")
    u_c, v_c = (a.detach().to(device=dev).contiguous() for a in (u, v))
    with torch.cuda.device(dev):
        return _ConvolveFunction.get().apply(
            texture.contiguous(), kernel.to(device=dev).contiguous(), u_c, v_c,
            _native.UV_MODE_CODES[uv_mode], bs.codes(), iterations,
        )


# ------------------------------------------------------------- graph plan --

class ConvolvePlan:
    """``convolve`` on torch CUDA tensors, recorded into one CUDA graph.

    The plan validates its arguments once, with ``convolve``'s rules and
    messages, and owns device buffers for the texture, u, v, the kernel,
    the output and the call's workspace.  ``run()`` launches the call on
    the current stream (``rlic_convolve_f32/_f64`` on device memory: the
    field's packing, the traced first pass, then the replayed passes,
    alternating between the output and a workspace buffer); ``capture()``
    records that call into a CUDA graph, and ``replay()`` re-runs it with
    one graph launch and returns the output tensor (the same tensor every
    time).  Between replays, write new values into ``plan.texture`` (or
    ``plan.u``, ``plan.v``) in place; shapes, dtype, kernel length, uv mode,
    boundaries and iterations are fixed.  New texture values are not
    checked for negative entries (the validation ran once).  The result is
    bit-identical to ``convolve`` on the same values.
    """

    def __init__(self, texture: Any, u: Any, v: Any, *, kernel: Any,
                 uv_mode: str = "velocity", boundaries: Any = "closed", iterations: int = 1):
        import torch

        use_torch, bs = _validated(texture, u, v, kernel, uv_mode, boundaries, iterations)
        if not use_torch:
            raise TypeError("ConvolvePlan takes torch CUDA tensors")
        dev = texture.device
        if dev.type != "cuda":
            raise ValueError("ConvolvePlan takes CUDA tensors")
        self.device = dev
        self.texture, self.u, self.v, self.kernel = (
            a.detach().to(device=dev).contiguous().clone() for a in (texture, u, v, kernel))
        self.iterations = int(iterations)
        self.out = torch.empty_like(self.texture)
        self.lib = _native.lib()
        f32 = self.texture.dtype == torch.float32
        self._fn = self.lib.rlic_convolve_f32 if f32 else self.lib.rlic_convolve_f64
        ny, nx = self.texture.shape
        klen = self.kernel.shape[0]
        nbytes = self.lib.rlic_workspace_bytes(ny, nx, klen, max(self.iterations, 1),
                                               4 if f32 else 8, 0)
        self.workspace = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
        self._args = (ny, nx, klen, _native.UV_MODE_CODES[uv_mode], bs.codes(), nbytes)
        self.graph = None

    def run(self) -> Any:
        """Launch the call on the current stream; returns the output tensor."""
        import torch

        ny, nx, klen, uv_code, bcodes, nbytes = self._args
        if self.iterations == 0:  # the texture itself, as convolve returns a copy
            self.out.copy_(self.texture)
            return self.out
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        _native.check(self._fn(
            self.texture.data_ptr(), self.u.data_ptr(), self.v.data_ptr(), ny, nx,
            self.kernel.data_ptr(), klen, uv_code, *bcodes, self.iterations, self.out.data_ptr(),
            self.workspace.data_ptr(), nbytes, stream, 0))
        return self.out

    def capture(self) -> None:
        """Record the call into a CUDA graph (replay() re-runs it).  One run
        on the current stream first sets up everything a first call does."""
        import torch

        with torch.cuda.device(self.device):
            self.run()
            torch.cuda.synchronize(self.device)
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.stream(side), torch.cuda.graph(graph, stream=side):
                self.run()
            torch.cuda.current_stream(self.device).wait_stream(side)
        self.graph = graph

    def replay(self) -> Any:
        """Re-run the recorded call; returns the output tensor."""
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()
        return self.out
