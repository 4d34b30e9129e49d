"""rlic_convolve_f32_noalloc: the entry point for callers that cannot allocate.

Some callers cannot allocate device memory: a plugin whose host application
owns the device-memory budget, code running inside another library's
allocator callback, or a latency-critical loop that cannot afford the
synchronisation cudaMalloc/cudaFree may cause.  For them the library offers
one variant of rlic_convolve_f32 whose scratch is a 64 MiB static device
array instead of an allocation.  These tests call it through the C ABI and
check that it returns exactly what the allocating entry point returns, on
two calls in a row (the second reusing the array the first one filled).

This file is named so that pytest collects it last; it passes on its own in
a fresh process as well.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from rlic_gb300 import _native

pytestmark = pytest.mark.gpu

NY, NX, KLEN = 300, 352, 33
BOUNDS = (1, 1, 0, 0)  # x periodic, y closed
POLARIZATION = 1


def _case(seed: int):
    import torch

    rng = np.random.default_rng(seed)
    u = (rng.random((NY, NX)) - 0.5).astype(np.float32)
    v = (rng.random((NY, NX)) - 0.5).astype(np.float32)
    u[rng.random((NY, NX)) < 0.02] = 0.0
    v[u == 0.0] = 0.0
    tex = rng.random((NY, NX)).astype(np.float32)
    k = np.hanning(KLEN).astype(np.float32)
    return [torch.from_numpy(a).cuda() for a in (tex, u, v, k)]


def _allocating(lib, tex, u, v, k, stream, iters, flags=0):
    import torch

    out = torch.empty_like(tex)
    nbytes = lib.rlic_workspace_bytes(NY, NX, KLEN, iters, 4, flags)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    _native.check(lib.rlic_convolve_f32(
        tex.data_ptr(), u.data_ptr(), v.data_ptr(), NY, NX, k.data_ptr(), KLEN, POLARIZATION,
        *BOUNDS, iters, out.data_ptr(), ws.data_ptr(), nbytes, stream, flags))
    return out


def _noalloc(lib, tex, u, v, k, stream, iters, flags=0):
    import torch

    out = torch.full_like(tex, float("nan"))
    _native.check(lib.rlic_convolve_f32_noalloc(
        tex.data_ptr(), u.data_ptr(), v.data_ptr(), NY, NX, k.data_ptr(), KLEN, POLARIZATION,
        *BOUNDS, iters, out.data_ptr(), stream, flags))
    return out


# 0 passes (the output is cleared), 1 pass (no ping-pong buffer, no path
# cache) and 3 passes (ping-pong buffer and, by default, the path cache)
@pytest.mark.parametrize("iters", [0, 1, 3])
@pytest.mark.parametrize("flags", [0, _native.RLIC_FLAG_NO_PATH_CACHE],
                         ids=["path-cache", "plain"])
def test_noalloc_matches_allocating_entry_point_twice(flags, iters) -> None:
    import torch

    lib = _native.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # two calls in a row on different inputs: the second finds the first
    # call's data in the static scratch and must not be affected by it
    for seed in (1, 2):
        tex, u, v, k = _case(seed)
        want = _allocating(lib, tex, u, v, k, stream, iters, flags)
        got = _noalloc(lib, tex, u, v, k, stream, iters, flags)
        torch.cuda.synchronize()
        # bit-exact, like every other parity check of this library
        assert torch.equal(got.view(torch.int32), want.view(torch.int32)), (seed, iters)


def test_noalloc_rejects_calls_beyond_its_scratch() -> None:
    lib = _native.lib()
    n = 4096  # 4096^2 float32, 5 passes: far beyond 64 MiB
    need = lib.rlic_workspace_bytes(n, n, 65, 5, 4, 0)
    assert need > _native.NOALLOC_SCRATCH_BYTES
    rc = lib.rlic_convolve_f32_noalloc(1, 1, 1, n, n, 1, 65, 0, 0, 0, 0, 0, 5, 1, None, 0)
    assert rc == _native.RLIC_ERR_WORKSPACE_TOO_SMALL
    msg = lib.rlic_last_error().decode()
    assert str(need) in msg and str(_native.NOALLOC_SCRATCH_BYTES) in msg
    # host memory and the texture check are refused before touching the GPU
    for flag in (_native.RLIC_FLAG_HOST_MEMORY, _native.RLIC_FLAG_CHECK_TEXTURE):
        rc = lib.rlic_convolve_f32_noalloc(1, 1, 1, 8, 8, 1, 5, 0, 0, 0, 0, 0, 1, 1, None, flag)
        assert rc == _native.RLIC_ERR_INVALID_ARGUMENT


def test_noalloc_zero_iterations_have_no_size_limit() -> None:
    import torch

    lib = _native.lib()
    n = 4096  # beyond the scratch for one or more passes, but 0 passes need none
    assert lib.rlic_workspace_bytes(n, n, 65, 1, 4, 0) > _native.NOALLOC_SCRATCH_BYTES
    x = torch.ones((n, n), dtype=torch.float32, device="cuda")
    k = torch.ones(65, dtype=torch.float32, device="cuda")
    out = torch.full_like(x, float("nan"))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _native.check(lib.rlic_convolve_f32_noalloc(
        x.data_ptr(), x.data_ptr(), x.data_ptr(), n, n, k.data_ptr(), 65, 0, 0, 0, 0, 0, 0,
        out.data_ptr(), stream, 0))
    torch.cuda.synchronize()
    assert int(torch.count_nonzero(out)) == 0
