"""Replayed passes with the texture staged in shared memory by TMA copies.

RLIC_REPLAY_STAGED replays each super-tile of pixels from a box of cells
copied into shared memory (cp.async.bulk.tensor); boxes across a periodic
edge, and images that do not fit the form, replay through L1.  Both forms
must give the same bits, and the same bits as the oracle: closed, periodic
and mixed edges, images that are not a whole number of super-tiles, rows
that are not a multiple of 16 bytes (the whole call then falls back), NaN
stops, kernels whose box is at the copy limit or beyond it, both dtypes,
and the replay entry point, which does not know the recording's boundaries.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300 import _native

pytestmark = pytest.mark.gpu

BOUNDS = ["closed", "periodic", {"x": "periodic", "y": "closed"},
          {"x": "closed", "y": "periodic"}]


@pytest.fixture
def staged():
    _native.set_replay_mode(_native.RLIC_REPLAY_STAGED)
    yield
    _native.set_replay_mode(_native.RLIC_REPLAY_AUTO)


def _field(ny, nx, dtype, seed, nans=False):
    rng = np.random.default_rng(seed)
    tex = rng.random((ny, nx)).astype(dtype)
    u = (rng.random((ny, nx)) - 0.5).astype(dtype)
    v = (rng.random((ny, nx)) - 0.5).astype(dtype)
    u[rng.random((ny, nx)) < 0.02] = 0.0
    v[u == 0.0] = 0.0
    if nans:
        u[rng.random((ny, nx)) < 0.002] = np.nan
    return tex, u, v


def _run(tex, u, v, k, bnd, iters, mode, rows=0):
    import torch

    _native.set_replay_mode(mode, rows)
    t = [torch.from_numpy(a).cuda() for a in (tex, u, v, k)]
    out = rlic_gb300.convolve(t[0], t[1], t[2], kernel=t[3], uv_mode="polarization",
                              boundaries=bnd, iterations=iters)
    return out.cpu().numpy()


def _same_bits(a, b):
    it = np.uint32 if a.dtype == np.float32 else np.uint64
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all((a.view(it) == b.view(it)) | both_nan))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("bnd", BOUNDS, ids=str)
@pytest.mark.parametrize("shape", [(200, 328), (97, 256), (130, 132), (60, 130)])
def test_staged_equals_l1_and_oracle(oracle, staged, dtype, bnd, shape) -> None:
    ny, nx = shape
    tex, u, v = _field(ny, nx, dtype, seed=ny + nx)
    k = np.hanning(33).astype(dtype)
    got = _run(tex, u, v, k, bnd, 3, _native.RLIC_REPLAY_STAGED)
    ref = _run(tex, u, v, k, bnd, 3, _native.RLIC_REPLAY_L1)
    assert _same_bits(got, ref)
    want = oracle.convolve(tex, u, v, k, uv_mode="polarization", boundaries=bnd, iterations=3,
                           nthreads=oracle.env_threads())
    assert _same_bits(got, want)


@pytest.mark.parametrize("klen", [2, 9, 64, 65, 129, 191])
@pytest.mark.parametrize("rows", [4, 32, 64])
def test_staged_kernel_lengths_and_tile_heights(staged, klen, rows) -> None:
    # 129 and 191 taps: boxes of 192 and 256 cells a side, most of them
    # beyond the shared memory that leaves two CTAs per SM (the call then
    # replays through L1)
    for dtype in (np.float32, np.float64):
        tex, u, v = _field(300, 264, dtype, seed=klen, nans=True)
        k = (1 - np.abs(np.linspace(-1, 1, klen + 2)[1:-1])).astype(dtype)
        got = _run(tex, u, v, k, {"x": "closed", "y": "closed"}, 2,
                   _native.RLIC_REPLAY_STAGED, rows)
        ref = _run(tex, u, v, k, {"x": "closed", "y": "closed"}, 2, _native.RLIC_REPLAY_L1)
        assert _same_bits(got, ref), (klen, rows, dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_replay_entry_point_staged(staged, dtype) -> None:
    """rlic_replay_* does not know the boundaries the codes were recorded
    with, so the staged form must not stage boxes across any edge (periodic
    wraps are in the codes); RLIC_FLAG_FIELD_NAN_FREE skips the stop tests."""
    import torch

    lib = _native.lib()
    ny, nx, klen = 160, 200, 33
    tex, u, v = (torch.from_numpy(a).cuda() for a in _field(ny, nx, dtype, seed=5))
    k = torch.from_numpy(np.hanning(klen).astype(dtype)).cuda()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    sfx = "f32" if dtype == np.float32 else "f64"
    uv = torch.empty((ny, nx, 2), dtype=tex.dtype, device="cuda")
    _native.check(getattr(lib, f"rlic_pack_field_{sfx}")(u.data_ptr(), v.data_ptr(), ny, nx,
                                                          uv.data_ptr(), sp))
    codes = torch.empty(lib.rlic_path_code_bytes(ny, nx, klen), dtype=torch.uint8, device="cuda")
    first = torch.empty_like(tex)
    _native.check(getattr(lib, f"rlic_sweep_{sfx}")(
        tex.data_ptr(), uv.data_ptr(), ny, nx, k.data_ptr(), klen, 1, 1, 1, 1, 1,
        first.data_ptr(), codes.data_ptr(), sp, 0))
    outs = {}
    for mode in (_native.RLIC_REPLAY_L1, _native.RLIC_REPLAY_STAGED):
        for flags in (0, _native.RLIC_FLAG_FIELD_NAN_FREE):
            _native.set_replay_mode(mode)
            out = torch.full_like(tex, float("nan"))
            _native.check(getattr(lib, f"rlic_replay_{sfx}")(
                first.data_ptr(), codes.data_ptr(), ny, nx, k.data_ptr(), klen, out.data_ptr(),
                sp, flags))
            outs[(mode, flags)] = out
    torch.cuda.synchronize()
    ref = outs[(_native.RLIC_REPLAY_L1, 0)]
    want = rlic_gb300.convolve(tex, u, v, kernel=k, uv_mode="polarization",
                               boundaries="periodic", iterations=2)
    assert torch.equal(ref, want)
    for key, out in outs.items():
        assert torch.equal(out, ref), key


def test_staged_on_the_benchmark_field(staged) -> None:
    """8192^2 float32, Hann-65, polarization, x periodic / y closed, 5
    passes: the staged replays give the bits of the L1 replays."""
    import torch

    from rlic_gb300.workloads import fourier_vortex_case

    c = fourier_vortex_case(n=8192, device="cuda", as_numpy=False)
    kw = dict(kernel=c["kernel"], uv_mode=c["uv_mode"], boundaries=c["boundaries"],
              iterations=5)
    _native.set_replay_mode(_native.RLIC_REPLAY_STAGED)
    got = rlic_gb300.convolve(c["texture"], c["u"], c["v"], **kw)
    _native.set_replay_mode(_native.RLIC_REPLAY_L1)
    ref = rlic_gb300.convolve(c["texture"], c["u"], c["v"], **kw)
    assert torch.equal(got.view(torch.int32), ref.view(torch.int32))
    assert _native.lib().rlic_stage_timeouts() == 0


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("bnd", ["closed", {"x": "periodic", "y": "closed"}], ids=str)
@pytest.mark.parametrize("shape", [(120, 200), (90, 134)])
def test_staged_reduced_precision_replay(storage, dtype, bnd, shape) -> None:
    """The FP16/BF16-storage form replays from TMA-staged boxes of 2-byte
    cells (compensated FP32 sums in the traced pass's order): the same bits
    as its L1 replay, NaN stops included.  134 columns are not a whole
    number of 16-byte rows of 2-byte cells, so that call uses L1 throughout."""
    from rlic_gb300.forms import convolve_lowp

    tex, u, v = _field(*shape, dtype, seed=23, nans=True)
    k = (1 - np.abs(np.linspace(-1, 1, 41))).astype(dtype)
    kw = dict(kernel=k, uv_mode="polarization", boundaries=bnd, iterations=3, storage=storage)
    try:
        _native.set_replay_mode(_native.RLIC_REPLAY_STAGED)
        got = convolve_lowp(tex, u, v, **kw)
        _native.set_replay_mode(_native.RLIC_REPLAY_L1)
        want = convolve_lowp(tex, u, v, **kw)
    finally:
        _native.set_replay_mode(_native.RLIC_REPLAY_AUTO)
    assert _same_bits(got, want)
