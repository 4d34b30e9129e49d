"""The paired traced pass: each pixel's two half-streamlines on two threads.

Images of at most ``rlic_set_split_pixels`` pixels trace every traced pass
with lanes 0-15 of a warp on the forward halves of 16 pixels and lanes 16-31
on their backward halves; the backward lanes hand their samples over through
shared memory and the forward lanes add them in the reference's order
(centre, forward taps ascending, backward taps descending, src/lib.rs:376-403).
The result must be the one-thread-per-pixel pass's bits and the oracle's:
both dtypes, both uv modes, closed, periodic and mixed edges, odd and even
kernel lengths (the forward half is one step shorter for even lengths), NaN
stops on either half, tiles cut by the image edge, the path cache recorded by
the paired pass and replayed, the host-memory path, CTA shapes other than the
default, and launches that do not fit the form (they keep one thread per
pixel).
"""

from __future__ import annotations

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300 import _native

pytestmark = pytest.mark.gpu

BOUNDS = ["closed", "periodic", {"x": "periodic", "y": "closed"},
          {"x": "closed", "y": "periodic"}]
ALL = 1 << 40  # every image takes the paired pass


@pytest.fixture
def restore_knobs():
    yield
    _native.set_split_pixels(-1)
    _native.set_block_shape(0, 0)


def _field(ny, nx, dtype, seed, nans=False):
    rng = np.random.default_rng(seed)
    tex = rng.random((ny, nx)).astype(dtype)
    u = (rng.random((ny, nx)) - 0.5).astype(dtype)
    v = (rng.random((ny, nx)) - 0.5).astype(dtype)
    u[rng.random((ny, nx)) < 0.02] = 0.0
    v[u == 0.0] = 0.0
    if nans:
        u[rng.random((ny, nx)) < 0.003] = np.nan
    return tex, u, v


def _device_run(tex, u, v, k, mode, bnd, iters, split):
    import torch

    _native.set_split_pixels(split)
    t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (tex, u, v, k)]
    out = rlic_gb300.convolve(t[0], t[1], t[2], kernel=t[3], uv_mode=mode, boundaries=bnd,
                              iterations=iters)
    return out.cpu().numpy()


def _same_bits(a, b):
    it = np.uint32 if a.dtype == np.float32 else np.uint64
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all((a.view(it) == b.view(it)) | both_nan))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("mode", ["velocity", "polarization"])
@pytest.mark.parametrize("bnd", BOUNDS, ids=str)
def test_paired_equals_single_thread_pass_and_oracle(oracle, restore_knobs, dtype, mode,
                                                     bnd) -> None:
    tex, u, v = _field(150, 172, dtype, seed=17, nans=True)
    for klen in (3, 4, 31, 64):
        k = np.hanning(klen + 2)[1:-1].astype(dtype)
        for iters in (1, 3):
            got = _device_run(tex, u, v, k, mode, bnd, iters, ALL)
            ref = _device_run(tex, u, v, k, mode, bnd, iters, 0)
            assert _same_bits(got, ref), (klen, iters)
            want = oracle.convolve(tex, u, v, k, uv_mode=mode, boundaries=bnd,
                                   iterations=iters)
            assert _same_bits(got, want), (klen, iters)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_paired_readme_field_every_kernel_length(oracle, restore_knobs, dtype) -> None:
    """The README field (256^2, periodic) with long kernels, including one
    longer than the image (129 and 301 taps: streamlines wrap around)."""
    from rlic_gb300.workloads import readme_case

    c = readme_case()
    tex = c["texture"].astype(dtype)
    u = np.ascontiguousarray(c["u"], dtype=dtype)
    v = np.ascontiguousarray(c["v"], dtype=dtype)
    for klen in (5, 65, 129, 301):
        k = (1.0 - np.abs(np.linspace(-1, 1, klen))).astype(dtype)
        got = _device_run(tex, u, v, k, "velocity", "periodic", 1, ALL)
        want = oracle.convolve(tex, u, v, k, boundaries="periodic", iterations=1)
        assert _same_bits(got, want), klen


@pytest.mark.parametrize("shape", [(1, 1), (1, 40), (40, 1), (17, 3), (3, 33)])
@pytest.mark.parametrize("klen", [1, 2, 3, 5, 65])
def test_paired_degenerate_shapes(oracle, restore_knobs, shape, klen) -> None:
    """Images narrower than a tile: the threads of absent pixels still take
    part in the warp's shuffle."""
    tex, u, v = _field(*shape, np.float64, seed=klen)
    k = np.linspace(0.1, 1.0, klen)
    for bnd in ("closed", "periodic"):
        got = _device_run(tex, u, v, k, "polarization", bnd, 2, ALL)
        want = oracle.convolve(tex, u, v, k, uv_mode="polarization", boundaries=bnd,
                               iterations=2)
        assert _same_bits(got, want), bnd


@pytest.mark.parametrize("block", [(4, 4), (16, 1), (8, 2), (16, 4), (32, 2), (64, 4)],
                         ids=str)
def test_paired_block_shapes(oracle, restore_knobs, block) -> None:
    """Tiles of 16, 32 and 64 pixels in several shapes; 64 x 4 (256 pixels)
    does not fit the paired form and keeps one thread per pixel."""
    tex, u, v = _field(83, 97, np.float32, seed=5, nans=True)
    k = np.hanning(33).astype(np.float32)
    _native.set_block_shape(*block)
    got = _device_run(tex, u, v, k, "polarization", {"x": "periodic", "y": "closed"}, 3, ALL)
    want = oracle.convolve(tex, u, v, k, uv_mode="polarization",
                           boundaries={"x": "periodic", "y": "closed"}, iterations=3)
    assert _same_bits(got, want)


def test_paired_larger_image(oracle, restore_knobs) -> None:
    """A 600 x 700 float32 image, mostly interior tiles (no boundary logic,
    NaN-free steps), through the paired pass."""
    from rlic_gb300.workloads import fourier_vortex_case

    c = fourier_vortex_case(n=640, as_numpy=True, iterations=2)
    tex, u, v = (c[key][:600, :] for key in ("texture", "u", "v"))
    got = _device_run(tex, u, v, c["kernel"], c["uv_mode"], c["boundaries"], 2, ALL)
    ref = _device_run(tex, u, v, c["kernel"], c["uv_mode"], c["boundaries"], 2, 0)
    assert _same_bits(got, ref)
    want = oracle.convolve(np.ascontiguousarray(tex), np.ascontiguousarray(u),
                           np.ascontiguousarray(v), c["kernel"], uv_mode=c["uv_mode"],
                           boundaries=c["boundaries"], iterations=2,
                           nthreads=oracle.env_threads())
    assert _same_bits(got, want)


def test_paired_through_host_arrays(oracle, restore_knobs) -> None:
    """The README case from numpy arrays (broadcast u, v read in place) with
    the paired pass: the host path's traced launches take it too."""
    from rlic_gb300.workloads import readme_case

    c = readme_case()
    _native.set_split_pixels(ALL)
    for iters in (1, 2):
        got = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"],
                                  boundaries="periodic", iterations=iters)
        want = oracle.convolve(c["texture"], c["u"], c["v"], c["kernel"], boundaries="periodic",
                               iterations=iters)
        assert _same_bits(got, want), iters


def test_paired_sweep_records_the_same_path_cache(restore_knobs) -> None:
    """rlic_sweep_f64's output and path cache recorded by the paired pass
    equal those recorded with one thread per pixel, word for word."""
    import ctypes

    import torch

    lib = _native.lib()
    ny, nx, klen = 96, 80, 41
    tex, u, v = _field(ny, nx, np.float64, seed=9, nans=True)
    t = [torch.from_numpy(a).cuda() for a in (tex, u, v, np.hanning(klen))]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    uv = torch.empty((ny, nx, 2), dtype=torch.float64, device="cuda")
    _native.check(lib.rlic_pack_field_f64(t[1].data_ptr(), t[2].data_ptr(), ny, nx,
                                          uv.data_ptr(), stream))
    results = []
    for split in (ALL, 0):
        _native.set_split_pixels(split)
        out = torch.empty_like(t[0])
        codes = torch.zeros(lib.rlic_path_code_bytes(ny, nx, klen), dtype=torch.uint8,
                            device="cuda")
        _native.check(lib.rlic_sweep_f64(t[0].data_ptr(), uv.data_ptr(), ny, nx, t[3].data_ptr(),
                                         klen, 1, 0, 0, 1, 1, out.data_ptr(), codes.data_ptr(),
                                         stream, 0))
        torch.cuda.synchronize()
        results.append((out, codes))
    assert torch.equal(results[0][1], results[1][1])
    assert torch.equal(results[0][0].view(torch.int64), results[1][0].view(torch.int64))


def test_paired_with_chunked_host_upload(oracle, restore_knobs) -> None:
    """A host call of 4 Mpx and more uploads in row chunks and launches the
    traced pass per group of tile rows, alternating two streams; with 8 x 8
    CTAs and the paired threshold raised, those launches take the paired
    form.  Same bits as the device-resident one-thread pass and the oracle,
    across a periodic y seam (the last chunk goes first)."""
    import torch

    rng = np.random.default_rng(21)
    ny, nx = 2101, 2050
    tex = rng.random((ny, nx), dtype=np.float32)
    u = (rng.random((ny, nx)) - 0.5).astype(np.float32)
    v = (rng.random((ny, nx)) - 0.5).astype(np.float32)
    k = np.hanning(15).astype(np.float32)
    bnd = {"x": "closed", "y": "periodic"}
    kw = dict(uv_mode="polarization", boundaries=bnd, iterations=2)
    _native.set_split_pixels(0)
    want = rlic_gb300.convolve(torch.from_numpy(tex).cuda(), torch.from_numpy(u).cuda(),
                               torch.from_numpy(v).cuda(), kernel=torch.from_numpy(k).cuda(),
                               **kw).cpu().numpy()
    _native.set_block_shape(8, 8)
    _native.set_split_pixels(ALL)
    got = rlic_gb300.convolve(tex, u, v, kernel=k, **kw)
    assert _same_bits(got, want)
    full = oracle.convolve(tex, u, v, k, uv_mode="polarization", boundaries=bnd, iterations=2,
                           nthreads=oracle.env_threads())
    assert _same_bits(got, full)
