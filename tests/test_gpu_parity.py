"""Bit-exact parity of the CUDA path with the oracle, through the C ABI.

The bar is bit-exact output (integer-exact streamline cells, identical
floating-point outputs): the device arithmetic reproduces every rounding of
the reference (src/lib.rs:157-406).  Cases cover the committed golden
vectors, the README workload, random fields with zeros / signed zeros /
NaNs / infinities, degenerate images, short, even and over-long kernels,
every boundary combination, both uv modes, several iterations and all four
Cargo feature variants.
"""

from __future__ import annotations

import ctypes
import zlib
from itertools import product
from pathlib import Path

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300 import _native
from rlic_gb300.workloads import fourier_vortex_case, readme_case

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CODES = {"closed": 0, "periodic": 1}


def _codes(bnd):
    if isinstance(bnd, str):
        return (CODES[bnd],) * 4
    if isinstance(bnd, dict):
        def pair(b):
            return (b, b) if isinstance(b, str) else tuple(b)
        bnd = (pair(bnd["x"]), pair(bnd["y"]))
    (xl, xr), (yl, yr) = bnd
    return tuple(CODES[b] for b in (xl, xr, yl, yr))


def _variant_flags(variant: int) -> int:
    flags = 0
    if not variant & 1:
        flags |= _native.RLIC_FLAG_NO_FMA
    if not variant & 2:
        flags |= _native.RLIC_FLAG_NO_BRANCHLESS
    return flags


def capi_convolve(tex, u, v, k, uv_mode="velocity", boundaries="closed", iterations=1,
                  variant=3, extra_flags=0):
    """rlic_convolve_* with host buffers (the call copies in and out)."""
    lib = _native.lib()
    dtype = np.asarray(tex).dtype
    tex, u, v, k = (np.ascontiguousarray(a, dtype=dtype) for a in (tex, u, v, k))
    out = np.full(tex.shape, np.nan, dtype=dtype)
    fn = lib.rlic_convolve_f32 if dtype == np.float32 else lib.rlic_convolve_f64
    ny, nx = tex.shape
    rc = fn(tex.ctypes.data, u.ctypes.data, v.ctypes.data, ny, nx, k.ctypes.data, k.size,
            int(uv_mode == "polarization"), *_codes(boundaries), iterations, out.ctypes.data,
            None, 0, None, _native.RLIC_FLAG_HOST_MEMORY | _variant_flags(variant) | extra_flags)
    _native.check(rc)
    return out


def capi_cells(u, v, klen, pix, uv_mode="velocity", boundaries="closed", variant=3):
    lib = _native.lib()
    dtype = np.asarray(u).dtype
    u, v = (np.ascontiguousarray(a, dtype=dtype) for a in (u, v))
    pix = np.ascontiguousarray(pix, dtype=np.int64)
    cells = np.full((pix.size, max(klen - 1, 0)), -7, dtype=np.int64)
    fn = lib.rlic_trace_cells_f32 if dtype == np.float32 else lib.rlic_trace_cells_f64
    ny, nx = u.shape
    rc = fn(u.ctypes.data, v.ctypes.data, ny, nx, klen, int(uv_mode == "polarization"),
            *_codes(boundaries), pix.size, pix.ctypes.data, cells.ctypes.data, None,
            _native.RLIC_FLAG_HOST_MEMORY | _variant_flags(variant))
    _native.check(rc)
    return cells


def assert_bitwise(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.dtype == b.dtype and a.shape == b.shape
    ia = a.view(np.uint32 if a.dtype == np.float32 else np.uint64)
    ib = b.view(np.uint32 if b.dtype == np.float32 else np.uint64)
    # NaN payloads differ between CPU architectures and the GPU: any NaN matches any NaN
    bad = np.flatnonzero((ia != ib) & ~(np.isnan(a) & np.isnan(b)))
    assert bad.size == 0, (
        f"{bad.size} of {a.size} elements differ; first at {np.unravel_index(bad[0], a.shape)}: "
        f"{a.ravel()[bad[0]]!r} vs {b.ravel()[bad[0]]!r}"
    )


# ------------------------------------------------------------- golden --

@pytest.mark.parametrize("path", sorted(GOLDEN.glob("*.npz")), ids=lambda p: p.stem)
def test_golden_vectors(path) -> None:
    g = np.load(path, allow_pickle=False)
    bnd = ((str(g["bx"][0]), str(g["bx"][1])), (str(g["by"][0]), str(g["by"][1])))
    out = capi_convolve(g["texture"], g["u"], g["v"], g["kernel"], str(g["uv_mode"]), bnd,
                        int(g["iterations"]), int(g["variant"]))
    assert_bitwise(out, g["out"])
    cells = capi_cells(g["u"], g["v"], g["kernel"].size, g["pix"], str(g["uv_mode"]), bnd,
                       int(g["variant"]))
    np.testing.assert_array_equal(cells, g["cells"])


# ------------------------------------------------------- README case --

def test_readme_case_output_and_every_path(oracle) -> None:
    c = readme_case()
    want = oracle.convolve(c["texture"], c["u"], c["v"], c["kernel"],
                           boundaries=c["boundaries"])
    got = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"],
                              boundaries=c["boundaries"])
    assert_bitwise(got, want)
    pix = np.arange(256 * 256)
    cells = capi_cells(c["u"], c["v"], 65, pix, boundaries="periodic")
    np.testing.assert_array_equal(cells, oracle.paths(c["u"], c["v"], 65, pix,
                                                      boundaries="periodic"))


# ----------------------------------------------------- random fields --

def _field(rng, ny, nx, dtype, kind):
    u = (rng.random((ny, nx)) - 0.5).astype(dtype)
    v = (rng.random((ny, nx)) - 0.5).astype(dtype)
    if kind == "specials":
        m = rng.random((ny, nx))
        u[m < 0.05] = 0.0
        v[m < 0.05] = 0.0
        u[(m > 0.05) & (m < 0.08)] = -0.0
        v[(m > 0.10) & (m < 0.12)] = 0.0
        v[(m > 0.12) & (m < 0.13)] = -0.0
        u[(m > 0.20) & (m < 0.205)] = np.nan
        v[(m > 0.30) & (m < 0.302)] = np.inf
        u[(m > 0.40) & (m < 0.402)] = -np.inf
        u[(m > 0.50) & (m < 0.52)] = np.finfo(dtype).tiny / 4  # subnormal
        v[(m > 0.60) & (m < 0.62)] = 1e30 if dtype == np.float32 else 1e300
    elif kind == "axis":
        # exact axis-aligned and diagonal flows exercise ties (tx == ty)
        u = np.where(rng.random((ny, nx)) < 0.5, 1.0, -1.0).astype(dtype)
        v = np.where(rng.random((ny, nx)) < 0.3, u, 0.0).astype(dtype)
    return u, v


BOUNDS = [
    "closed", "periodic", {"x": "periodic", "y": "closed"}, {"x": "closed", "y": "periodic"},
    # mixed sides: rejected by the Python layer, computed by the native core
    {"x": ("closed", "periodic"), "y": ("periodic", "closed")},
]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("uv_mode", ["velocity", "polarization"])
@pytest.mark.parametrize("bnd", BOUNDS, ids=lambda b: str(b).replace(" ", ""))
@pytest.mark.parametrize("kind", ["random", "specials", "axis"])
def test_random_fields(oracle, dtype, uv_mode, bnd, kind) -> None:
    rng = np.random.default_rng(zlib.crc32(f"{dtype}{uv_mode}{bnd}{kind}".encode()))
    ny, nx = 37, 53
    u, v = _field(rng, ny, nx, dtype, kind)
    tex = rng.random((ny, nx)).astype(dtype)
    k = rng.random(31).astype(dtype)
    want = oracle.convolve(tex, u, v, k, uv_mode=uv_mode, boundaries=bnd, iterations=3)
    got = capi_convolve(tex, u, v, k, uv_mode, bnd, iterations=3)  # path cache
    assert_bitwise(got, want)
    plain = capi_convolve(tex, u, v, k, uv_mode, bnd, iterations=3,
                          extra_flags=_native.RLIC_FLAG_NO_PATH_CACHE)
    assert_bitwise(plain, want)
    pix = np.arange(ny * nx)
    np.testing.assert_array_equal(
        capi_cells(u, v, 31, pix, uv_mode, bnd),
        oracle.paths(u, v, 31, pix, uv_mode=uv_mode, boundaries=bnd),
    )


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("where", ["none", "centre", "corner"])
def test_nan_free_fields_and_isolated_nans(oracle, dtype, where) -> None:
    """Interior tiles of a field without NaN samples skip the per-step NaN
    test; one NaN sample anywhere sends every step back to the checked path.
    Both must give the oracle's bits and cells."""
    rng = np.random.default_rng(21)
    ny, nx = 96, 160
    u, v = _field(rng, ny, nx, dtype, "random")
    if where == "centre":
        u[48, 80] = np.nan
    elif where == "corner":
        v[0, 0] = np.nan
    tex = rng.random((ny, nx)).astype(dtype)
    k = np.hanning(17).astype(dtype)
    for mode in ("velocity", "polarization"):
        want = oracle.convolve(tex, u, v, k, uv_mode=mode, boundaries="periodic", iterations=3)
        assert_bitwise(capi_convolve(tex, u, v, k, mode, "periodic", iterations=3), want)
        assert_bitwise(capi_convolve(tex, u, v, k, mode, "periodic", iterations=3,
                                     extra_flags=_native.RLIC_FLAG_NO_PATH_CACHE), want)


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("uv_mode", ["velocity", "polarization"])
def test_float64_near_ties_and_exponent_edges(oracle, variant, uv_mode) -> None:
    """float64 steps settle tx < ty from float32 cross products when they are
    2^-16 apart or more, and divide both times otherwise.  Fields with
    |u| = |v| (1 + e) for e around that margin and down to one ulp, and
    components at the edges of the screened exponent range (2^-61 .. 2^-59,
    2^59 .. 2^61), must still give the oracle's cells and bits."""
    rng = np.random.default_rng(7 + variant)
    ny, nx = 43, 57
    v = rng.uniform(0.2, 2.0, (ny, nx)) * rng.choice([-1.0, 1.0], (ny, nx))
    eps = rng.choice([0.0, 2.0**-52, -(2.0**-52), 2.0**-40, 2.0**-20, -(2.0**-20), 2.0**-17,
                      2.0**-16, -(2.0**-16), 2.0**-15, -(2.0**-15), 2.0**-10], (ny, nx))
    u = v * (1.0 + eps) * rng.choice([-1.0, 1.0], (ny, nx))
    m = rng.random((ny, nx))
    scale = np.where(m < 0.1, 2.0**-60, np.where(m < 0.2, 2.0**60, 1.0))
    scale *= np.where((m > 0.3) & (m < 0.35), 2.0**-61, 1.0)
    scale *= np.where((m > 0.4) & (m < 0.45), 2.0**61, 1.0)
    u, v = u * scale, v * scale
    u[(m > 0.5) & (m < 0.53)] *= 2.0**-1000  # subnormal-range partners
    tex = rng.random((ny, nx))
    k = rng.random(33)
    for bnd in ("closed", "periodic"):
        want = oracle.convolve(tex, u, v, k, uv_mode=uv_mode, boundaries=bnd, iterations=2,
                               variant=variant)
        assert_bitwise(capi_convolve(tex, u, v, k, uv_mode, bnd, 2, variant), want)
        assert_bitwise(capi_convolve(tex, u, v, k, uv_mode, bnd, 2, variant,
                                     _native.RLIC_FLAG_NO_PATH_CACHE), want)
        pix = np.arange(ny * nx)
        np.testing.assert_array_equal(
            capi_cells(u, v, 33, pix, uv_mode, bnd, variant),
            oracle.paths(u, v, 33, pix, uv_mode=uv_mode, boundaries=bnd, variant=variant),
        )


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_feature_variants(oracle, variant, dtype) -> None:
    rng = np.random.default_rng(100 + variant)
    u, v = _field(rng, 41, 29, dtype, "specials")
    tex = rng.random((41, 29)).astype(dtype)
    k = np.hanning(25).astype(dtype)
    for mode in ("velocity", "polarization"):
        want = oracle.convolve(tex, u, v, k, uv_mode=mode, boundaries="periodic",
                               iterations=2, variant=variant)
        got = capi_convolve(tex, u, v, k, mode, "periodic", 2, variant)
        assert_bitwise(got, want)
        plain = capi_convolve(tex, u, v, k, mode, "periodic", 2, variant,
                              _native.RLIC_FLAG_NO_PATH_CACHE)
        assert_bitwise(plain, want)


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (7, 1), (2, 2), (3, 130), (130, 3)])
@pytest.mark.parametrize("klen", [1, 2, 3, 4, 5, 64, 65, 301])
def test_degenerate_shapes_and_kernels(oracle, shape, klen) -> None:
    rng = np.random.default_rng(sum(shape) * 1000 + klen)
    u, v = _field(rng, *shape, np.float64, "specials")
    tex = rng.random(shape)
    k = rng.random(klen)
    for bnd, mode in product(["closed", "periodic"], ["velocity", "polarization"]):
        want = oracle.convolve(tex, u, v, k, uv_mode=mode, boundaries=bnd, iterations=3)
        got = capi_convolve(tex, u, v, k, mode, bnd, iterations=3)
        assert_bitwise(got, want)
        plain = capi_convolve(tex, u, v, k, mode, bnd, iterations=3,
                              extra_flags=_native.RLIC_FLAG_NO_PATH_CACHE)
        assert_bitwise(plain, want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("klen", [9, 33, 65])
def test_replay_interior_and_border_tiles(oracle, dtype, klen) -> None:
    """Images large enough that replays run both from staged shared-memory
    blocks (interior super-tiles) and from global memory (border ones)."""
    rng = np.random.default_rng(klen)
    ny, nx = 280, 344
    u, v = _field(rng, ny, nx, dtype, "specials")
    tex = rng.random((ny, nx)).astype(dtype)
    k = rng.random(klen).astype(dtype)
    for bnd, mode in (("periodic", "polarization"), ({"x": "closed", "y": "periodic"}, "velocity")):
        want = oracle.convolve(tex, u, v, k, uv_mode=mode, boundaries=bnd, iterations=3,
                               nthreads=oracle.env_threads())
        assert_bitwise(capi_convolve(tex, u, v, k, mode, bnd, iterations=3), want)


@pytest.mark.parametrize("iterations", [0, 1, 2, 3, 4])
def test_iteration_counts(oracle, iterations) -> None:
    rng = np.random.default_rng(iterations)
    u, v = _field(rng, 33, 35, np.float32, "random")
    tex = rng.random((33, 35)).astype(np.float32)
    k = np.hanning(17).astype(np.float32)
    want = oracle.convolve(tex, u, v, k, uv_mode="polarization", iterations=iterations)
    got = capi_convolve(tex, u, v, k, "polarization", "closed", iterations)
    assert_bitwise(got, want)  # iterations == 0: zeros, as the native core


def test_uniform_fields(oracle) -> None:
    for uu, vv in [(0.0, 0.0), (np.nan, np.nan), (1.0, 0.0), (0.0, -1.0), (1.0, 1.0),
                   (-0.0, -0.0), (3.0, -3.0), (np.inf, 1.0)]:
        u = np.full((20, 21), uu)
        v = np.full((20, 21), vv)
        tex = np.random.default_rng(5).random((20, 21))
        k = np.linspace(0.5, 1, 15)
        for bnd in ("closed", "periodic"):
            want = oracle.convolve(tex, u, v, k, boundaries=bnd, iterations=2)
            assert_bitwise(capi_convolve(tex, u, v, k, "velocity", bnd, 2), want)


# --------------------------------------------------- at-scale workload --

def test_fourier_vortex_1024_full(oracle) -> None:
    c = fourier_vortex_case(n=1024, device="cuda", iterations=2)
    want = oracle.convolve(c["texture"], c["u"], c["v"], c["kernel"], uv_mode=c["uv_mode"],
                           boundaries=c["boundaries"], iterations=2,
                           nthreads=oracle.env_threads())
    got = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"],
                              uv_mode=c["uv_mode"], boundaries=c["boundaries"], iterations=2)
    assert_bitwise(got, want)


def test_fourier_vortex_full_size_properties(oracle) -> None:
    """8192^2 float32, K=65, 5 iterations: too large for the oracle in full,
    so: (1) the first pass of sampled row bands equals the oracle's rows;
    (2) sampled pixels' streamline cells equal the oracle's; (3) five
    iterations equal five chained single passes, bit for bit."""
    import torch

    c = fourier_vortex_case(n=8192, device="cuda", as_numpy=False)
    tex, u, v, k = c["texture"], c["u"], c["v"], c["kernel"]
    kw = dict(kernel=k, uv_mode=c["uv_mode"], boundaries=c["boundaries"])
    one = rlic_gb300.convolve(tex, u, v, iterations=1, **kw)
    un, vn, tn, kn = (a.cpu().numpy() for a in (u, v, tex, k))
    onen = one.cpu().numpy()
    for r0 in (0, 4093, 8192 - 6):
        rows = oracle.sweep_rows(tn, un, vn, kn, r0, r0 + 6, uv_mode=c["uv_mode"],
                                 boundaries=c["boundaries"], nthreads=oracle.env_threads())
        assert_bitwise(onen[r0:r0 + 6], rows)
    rng = np.random.default_rng(11)
    pix = rng.integers(0, 8192 * 8192, size=20000)
    np.testing.assert_array_equal(
        capi_cells(un, vn, 65, pix, c["uv_mode"], c["boundaries"]),
        oracle.paths(un, vn, 65, pix, uv_mode=c["uv_mode"], boundaries=c["boundaries"]),
    )
    five = rlic_gb300.convolve(tex, u, v, iterations=5, **kw)
    chain = one
    for _ in range(4):
        chain = rlic_gb300.convolve(chain, u, v, iterations=1, **kw)
    assert torch.equal(five.view(torch.int32), chain.view(torch.int32))


def test_images_beyond_2_31_pixels() -> None:
    """32768 x 65600 float32 (2.15e9 pixels): the 64-bit index kernels, traced
    and replayed.  With u = 1 and v = 0 every streamline runs along its row
    one cell per step (x periodic), so each pass is a row convolution whose
    float32 result numpy reproduces exactly: the weights are powers of two,
    so every product is exact and each sum rounds once, as the FMAs do."""
    import torch

    ny, nx = 32768, 65600
    assert ny * nx > 2**31
    gen = torch.Generator(device="cuda").manual_seed(8)
    tex = torch.rand((ny, nx), generator=gen, device="cuda", dtype=torch.float32)
    u = torch.ones_like(tex)
    v = torch.zeros_like(tex)
    k = torch.tensor([0.25, 0.5, 0.25], device="cuda", dtype=torch.float32)
    out = rlic_gb300.convolve(tex, u, v, kernel=k, boundaries={"x": "periodic", "y": "closed"},
                              iterations=2)
    del u, v
    f32 = np.float32

    def row_pass(t):  # acc = 0.5 t[j]; acc += 0.25 t[j+1]; acc += 0.25 t[j-1]
        acc = (f32(0.5) * t).astype(f32)
        acc = (acc + f32(0.25) * np.roll(t, -1)).astype(f32)
        return (acc + f32(0.25) * np.roll(t, 1)).astype(f32)

    for i in (0, 1, 12345, ny - 2, ny - 1):
        row = tex[i].cpu().numpy()
        assert_bitwise(out[i].cpu().numpy(), row_pass(row_pass(row)))


# ------------------------------------------------- public API / torch --

@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_torch_and_numpy_paths_agree(dtype) -> None:
    import torch

    rng = np.random.default_rng(9)
    u, v = _field(rng, 64, 80, dtype, "specials")
    tex = rng.random((64, 80)).astype(dtype)
    k = np.hanning(21).astype(dtype)
    kw = dict(uv_mode="polarization", boundaries={"x": "closed", "y": "periodic"}, iterations=3)
    a = rlic_gb300.convolve(tex, u, v, kernel=k, **kw)
    t = [torch.from_numpy(x).cuda() for x in (tex, u, v)]
    b = rlic_gb300.convolve(*t[:1], t[1], t[2], kernel=torch.from_numpy(k).cuda(), **kw)
    assert b.is_cuda and b.dtype == t[0].dtype
    assert_bitwise(a, b.cpu().numpy())


def test_strided_and_broadcast_inputs(oracle) -> None:
    c = readme_case(n=96)
    tex_f = np.asfortranarray(c["texture"])
    got = rlic_gb300.convolve(tex_f, c["u"], c["v"], kernel=c["kernel"][::-1][::-1],
                              boundaries="periodic")
    want = oracle.convolve(c["texture"], c["u"], c["v"], c["kernel"], boundaries="periodic")
    assert_bitwise(got, want)


def test_launches_are_counted() -> None:
    before = _native.launch_count()
    c = readme_case(n=64)
    u, v = np.ascontiguousarray(c["u"]), np.ascontiguousarray(c["v"])
    # pack + traced pass + 2 replays, plus the texture upload as a gather
    # kernel that also scans it for negative elements where the device reads
    # host memory in place (else a copy-engine copy and a scan kernel); one
    # row chunk at this size
    want = 5
    rlic_gb300.convolve(c["texture"], u, v, kernel=c["kernel"], iterations=3)
    assert _native.launch_count() - before == want
    before = _native.launch_count()
    # broadcast u, v: read in place where the device reaches host memory,
    # else made contiguous and copied
    rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"], iterations=3)
    assert _native.launch_count() - before == want


def test_device_entry_points_with_workspace(oracle) -> None:
    """rlic_convolve_f32 on device pointers with a caller workspace, and the
    pack + sweep building blocks, on a torch stream."""
    import torch

    lib = _native.lib()
    rng = np.random.default_rng(21)
    u, v = _field(rng, 70, 90, np.float32, "specials")
    tex = rng.random((70, 90)).astype(np.float32)
    k = np.hanning(33).astype(np.float32)
    want1 = oracle.convolve(tex, u, v, k, uv_mode="polarization", boundaries="periodic")
    want3 = oracle.convolve(tex, u, v, k, uv_mode="polarization", boundaries="periodic",
                            iterations=3)
    d = {n: torch.from_numpy(a).cuda() for n, a in dict(t=tex, u=u, v=v, k=k).items()}
    out = torch.empty_like(d["t"])
    nbytes = lib.rlic_workspace_bytes(70, 90, 33, 3, 4, 0)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _native.check(lib.rlic_convolve_f32(
        d["t"].data_ptr(), d["u"].data_ptr(), d["v"].data_ptr(), 70, 90, d["k"].data_ptr(), 33,
        1, 1, 1, 1, 1, 3, out.data_ptr(), ws.data_ptr(), nbytes, stream, 0))
    assert_bitwise(out.cpu().numpy(), want3)
    rc = lib.rlic_convolve_f32(
        d["t"].data_ptr(), d["u"].data_ptr(), d["v"].data_ptr(), 70, 90, d["k"].data_ptr(), 33,
        1, 1, 1, 1, 1, 3, out.data_ptr(), ws.data_ptr(), nbytes - 1, stream, 0)
    assert rc == _native.RLIC_ERR_WORKSPACE_TOO_SMALL
    uv = torch.empty((70, 90, 2), dtype=torch.float32, device="cuda")
    _native.check(lib.rlic_pack_field_f32(d["u"].data_ptr(), d["v"].data_ptr(), 70, 90,
                                          uv.data_ptr(), stream))
    codes = torch.empty(lib.rlic_path_code_bytes(70, 90, 33) // 4, dtype=torch.int32,
                        device="cuda")
    _native.check(lib.rlic_sweep_f32(d["t"].data_ptr(), uv.data_ptr(), 70, 90,
                                     d["k"].data_ptr(), 33, 1, 1, 1, 1, 1, out.data_ptr(),
                                     codes.data_ptr(), stream, 0))
    assert_bitwise(out.cpu().numpy(), want1)
    # replaying the recorded paths on another texture = tracing it
    tex2 = torch.from_numpy(rng.random((70, 90)).astype(np.float32)).cuda()
    traced = torch.empty_like(out)
    _native.check(lib.rlic_sweep_f32(tex2.data_ptr(), uv.data_ptr(), 70, 90,
                                     d["k"].data_ptr(), 33, 1, 1, 1, 1, 1, traced.data_ptr(),
                                     None, stream, 0))
    _native.check(lib.rlic_replay_f32(tex2.data_ptr(), codes.data_ptr(), 70, 90,
                                      d["k"].data_ptr(), 33, out.data_ptr(), stream, 0))
    assert_bitwise(out.cpu().numpy(), traced.cpu().numpy())
    want2 = oracle.convolve(tex2.cpu().numpy(), u, v, k, uv_mode="polarization",
                            boundaries="periodic")
    assert_bitwise(out.cpu().numpy(), want2)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sweep_with_a_nan_free_promise(oracle, dtype) -> None:
    """RLIC_FLAG_FIELD_NAN_FREE on a field without NaN samples gives the same
    bits and codes as the checked steps."""
    import torch

    lib = _native.lib()
    sfx = "f32" if dtype == np.float32 else "f64"
    rng = np.random.default_rng(23)
    ny, nx, klen = 120, 200, 21
    u, v = _field(rng, ny, nx, dtype, "random")
    tex = rng.random((ny, nx)).astype(dtype)
    k = np.hanning(klen).astype(dtype)
    d = {n: torch.from_numpy(a).cuda() for n, a in dict(t=tex, u=u, v=v, k=k).items()}
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    uv = torch.empty((ny, nx, 2), dtype=d["t"].dtype, device="cuda")
    _native.check(getattr(lib, f"rlic_pack_field_{sfx}")(d["u"].data_ptr(), d["v"].data_ptr(),
                                                         ny, nx, uv.data_ptr(), stream))
    outs, codes = [], []
    for flags in (0, _native.RLIC_FLAG_FIELD_NAN_FREE):
        out = torch.empty_like(d["t"])
        c = torch.empty(lib.rlic_path_code_bytes(ny, nx, klen) // 4, dtype=torch.int32,
                        device="cuda")
        _native.check(getattr(lib, f"rlic_sweep_{sfx}")(
            d["t"].data_ptr(), uv.data_ptr(), ny, nx, d["k"].data_ptr(), klen, 1, 1, 1, 0, 0,
            out.data_ptr(), c.data_ptr(), stream, flags))
        outs.append(out.cpu().numpy())
        codes.append(c.cpu().numpy())
    want = oracle.convolve(tex, u, v, k, uv_mode="polarization",
                           boundaries={"x": "periodic", "y": "closed"})
    assert_bitwise(outs[0], want)
    assert_bitwise(outs[1], want)
    np.testing.assert_array_equal(codes[0], codes[1])
    # the convolve entry points take no such promise: they find it out
    rc = getattr(lib, f"rlic_convolve_{sfx}")(
        d["t"].data_ptr(), d["u"].data_ptr(), d["v"].data_ptr(), ny, nx, d["k"].data_ptr(),
        klen, 1, 1, 1, 0, 0, 1, torch.empty_like(d["t"]).data_ptr(), None, 0, stream,
        _native.RLIC_FLAG_FIELD_NAN_FREE)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT


def test_host_path_checks_negative_texture_on_device() -> None:
    rng = np.random.default_rng(31)
    tex = rng.random((64, 80))
    u, v = _field(rng, 64, 80, np.float64, "random")
    k = np.hanning(9)
    bad = tex.copy()
    bad[17, 3] = -1e-300
    with pytest.raises(ValueError, match=r"^Found invalid texture element\(s\)\. Expected only positive values\.$"):
        rlic_gb300.convolve(bad, u, v, kernel=k, iterations=2)
    # -0.0 and NaN are not below zero: no error, as np.any(texture < 0)
    ok = tex.copy()
    ok[0, 0] = -0.0
    ok[1, 1] = np.nan
    out = rlic_gb300.convolve(ok, u, v, kernel=k)
    assert out.shape == ok.shape
    # several problems at once are still grouped on the host, in order
    with pytest.raises(ExceptionGroup) as info:
        rlic_gb300.convolve(bad, u, v, kernel=k, iterations=-1)
    assert [type(e) for e in info.value.exceptions] == [ValueError, ValueError]


_NEGATIVE_MSG = r"^Found invalid texture element\(s\)\. Expected only positive values\.$"


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("layout", ["contiguous", "transposed", "odd_width", "chunked"])
def test_texture_check_in_every_upload_form(dtype, layout) -> None:
    """The texture's scan for elements below zero runs inside its upload, in
    each upload form: 16-byte vector copies (contiguous rows), element
    gathers (a transposed view, rows of a width that is no multiple of 16
    bytes) and row chunks (4 Mpx), with the element in the last rows read.
    -0.0, NaN and +inf are not below zero; -inf and the smallest subnormal
    below zero are."""
    ny, nx = {"contiguous": (96, 128), "transposed": (96, 128), "odd_width": (90, 127),
              "chunked": (2048, 2048)}[layout]
    rng = np.random.default_rng(47)
    tex = rng.random((ny, nx)).astype(dtype)
    u, v = _field(rng, ny, nx, dtype, "random")
    k = np.hanning(9).astype(dtype)

    def shaped(a: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(a.T).T if layout == "transposed" else a

    tiny = np.finfo(dtype).smallest_subnormal
    for value in (-1.0, -np.inf, -tiny):
        bad = tex.copy()
        bad[ny - 1, nx - 2] = value
        with pytest.raises(ValueError, match=_NEGATIVE_MSG):
            rlic_gb300.convolve(shaped(bad), shaped(u), shaped(v), kernel=k, iterations=2)
    ok = tex.copy()
    ok[ny - 1, nx - 1] = -0.0
    ok[ny - 1, nx - 2] = np.nan
    ok[ny - 1, nx - 3] = np.inf
    got = rlic_gb300.convolve(shaped(ok), shaped(u), shaped(v), kernel=k, iterations=2)
    assert got.shape == (ny, nx)
    # the scan leaves the convolution itself alone
    want = rlic_gb300.convolve(tex, u, v, kernel=k, iterations=2)
    assert_bitwise(rlic_gb300.convolve(shaped(tex), shaped(u), shaped(v), kernel=k,
                                       iterations=2), want)


def test_host_path_without_direct_access(tmp_path) -> None:
    """The copy-based host path (devices without pageable-memory access) gives
    the same bits as the direct one."""
    import subprocess
    import sys

    script = tmp_path / "noh.py"
    script.write_text(
        "import sys, numpy as np\n"
        f"sys.path.insert(0, {str(Path(__file__).resolve().parents[1])!r})\n"
        "import rlic_gb300\n"
        "from rlic_gb300.workloads import readme_case\n"
        "c = readme_case(n=96)\n"
        "out = rlic_gb300.convolve(c['texture'], c['u'], c['v'], kernel=c['kernel'],\n"
        "                          boundaries='periodic', iterations=3)\n"
        f"np.save({str(tmp_path / 'out.npy')!r}, out)\n"
        "c = readme_case(n=2100, dtype=np.float32, seed=5)\n"
        "out = rlic_gb300.convolve(c['texture'], c['u'], c['v'], kernel=c['kernel'],\n"
        "                          boundaries='periodic', iterations=2)\n"
        f"np.save({str(tmp_path / 'big.npy')!r}, out)\n"
        # copied uploads scan the texture in a pass of their own
        "for n in (96, 2100):\n"
        "    c = readme_case(n=n)\n"
        "    c['texture'][n - 1, 3] = -1.0\n"
        "    try:\n"
        "        rlic_gb300.convolve(c['texture'], c['u'], c['v'], kernel=c['kernel'],\n"
        "                            iterations=2)\n"
        "    except ValueError as exc:\n"
        "        assert str(exc).startswith('Found invalid texture'), exc\n"
        "    else:\n"
        "        raise SystemExit('a negative texture element was not reported')\n"
    )
    env = dict(__import__("os").environ, RLIC_NO_HOST_DIRECT="1")
    subprocess.run([sys.executable, str(script)], check=True, env=env, timeout=300)
    c = readme_case(n=96)
    want = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"],
                               boundaries="periodic", iterations=3)
    assert_bitwise(np.load(tmp_path / "out.npy"), want)
    # 4.4 Mpx: uploaded in row chunks by copy-engine copies
    c = readme_case(n=2100, dtype=np.float32, seed=5)
    want = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"],
                               boundaries="periodic", iterations=2)
    assert_bitwise(np.load(tmp_path / "big.npy"), want)


@pytest.mark.parametrize("bnd, klen, iterations", [
    ({"x": "periodic", "y": "closed"}, 65, 5),
    ("periodic", 129, 3),
    ({"x": "closed", "y": "periodic"}, 33, 1),
    ("closed", 9, 2),
])
def test_host_path_row_chunks(bnd, klen, iterations) -> None:
    """Host arrays of 4 Mpx and more go up in row chunks, with the traced pass
    started per group of tile rows as their rows and halo arrive (across the
    seam for a periodic y axis): same bits as the device-resident path,
    contiguous and strided, on a ragged row count, with and without NaN
    samples in the last chunk."""
    import torch

    rng = np.random.default_rng(klen)
    ny, nx = 2101, 2050
    u, v = _field(rng, ny, nx, np.float32, "random")
    if klen != 33:
        # NaN samples only in the last rows: tile rows traced before that
        # chunk arrives take the NaN-free steps, the others check every step
        u[ny - 40:ny - 30, 100:140] = np.nan
    tex = rng.random((ny, nx), dtype=np.float32)
    k = np.hanning(klen).astype(np.float32)
    kw = dict(uv_mode="polarization", boundaries=bnd, iterations=iterations)
    want = rlic_gb300.convolve(torch.from_numpy(tex).cuda(), torch.from_numpy(u).cuda(),
                               torch.from_numpy(v).cuda(), kernel=torch.from_numpy(k).cuda(),
                               **kw).cpu().numpy()
    assert_bitwise(rlic_gb300.convolve(tex, u, v, kernel=k, **kw), want)
    # the same arrays read through transposed views of their transposes
    tt, ut, vt = (np.ascontiguousarray(a.T).T for a in (tex, u, v))
    assert_bitwise(rlic_gb300.convolve(tt, ut, vt, kernel=k, **kw), want)


def test_concurrent_host_calls_from_threads() -> None:
    """The ctypes call releases the GIL and a host-memory call runs on its
    thread's own stream: calls from several Python threads at once (large
    enough to take the chunked upload) give each caller its own result."""
    from concurrent.futures import ThreadPoolExecutor

    cases = [readme_case(n=2100, klen=k, dtype=np.float32, seed=s)
             for s, k in ((1, 33), (2, 65), (3, 17), (4, 65))]
    kw = dict(boundaries={"x": "periodic", "y": "closed"}, uv_mode="polarization",
              iterations=3)

    def run(c):
        return rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"], **kw)

    want = [run(c) for c in cases]
    with ThreadPoolExecutor(max_workers=4) as pool:
        for _ in range(3):
            got = list(pool.map(run, cases))
            for g, w in zip(got, want):
                assert_bitwise(g, w)


def test_strided_views_read_in_place(oracle) -> None:
    """Broadcast, transposed, reversed and sliced numpy views give the bits of
    their contiguous copies (read in place where the device can reach host
    memory, copied otherwise)."""
    c = readme_case(n=300)
    big = np.random.default_rng(41).random((600, 700))
    views = {
        "broadcast_uv": (c["texture"], c["u"], c["v"]),
        "transposed": (big[:300, :300].T, c["u"].T, c["v"].T),
        "reversed_sliced": (big[::-2, 5:605:2], np.ascontiguousarray(c["u"])[::-1, ::-1],
                            np.ascontiguousarray(c["v"])[:, ::-1]),
        "broadcast_texture": (np.broadcast_to(big[0, :300], (300, 300)), c["u"], c["v"]),
    }
    for name, (t, u, v) in views.items():
        for dtype in (np.float64, np.float32):
            t_, u_, v_ = (np.asarray(a, dtype=dtype) if a.dtype != dtype else a for a in (t, u, v))
            k = c["kernel"].astype(dtype)
            got = rlic_gb300.convolve(t_, u_, v_, kernel=k, uv_mode="polarization",
                                      boundaries={"x": "periodic", "y": "closed"}, iterations=2)
            want = rlic_gb300.convolve(np.ascontiguousarray(t_), np.ascontiguousarray(u_),
                                       np.ascontiguousarray(v_), kernel=k, uv_mode="polarization",
                                       boundaries={"x": "periodic", "y": "closed"}, iterations=2)
            assert_bitwise(got, want)
    # and the contiguous result is the oracle's
    t, u, v = views["transposed"]
    want = oracle.convolve(np.ascontiguousarray(t), u, v, c["kernel"], iterations=1)
    assert_bitwise(rlic_gb300.convolve(t, u, v, kernel=c["kernel"]), want)
