"""Parity at the benchmark workloads' own sizes, through the public API and
the C ABI.

The oracle is too slow to convolve these images in full for many passes, so
each check uses an exact shortcut:

* ``oracle.convolve_rows`` evaluates rows [r0, r1) of an n-pass result from
  bands of rows only (a streamline moves at most klen // 2 rows, so pass p
  needs klen // 2 more rows on each side than pass p + 1); every such band is
  compared bit for bit;
* streamline cells of sampled pixels are compared index for index;
* the gradients obey identities that hold at any size: the adjoint identity
  <W, A x> = <A^T W, x>, and Euler's identity for the kernel weights (an
  n-pass output is homogeneous of degree n in the kernel, so
  sum_q k_q dL/dk_q = n L), beside central finite differences.

Workloads: the 8192^2 float32 polarization case with mixed boundaries and
5 passes; 8192^2 float64, 129 taps, periodic, 10 passes (the precision
workload's exact path); the 64-instance batched mix; 1024^2 float32,
33 taps, 3 passes (the differentiable workload).
"""

from __future__ import annotations

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300 import _native
from rlic_gb300.workloads import batch_case, fourier_vortex_case, readme_case

pytestmark = pytest.mark.gpu

CODES = {"closed": 0, "periodic": 1}


def assert_bitwise(got, want) -> None:
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape and got.dtype == want.dtype
    itype = np.uint32 if got.dtype == np.float32 else np.uint64
    bad = got.view(itype) != want.view(itype)
    bad &= ~(np.isnan(got) & np.isnan(want))
    assert not bad.any(), (np.argwhere(bad)[:5], got[bad][:5], want[bad][:5])


def _bcodes(bnd):
    if isinstance(bnd, str):
        return (CODES[bnd],) * 4
    return (CODES[bnd["x"]],) * 2 + (CODES[bnd["y"]],) * 2


def _cells(u, v, klen, pix, uv_mode, bnd):
    """rlic_trace_cells_* on host arrays."""
    lib = _native.lib()
    dtype = np.asarray(u).dtype
    u, v = (np.ascontiguousarray(a, dtype=dtype) for a in (u, v))
    pix = np.ascontiguousarray(pix, dtype=np.int64)
    cells = np.full((pix.size, klen - 1), -7, dtype=np.int64)
    fn = lib.rlic_trace_cells_f32 if dtype == np.float32 else lib.rlic_trace_cells_f64
    ny, nx = u.shape
    _native.check(fn(u.ctypes.data, v.ctypes.data, ny, nx, klen, int(uv_mode == "polarization"),
                     *_bcodes(bnd), pix.size, pix.ctypes.data, cells.ctypes.data, None,
                     _native.RLIC_FLAG_HOST_MEMORY))
    return cells


# ------------------------------------- 8192^2 float32, 65 taps, 5 passes --

def test_fourier_vortex_8192_five_passes_on_row_bands(oracle) -> None:
    c = fourier_vortex_case(n=8192, device="cuda", as_numpy=False)
    kw = dict(uv_mode=c["uv_mode"], boundaries=c["boundaries"])
    got = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"], iterations=5,
                              **kw).cpu().numpy()
    tn, un, vn, kn = (c[x].cpu().numpy() for x in ("texture", "u", "v", "kernel"))
    # the closed top and bottom edges and the middle of the image
    for r0, r1 in ((0, 4), (4093, 4101), (8188, 8192)):
        want = oracle.convolve_rows(tn, un, vn, kn, r0, r1, iterations=5,
                                    nthreads=oracle.env_threads(), **kw)
        assert_bitwise(got[r0:r1], want)


# ---------------------- 8192^2 float64, 129 taps, periodic, 10 passes --

@pytest.fixture(scope="module")
def precision_case():
    c = readme_case(n=8192, klen=129, dtype=np.float64, seed=2)
    c.update(iterations=10)
    return c


def test_precision_workload_ten_passes_on_row_bands(oracle, precision_case) -> None:
    """The exact float64 path of the precision workload (path cache: one
    traced pass, nine replays) against the oracle on a middle band, and its
    first pass on bands that wrap across the periodic seams."""
    c = precision_case
    kw = dict(boundaries="periodic")
    got = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"], iterations=10,
                              **kw)
    want = oracle.convolve_rows(c["texture"], c["u"], c["v"], c["kernel"], 4094, 4098,
                                iterations=10, nthreads=oracle.env_threads(), **kw)
    assert_bitwise(got[4094:4098], want)
    one = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"], iterations=1,
                              **kw)
    for r0, r1 in ((0, 3), (8189, 8192)):
        want = oracle.sweep_rows(c["texture"], c["u"], c["v"], c["kernel"], r0, r1,
                                 nthreads=oracle.env_threads(), **kw)
        assert_bitwise(one[r0:r1], want)


def test_precision_workload_cells(oracle, precision_case) -> None:
    c = precision_case
    rng = np.random.default_rng(21)
    pix = rng.integers(0, 8192 * 8192, size=20000)
    pix[:64] = np.arange(64) * 8192  # column 0, where v is exactly +0
    np.testing.assert_array_equal(
        _cells(c["u"], c["v"], 129, pix, "velocity", "periodic"),
        oracle.paths(c["u"], c["v"], 129, pix, boundaries="periodic"))


def _step_operands(u, v, pix, klen, oracle):
    """(ax, ay, u, v) of every step of the streamlines of `pix`: the time
    numerators fma(1 + signum(vel), 0.5 - f, f) of both axes and the
    sign-adjusted velocity (src/lib.rs:168-179, 241-249), in velocity mode.
    A still lane's velocity is given as (1, 1), the stand-in the float64 step
    divides by.  The state follows the oracle's advance."""
    ny, nx = u.shape
    rows = []
    kmid = klen // 2
    for p in pix:
        for backward, count in ((False, klen - kmid - 1), (True, kmid)):
            i, j = divmod(int(p), nx)
            fx = fy = 0.5
            for _ in range(count):
                pu, pv = float(u[i, j]), float(v[i, j])
                if np.isnan(pu) or np.isnan(pv):
                    break
                if backward:
                    pu, pv = -pu, -pv
                still = pu == 0.0 and pv == 0.0
                su, sv = (1.0, 1.0) if still else (pu, pv)
                # 1 + signum(v) is 2 or 0 (signum(-0.0) = -1); 2 * (0.5 - f) is
                # exact, so one Python rounding is the fma's single rounding
                ax = fx if np.signbit(su) else 2.0 * (0.5 - fx) + fx
                ay = fy if np.signbit(sv) else 2.0 * (0.5 - fy) + fy
                rows.append((ax, ay, su, sv))
                i, j, fx, fy = oracle.advance(pu, pv, i, j, fx, fy, (ny, nx),
                                              boundaries="periodic")
    return np.array(rows, dtype=np.float64).T


def _truncate_to_f32(x):
    """|x| with 23 fraction bits, as float32 (exponents in [-60, 60])."""
    b = np.abs(x).view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64) - (1023 - 127)
    e = np.clip(e, 1, 254).astype(np.uint32)
    frac = ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)).astype(np.uint32)
    return ((e << np.uint32(23)) | frac).view(np.float32)


def _in_range(x):
    e = ((np.abs(x).view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    return (e >= 1023 - 60) & (e <= 1023 + 60)


def test_precision_workload_float64_screen(oracle, precision_case) -> None:
    """The float64 step settles tx < ty from float32 cross products before it
    divides, then divides once by a certified Newton sequence; anything else
    falls back to IEEE divisions.  On the precision workload's own field:
    every settled comparison equals the comparison of the correctly rounded
    times, and the share of steps that fall back is small."""
    import torch

    c = precision_case
    u = np.ascontiguousarray(c["u"])
    v = np.ascontiguousarray(c["v"])
    rng = np.random.default_rng(22)
    pix = rng.integers(0, 8192 * 8192, size=2000)
    pix[:8] = rng.integers(0, 8192, 8) * 8192  # column 0, where v is exactly +0
    ax, ay, su, sv = _step_operands(u, v, pix, 129, oracle)
    # the screen, as the device computes it (screen_step)
    ax0, ay0 = ax == 0, ay == 0
    in_range = _in_range(su) & _in_range(sv) & (ax0 | _in_range(ax)) & (ay0 | _in_range(ay))
    with np.errstate(all="ignore"):
        p1 = _truncate_to_f32(ax) * _truncate_to_f32(sv)
        p2 = _truncate_to_f32(ay) * _truncate_to_f32(su)
        lt = p1 < p2 * np.float32(1 - 2.0**-16)
        gt = p1 > p2 * np.float32(1 + 2.0**-16)
        any0 = ax0 | ay0
        xstep = np.where(any0, ax0 & ~ay0, lt)
        settled = in_range & (any0 | lt | gt)
        tx, ty = np.abs(ax / su), np.abs(ay / sv)
    # a settled comparison is the comparison of the IEEE times
    assert np.array_equal(xstep[settled], (tx < ty)[settled])
    # the one division of a settled step, certified or not
    first_x = ~settled | xstep
    num = np.where(first_x, ax, ay)
    den = np.where(first_x, su, sv)
    a = torch.from_numpy(np.where(num == 0, 1.0, num)).cuda()
    b = torch.from_numpy(den).cuda()
    q = torch.empty_like(a)
    cert = torch.empty(a.shape, dtype=torch.int32, device="cuda")
    _native.check(_native.lib().rlic_check_quotients_f64(
        a.data_ptr(), b.data_ptr(), a.numel(), q.data_ptr(), cert.data_ptr(), None))
    torch.cuda.synchronize()
    cert = cert.cpu().numpy().astype(bool)
    fallback = ~(settled & cert)
    rate = float(fallback.mean())
    print(f"\nfloat64 screen on the precision workload: {ax.size} steps, "
          f"unsettled {float((~settled).mean()):.4%}, "
          f"settled but uncertified {float((settled & ~cert).mean()):.4%}, "
          f"fallback {rate:.4%}")
    assert rate < 0.02


# ----------------------------------------- 64-instance batched workload --

def test_batched_workload_on_row_bands(oracle) -> None:
    """The 64-instance mix (sides 256-4096, 17-129 taps, 1-10 passes, mixed
    boundaries and modes) in one batched call, each instance against the
    oracle on a band of rows at its middle and at its top edge."""
    from rlic_gb300.batch import convolve_batch

    items = batch_case(count=64, seed=3)
    outs = convolve_batch(items)
    for k, (it, got) in enumerate(zip(items, outs)):
        ny = int(it["texture"].shape[0])
        host = {x: it[x].cpu().numpy() for x in ("texture", "u", "v", "kernel")}
        gotn = got.cpu().numpy()
        kw = dict(uv_mode=it["uv_mode"], boundaries=it["boundaries"],
                  iterations=it["iterations"], nthreads=oracle.env_threads())
        bands = [(ny // 2 - 2, ny // 2 + 2)]
        if it["boundaries"]["y"] == "closed":
            bands.append((0, 2))  # the edge band costs no more than the middle one
        for r0, r1 in bands:
            want = oracle.convolve_rows(host["texture"], host["u"], host["v"], host["kernel"],
                                        r0, r1, **kw)
            assert_bitwise(gotn[r0:r1], want)


# ------------------------- 1024^2 float32, 33 taps, 3 passes, gradients --

def test_differentiable_workload_forward_in_full(oracle) -> None:
    from rlic_gb300.forms import convolve_autograd

    c = readme_case(n=1024, klen=33, dtype=np.float32, seed=4)
    import torch

    t = {x: torch.from_numpy(np.ascontiguousarray(c[x])).cuda()
         for x in ("texture", "u", "v", "kernel")}
    got = convolve_autograd(t["texture"], t["u"], t["v"], kernel=t["kernel"],
                            boundaries="periodic", iterations=3)
    want = oracle.convolve(c["texture"], c["u"], c["v"], c["kernel"], boundaries="periodic",
                           iterations=3, nthreads=oracle.env_threads())
    assert_bitwise(got.detach().cpu().numpy(), want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_differentiable_workload_gradient_identities(dtype) -> None:
    """At 1024^2, 33 taps, 3 passes: the texture gradient satisfies the
    adjoint identity sum(W * out) = sum(grad_texture * texture), and the
    kernel gradient Euler's identity sum(k * grad_kernel) = 3 * loss."""
    import torch

    from rlic_gb300.forms import convolve_autograd

    n, iters = 1024, 3
    c = readme_case(n=n, klen=33, dtype=dtype, seed=4)
    t = {x: torch.from_numpy(np.ascontiguousarray(c[x])).cuda()
         for x in ("texture", "u", "v", "kernel")}
    W = torch.from_numpy(np.random.default_rng(4).normal(size=(n, n)).astype(dtype)).cuda()
    tex = t["texture"].clone().requires_grad_(True)
    k = t["kernel"].clone().requires_grad_(True)
    out = convolve_autograd(tex, t["u"], t["v"], kernel=k, boundaries="periodic",
                            iterations=iters)
    loss = (out * W).sum()
    loss.backward()
    L = float(loss.detach().double())
    adj = float((tex.grad.double() * t["texture"].double()).sum())
    euler = float((k.grad.double() * t["kernel"].double()).sum())
    scale = float((out.detach().abs() * W.abs()).sum().double())  # size of the sum's terms
    tol = 1e-10 if dtype == np.float64 else 2e-4
    assert abs(adj - L) <= tol * scale
    assert abs(euler - iters * L) <= tol * iters * scale


def test_differentiable_workload_finite_differences() -> None:
    """Central finite differences in float64 (h = 1e-6) at 1024^2: texture
    entries >= 2h (validation rejects negative textures) and a random
    direction in kernel space.  The loss difference is taken as
    sum(W * (out(+h) - out(-h))), so that only the outputs the perturbation
    changes contribute rounding."""
    import torch

    from rlic_gb300.forms import convolve_autograd

    n, klen, iters, h = 1024, 33, 3, 1e-6
    c = readme_case(n=n, klen=klen, dtype=np.float64, seed=4)
    rng = np.random.default_rng(5)
    t = {x: torch.from_numpy(np.ascontiguousarray(c[x])).cuda()
         for x in ("texture", "u", "v", "kernel")}
    W = torch.from_numpy(rng.normal(size=(n, n))).cuda()
    kw = dict(boundaries="periodic", iterations=iters)

    def out(tex, k):
        return rlic_gb300.convolve(tex, t["u"], t["v"], kernel=k, **kw)

    def central(plus, minus):
        return float(((out(*plus) - out(*minus)) * W).sum()) / (2 * h)

    tex = t["texture"].clone().requires_grad_(True)
    k = t["kernel"].clone().requires_grad_(True)
    (convolve_autograd(tex, t["u"], t["v"], kernel=k, **kw) * W).sum().backward()
    gt, gk = tex.grad.cpu().numpy(), k.grad.cpu().numpy()
    flat = np.flatnonzero(c["texture"].ravel() >= 2 * h)
    for idx in rng.choice(flat, size=6, replace=False):
        i, j = divmod(int(idx), n)
        tp, tm = t["texture"].clone(), t["texture"].clone()
        tp[i, j] += h
        tm[i, j] -= h
        fd = central((tp, t["kernel"]), (tm, t["kernel"]))
        assert fd == pytest.approx(gt[i, j], rel=1e-5, abs=1e-6 * np.abs(gt).max())
    d = torch.from_numpy(rng.normal(size=klen)).cuda()
    fd = central((t["texture"], t["kernel"] + h * d), (t["texture"], t["kernel"] - h * d))
    assert fd == pytest.approx(float(np.dot(gk, d.cpu().numpy())), rel=1e-6)
