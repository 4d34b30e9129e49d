"""Seeded synthetic inputs with the shapes of the benchmark workloads.

The reference publishes no benchmark dataset; these generators stand in for
it with the recipes below.  Each returns a dict with the arguments of
``convolve``: ``texture``, ``u``, ``v``, ``kernel`` (arrays) and
``uv_mode``, ``boundaries``, ``iterations``.

* ``readme_case``: the reference's README example (README.md:49-56, 78):
  256 x 256 float64, texture ~ U[0, 1) from default_rng(0),
  u = cos(2x) broadcast over rows, v = sin(x) broadcast over rows,
  x = linspace(0, pi, 256), kernel 1 - |linspace(-1, 1, 65)|, periodic,
  velocity, one iteration.  u and v are zero-stride broadcast views as in
  the README; note v[:, 0] is exactly +0.0.
* ``fourier_vortex_case``: the at-scale workload, 8192 x 8192 float32 by
  default: texture ~ U[0, 1) (default_rng(1)); (u, v) = sum of 32 random
  Fourier modes with integer wavevectors of norm in [1, 16] and amplitudes
  N(0, 1) / (1 + |k|^2), plus 8 point vortices / sinks with a core softened
  over two cells, evaluated in float64 and cast; 1% of cells (seeded) set
  to u = v = 0 exactly; kernel = Hann window of 65 taps; boundaries
  {x: periodic, y: closed}; polarization; 5 iterations.
"""

from __future__ import annotations

import math

import numpy as np


def readme_case(n: int = 256, klen: int = 65, dtype=np.float64, seed: int = 0) -> dict:
    prng = np.random.default_rng(seed)
    shape = (n, n)
    texture = prng.random(shape).astype(dtype, copy=False)
    x = np.linspace(0, np.pi, n)
    u = np.broadcast_to(np.cos(2 * x).astype(dtype), shape)
    v = np.broadcast_to(np.sin(x).T.astype(dtype), shape)
    kernel = (1 - np.abs(np.linspace(-1, 1, klen))).astype(dtype)
    return dict(
        texture=texture, u=u, v=v, kernel=kernel, uv_mode="velocity",
        boundaries="periodic", iterations=1,
    )


def _field_parameters(seed: int):
    """Mode and vortex parameters, drawn with numpy so they never depend on torch."""
    rng = np.random.default_rng(seed)
    modes = []
    while len(modes) < 32:
        kx, ky = rng.integers(-16, 17, size=2)
        kn = math.hypot(kx, ky)
        if 1 <= kn <= 16:
            au, av = rng.normal(size=2) / (1 + kn * kn)
            pu, pv = rng.uniform(0, 2 * np.pi, size=2)
            modes.append((int(kx), int(ky), float(au), float(av), float(pu), float(pv)))
    vortices = []
    for _ in range(8):
        x0, y0 = rng.uniform(0, 1, size=2)
        strength = float(rng.normal()) * 0.02
        kind = int(rng.integers(0, 2))  # 0: vortex, 1: sink/source
        vortices.append((float(x0), float(y0), strength, kind))
    return modes, vortices


def fourier_vortex_field(n: int, seed: int = 1, device: str = "cpu", dtype=None):
    """(u, v) torch tensors of shape (n, n) built in float64 on `device`, then cast."""
    import torch

    modes, vortices = _field_parameters(seed + 1000)
    f64 = torch.float64
    coord = torch.arange(n, dtype=f64, device=device) / n  # unit square, periodic
    u = torch.zeros((n, n), dtype=f64, device=device)
    v = torch.zeros((n, n), dtype=f64, device=device)
    # cos(a x + b y + p) = cos(a x + p) cos(b y) - sin(a x + p) sin(b y): rank-2 per mode
    for kx, ky, au, av, pu, pv in modes:
        ax = 2 * np.pi * kx * coord
        by = 2 * np.pi * ky * coord
        cy, sy = torch.cos(by), torch.sin(by)
        u += au * (torch.outer(cy, torch.cos(ax + pu)) - torch.outer(sy, torch.sin(ax + pu)))
        v += av * (torch.outer(cy, torch.cos(ax + pv)) - torch.outer(sy, torch.sin(ax + pv)))
    eps2 = (2.0 / n) ** 2
    for x0, y0, strength, kind in vortices:
        dx = (coord - x0)[None, :]
        dy = (coord - y0)[:, None]
        inv = strength / (dx * dx + dy * dy + eps2)
        if kind == 0:
            u -= dy * inv
            v += dx * inv
        else:
            u += dx * inv
            v += dy * inv
    gen = torch.Generator(device="cpu").manual_seed(seed + 2000)
    zero = (torch.rand((n, n), generator=gen) < 0.01).to(device)
    u[zero] = 0.0
    v[zero] = 0.0
    if dtype is not None:
        u, v = u.to(dtype), v.to(dtype)
    return u, v


def fourier_vortex_case(
    n: int = 8192, klen: int = 65, seed: int = 1, device: str = "cpu", as_numpy: bool = True,
    dtype=np.float32, iterations: int = 5,
) -> dict:
    import torch

    tdtype = torch.float32 if dtype == np.float32 else torch.float64
    u, v = fourier_vortex_field(n, seed=seed, device=device, dtype=tdtype)
    texture = np.random.default_rng(seed).random((n, n), dtype=dtype)
    kernel = np.hanning(klen).astype(dtype)
    if as_numpy:
        u, v = u.cpu().numpy(), v.cpu().numpy()
    else:
        texture = torch.from_numpy(texture).to(device)
        kernel = torch.from_numpy(kernel).to(device)
    return dict(
        texture=texture, u=u, v=v, kernel=kernel, uv_mode="polarization",
        boundaries={"x": "periodic", "y": "closed"}, iterations=iterations,
    )


def batch_case(count: int = 64, seed: int = 3, device: str = "cuda", min_side: int = 256,
               max_side: int = 4096) -> list[dict]:
    """Batched workload: `count` independent float32 instances.

    Square sides log-uniform in [min_side, max_side] (seed 3), fields and
    textures as in ``readme_case`` with per-instance seeds, kernel lengths
    uniform over the odd values in [17, 129] (triangle or Hann), boundaries
    drawn per axis from {closed, periodic}, uv_mode drawn per instance,
    iterations uniform in [1, 10].  Returns dicts of ``convolve`` arguments
    with torch tensors on `device`.
    """
    import torch

    rng = np.random.default_rng(seed)
    items = []
    for k in range(count):
        side = int(round(math.exp(rng.uniform(math.log(min_side), math.log(max_side)))))
        klen = int(rng.choice(np.arange(17, 130, 2)))
        hann = bool(rng.integers(0, 2))
        bx = ["closed", "periodic"][int(rng.integers(0, 2))]
        by = ["closed", "periodic"][int(rng.integers(0, 2))]
        uv_mode = ["velocity", "polarization"][int(rng.integers(0, 2))]
        iterations = int(rng.integers(1, 11))
        c = readme_case(n=side, klen=klen, dtype=np.float32, seed=seed * 1000 + k)
        kernel = np.hanning(klen).astype(np.float32) if hann else c["kernel"]
        items.append(dict(
            texture=torch.from_numpy(c["texture"]).to(device),
            u=torch.from_numpy(np.ascontiguousarray(c["u"])).to(device),
            v=torch.from_numpy(np.ascontiguousarray(c["v"])).to(device),
            kernel=torch.from_numpy(kernel).to(device), uv_mode=uv_mode,
            boundaries={"x": bx, "y": by}, iterations=iterations,
        ))
    return items


def samples(case: dict) -> int:
    """Kernel-weighted texture reads of a case: H * W * K * iterations."""
    ny, nx = case["texture"].shape
    return int(ny) * int(nx) * int(case["kernel"].shape[0]) * int(case["iterations"])
