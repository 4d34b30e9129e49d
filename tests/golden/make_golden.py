"""Regenerates the golden vectors in this directory.

The reference cannot run in this environment (its Rust core needs a
toolchain that is absent), so these vectors come from the C oracle
(oracle/lic_oracle.c), each tiny case cross-checked first against the
independent pure-Python restatement (oracle/pyoracle.py).  They pin the
oracle across hosts (x86_64 here, aarch64 on the GPU machine) and give the
GPU tests fixed expected outputs.

Run from the repository root:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import oracle, pyoracle  # noqa: E402


def case_readme_wrap(rng):
    # README field on a 24x24 grid with a 65-tap kernel: streamlines wrap the
    # periodic image more than once.
    n = 24
    x = np.linspace(0, np.pi, n)
    return dict(
        name="readme_wrap_f64", texture=rng.random((n, n)),
        u=np.broadcast_to(np.cos(2 * x), (n, n)).copy(),
        v=np.broadcast_to(np.sin(x), (n, n)).copy(),
        kernel=1 - np.abs(np.linspace(-1, 1, 65)),
        uv_mode="velocity", bx=("periodic", "periodic"), by=("periodic", "periodic"),
        iterations=1, variant=3, check_python=False,
    )


def case_pol_mixed_f32(rng):
    ny, nx = 13, 17
    u = (rng.random((ny, nx)) - 0.5).astype(np.float32)
    v = (rng.random((ny, nx)) - 0.5).astype(np.float32)
    u[4, 4] = v[4, 4] = 0.0
    u[6, 1] = -0.0
    v[0, 0] = np.nan
    return dict(
        name="pol_mixed_f32", texture=rng.random((ny, nx)).astype(np.float32), u=u, v=v,
        kernel=np.hanning(11).astype(np.float32), uv_mode="polarization",
        bx=("periodic", "periodic"), by=("closed", "closed"), iterations=2, variant=3,
        check_python=True,
    )


def case_variants(rng, variant):
    ny, nx = 9, 10
    u = (rng.random((ny, nx)) - 0.5).astype(np.float32)
    v = np.zeros((ny, nx), dtype=np.float32)
    v[:, ::3] = (rng.random((ny, 4)) - 0.5).astype(np.float32)
    return dict(
        name=f"variant{variant}_f32", texture=rng.random((ny, nx)).astype(np.float32),
        u=u, v=v, kernel=rng.random(7).astype(np.float32), uv_mode="velocity",
        bx=("closed", "closed"), by=("periodic", "periodic"), iterations=1,
        variant=variant, check_python=variant == 3,
    )


def case_even_kernel_f64(rng):
    ny, nx = 8, 5
    return dict(
        name="even_kernel_f64", texture=rng.random((ny, nx)),
        u=rng.normal(size=(ny, nx)), v=rng.normal(size=(ny, nx)),
        kernel=rng.random(6), uv_mode="polarization", bx=("closed", "closed"),
        by=("closed", "closed"), iterations=3, variant=3, check_python=True,
    )


def main() -> None:
    rng = np.random.default_rng(2024)
    cases = [case_readme_wrap(rng), case_pol_mixed_f32(rng), case_even_kernel_f64(rng)]
    cases += [case_variants(rng, var) for var in range(4)]
    for c in cases:
        bnd = (c["bx"], c["by"])
        out = oracle.convolve(
            c["texture"], c["u"], c["v"], c["kernel"], uv_mode=c["uv_mode"], boundaries=bnd,
            iterations=c["iterations"], variant=c["variant"],
        )
        if c["check_python"]:
            want = pyoracle.convolve(
                c["texture"], c["u"], c["v"], c["kernel"], c["uv_mode"], bnd, c["iterations"]
            )
            assert np.array_equal(out, want, equal_nan=True), c["name"]
        ny, nx = c["texture"].shape
        pix = np.arange(ny * nx, dtype=np.int64)
        cells = oracle.paths(c["u"], c["v"], c["kernel"].size, pix, uv_mode=c["uv_mode"],
                             boundaries=bnd, variant=c["variant"])
        np.savez_compressed(
            HERE / f"{c['name']}.npz", texture=c["texture"], u=c["u"], v=c["v"],
            kernel=c["kernel"], uv_mode=np.array(c["uv_mode"]), bx=np.array(c["bx"]),
            by=np.array(c["by"]), iterations=np.array(c["iterations"]),
            variant=np.array(c["variant"]), out=out, pix=pix, cells=cells,
        )
        print("wrote", c["name"])


if __name__ == "__main__":
    main()
