"""ctypes wrapper of the CPU oracle ``liblic_oracle.so`` (lic_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, the smoke check and the
CPU-baseline leg of bench.py, never by the product package.

The oracle restates the reference's native core (neutrinoceros/rlic
src/lib.rs:157-443) in C; see lic_oracle.c for the line-by-line mapping.
``variant`` selects the reference's Cargo feature set: bit 0 = ``fma``,
bit 1 = ``branchless``; 3 (both, the reference's default) is the parity
target.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liblic_oracle.so"

VARIANT_FMA = 1
VARIANT_BRANCHLESS = 2
DEFAULT_VARIANT = VARIANT_FMA | VARIANT_BRANCHLESS

BOUNDARY_CODES = {"closed": 0, "periodic": 1}

_lib: ctypes.CDLL | None = None


def build(force: bool = False) -> Path:
    """Compile liblic_oracle.so with the Makefile next to this file."""
    src = ORACLE_DIR / "lic_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        cmd = ["make", "-s", "-C", str(ORACLE_DIR)]
        if force:
            cmd.append("-B")
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            # retry without OpenMP (a host compiler without libgomp)
            res = subprocess.run(cmd + ["OMPFLAGS="], capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        P, I64, INT, U = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_uint
        for s, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            f = getattr(L, f"lic_oracle_convolve_{s}")
            f.argtypes = [P, P, P, I64, I64, P, I64, INT, INT, INT, INT, INT, I64, P, U, INT]
            f.restype = INT
            f = getattr(L, f"lic_oracle_sweep_rows_{s}")
            f.argtypes = [P, P, P, I64, I64, P, I64, INT, INT, INT, INT, INT, I64, I64, P, U, INT]
            f.restype = INT
            f = getattr(L, f"lic_oracle_paths_{s}")
            f.argtypes = [P, P, I64, I64, I64, INT, INT, INT, INT, INT, I64, P, P, U]
            f.restype = INT
            f = getattr(L, f"lic_oracle_time_to_next_pixel_{s}")
            f.argtypes = [ct, ct, U]
            f.restype = ct
        L.lic_oracle_advance_state_f64.argtypes = [
            ctypes.c_double, ctypes.c_double, P, P, P, P, I64, I64, INT, INT, INT, INT, U,
        ]
        L.lic_oracle_advance_state_f64.restype = INT
        L.lic_oracle_num_threads.restype = INT
        _lib = L
    return _lib


def _suffix(dtype: np.dtype) -> str:
    if dtype == np.float32:
        return "f32"
    if dtype == np.float64:
        return "f64"
    raise TypeError(f"oracle supports float32/float64, got {dtype}")


def _bcodes(boundaries) -> tuple[int, int, int, int]:
    """Accepts 'closed'/'periodic', {'x':..,'y':..} or ((xl,xr),(yl,yr))."""
    if isinstance(boundaries, str):
        c = BOUNDARY_CODES[boundaries]
        return (c, c, c, c)
    if isinstance(boundaries, dict):
        def pair(b):
            return (b, b) if isinstance(b, str) else tuple(b)
        (xl, xr), (yl, yr) = pair(boundaries["x"]), pair(boundaries["y"])
    else:
        (xl, xr), (yl, yr) = boundaries
    return tuple(BOUNDARY_CODES[b] for b in (xl, xr, yl, yr))  # type: ignore[return-value]


def max_threads() -> int:
    return int(lib().lic_oracle_num_threads())


def convolve(texture, u, v, kernel, *, uv_mode="velocity", boundaries="closed", iterations=1,
             variant=DEFAULT_VARIANT, nthreads=1) -> np.ndarray:
    """convolve_iteratively (src/lib.rs:408-443); iterations <= 0 gives zeros."""
    dtype = np.asarray(texture).dtype
    s = _suffix(dtype)
    tex = np.ascontiguousarray(texture, dtype=dtype)
    uu = np.ascontiguousarray(u, dtype=dtype)
    vv = np.ascontiguousarray(v, dtype=dtype)
    kk = np.ascontiguousarray(kernel, dtype=dtype)
    out = np.empty_like(tex)
    ny, nx = tex.shape
    rc = getattr(lib(), f"lic_oracle_convolve_{s}")(
        tex.ctypes.data, uu.ctypes.data, vv.ctypes.data, ny, nx, kk.ctypes.data, kk.size,
        int(uv_mode == "polarization"), *_bcodes(boundaries), int(iterations),
        out.ctypes.data, int(variant), int(nthreads),
    )
    if rc != 0:
        raise RuntimeError(f"oracle convolve failed: {rc}")
    return out


def sweep_rows(texture, u, v, kernel, row0, row1, *, uv_mode="velocity", boundaries="closed",
               variant=DEFAULT_VARIANT, nthreads=1) -> np.ndarray:
    """One pass over rows [row0, row1) of the full image (CPU baseline sampling)."""
    dtype = np.asarray(texture).dtype
    s = _suffix(dtype)
    tex = np.ascontiguousarray(texture, dtype=dtype)
    uu = np.ascontiguousarray(u, dtype=dtype)
    vv = np.ascontiguousarray(v, dtype=dtype)
    kk = np.ascontiguousarray(kernel, dtype=dtype)
    ny, nx = tex.shape
    out = np.empty((row1 - row0, nx), dtype=dtype)
    rc = getattr(lib(), f"lic_oracle_sweep_rows_{s}")(
        tex.ctypes.data, uu.ctypes.data, vv.ctypes.data, ny, nx, kk.ctypes.data, kk.size,
        int(uv_mode == "polarization"), *_bcodes(boundaries), int(row0), int(row1),
        out.ctypes.data, int(variant), int(nthreads),
    )
    if rc != 0:
        raise RuntimeError(f"oracle sweep_rows failed: {rc}")
    return out


def convolve_rows(texture, u, v, kernel, row0, row1, *, uv_mode="velocity",
                  boundaries="closed", iterations=1, variant=DEFAULT_VARIANT,
                  nthreads=1) -> np.ndarray:
    """Rows [row0, row1) of ``convolve(..., iterations)``, computed exactly from
    bands of rows.

    A streamline moves at most klen // 2 rows away from its pixel (one cell
    per step, src/lib.rs:325-329), so rows [row0, row1) of pass p depend only
    on rows [row0 - r, row1 + r) of pass p - 1, r = klen // 2.  Pass p is
    therefore evaluated on rows [row0 - (n - p) r, row1 + (n - p) r) only.
    With a closed y axis the band is clipped to the image (no streamline
    crosses a closed edge); with a periodic one, a band that would cross the
    seam is widened to the whole image.  Rows outside each band hold NaN, so
    that a read outside it would show in the result.
    """
    dtype = np.asarray(texture).dtype
    tex = np.ascontiguousarray(texture, dtype=dtype)
    ny, nx = tex.shape
    if iterations <= 0:
        return np.zeros((row1 - row0, nx), dtype=dtype)
    r = int(np.asarray(kernel).size) // 2
    yl, yr = _bcodes(boundaries)[2:]
    periodic_y = BOUNDARY_CODES["periodic"] in (yl, yr)
    cur = tex
    for p in range(1, iterations + 1):
        m = (iterations - p) * r
        a, b = row0 - m, row1 + m
        if periodic_y and (a < 0 or b > ny):
            a, b = 0, ny
        a, b = max(0, a), min(ny, b)
        nxt = np.full_like(tex, np.nan)
        nxt[a:b] = sweep_rows(cur, u, v, kernel, a, b, uv_mode=uv_mode, boundaries=boundaries,
                              variant=variant, nthreads=nthreads)
        cur = nxt
    return cur[row0:row1].copy()


def paths(u, v, klen, pix, *, uv_mode="velocity", boundaries="closed",
          variant=DEFAULT_VARIANT) -> np.ndarray:
    """(npix, klen-1) int64 linear cells: forward trace, then backward; -1 after a stop."""
    dtype = np.asarray(u).dtype
    s = _suffix(dtype)
    uu = np.ascontiguousarray(u, dtype=dtype)
    vv = np.ascontiguousarray(v, dtype=dtype)
    px = np.ascontiguousarray(pix, dtype=np.int64)
    ny, nx = uu.shape
    cells = np.full((px.size, max(klen - 1, 0)), -1, dtype=np.int64)
    rc = getattr(lib(), f"lic_oracle_paths_{s}")(
        uu.ctypes.data, vv.ctypes.data, ny, nx, int(klen), int(uv_mode == "polarization"),
        *_bcodes(boundaries), px.size, px.ctypes.data, cells.ctypes.data, int(variant),
    )
    if rc != 0:
        raise RuntimeError(f"oracle paths failed: {rc}")
    return cells


def time_to_next_pixel(velocity, frac, dtype=np.float64, variant=DEFAULT_VARIANT):
    """time_to_next_pixel (src/lib.rs:157-180) on one scalar pair."""
    s = _suffix(np.dtype(dtype))
    return getattr(lib(), f"lic_oracle_time_to_next_pixel_{s}")(velocity, frac, int(variant))


def advance(u, v, i, j, fx, fy, shape, boundaries="closed", variant=DEFAULT_VARIANT):
    """advance (src/lib.rs:236-273) on one f64 state; returns (i, j, fx, fy)."""
    ci, cj = ctypes.c_int64(i), ctypes.c_int64(j)
    cfx, cfy = ctypes.c_double(fx), ctypes.c_double(fy)
    ny, nx = shape
    lib().lic_oracle_advance_state_f64(
        u, v, ctypes.byref(ci), ctypes.byref(cj), ctypes.byref(cfx), ctypes.byref(cfy),
        ny, nx, *_bcodes(boundaries), int(variant),
    )
    return ci.value, cj.value, cfx.value, cfy.value


def env_threads() -> int:
    """Host threads for the multi-core baseline (all cores unless limited)."""
    return int(os.environ.get("RLIC_ORACLE_THREADS", os.cpu_count() or 1))
