"""numpy definition of histogram equalization (test infrastructure only).

TEST INFRASTRUCTURE ONLY: imported by the tests, never by the product
package.

The reference declares three equalization functions in its native-module
stubs (neutrinoceros/rlic src/rlic/_core.pyi:30-57:
``equalize_histogram_{f32,f64}(image, nbins)``,
``equalize_histogram_sliding_tile_*(image, nbins, tile_shape)`` and
``equalize_histogram_tile_interpolation_*(image, nbins, tile_shape)``) but
implements none of them: its native core (src/lib.rs) has no such function,
and its README (README.md:19-23) points to the separate ``ahe`` package.
There is therefore no reference output to pin.  This module is the
definition that the GPU implementation (rlic_gb300.equalize) reproduces bit
for bit; every arithmetic step is done in the image's dtype, one rounding
per operation, in the order written here.

Definitions, for an image x of dtype T (float32 or float64) and V the set
of its finite pixels:

* bins: lo = min(x[V]), hi = max(x[V]).  When hi > lo and hi - lo is
  finite, scale = T(nbins) / (hi - lo) and
  bin(p) = min(nbins - 1, floor((x[p] - lo) * scale)); otherwise every
  finite pixel is in bin 0.
* global: out[p] = T(cdf[bin(p)]) / T(|V|), with cdf the inclusive
  cumulative histogram over V.
* sliding tile (th, tw): the window of p is rows
  [i - th//2, i - th//2 + th) and columns [j - tw//2, j - tw//2 + tw),
  clipped to the image; out[p] = T(#{q in window and V: bin(q) <= bin(p)})
  / T(#(window and V)).
* tile interpolation (th, tw): the image is cut into tiles of th x tw
  (the last row and column of tiles ragged); each tile t maps bin k to
  m_t(k) = T(cdf_t[k]) / T(n_t) (0 when the tile has no finite pixel).
  Tile centres are cy_a = (r0 + r1 - 1) / 2 for rows [r0, r1) (columns
  alike).  Pixel row i lies between centre rows a0 = a1 = 0 (i <= cy_0),
  a0 = a1 = last (i >= cy_last), or a0 = the last centre row <= i and
  a1 = a0 + 1 with fy = (i - cy_a0) / (cy_a1 - cy_a0) (fy = 0 when
  a0 = a1); columns alike with fx.  With lerp(u, w, f) = u + f * (w - u),
  out[p] = lerp(lerp(m00, m01, fx), lerp(m10, m11, fx), fy), m_rc the
  mappings of tiles (a_r, c_c) at bin(p).
* non-finite pixels are returned unchanged.
"""

from __future__ import annotations

import numpy as np

STRATEGIES = ("global", "sliding_tile", "tile_interpolation")


def bins(x: np.ndarray, nbins: int) -> np.ndarray:
    """bin(p) as int64, -1 for non-finite pixels."""
    t = x.dtype.type
    fin = np.isfinite(x)
    out = np.full(x.shape, -1, dtype=np.int64)
    if not fin.any():
        return out
    lo, hi = x[fin].min(), x[fin].max()
    with np.errstate(over="ignore"):
        span = t(hi - lo)
    if hi > lo and np.isfinite(span):
        scale = t(t(nbins) / span)
        d = (x[fin] - lo).astype(x.dtype)
        s = np.floor((d * scale).astype(x.dtype))
        out[fin] = np.minimum(s, nbins - 1).astype(np.int64)
    else:
        out[fin] = 0
    return out


def _ratio(num, den, dtype):
    t = np.dtype(dtype).type
    return (np.asarray(num, dtype=np.int64).astype(dtype) / t(den)).astype(dtype) \
        if np.ndim(den) == 0 else \
        (np.asarray(num, dtype=np.int64).astype(dtype) / np.asarray(den).astype(dtype))


def equalize_global(x: np.ndarray, nbins: int) -> np.ndarray:
    b = bins(x, nbins)
    fin = b >= 0
    out = x.copy()
    n = int(fin.sum())
    if n == 0:
        return out
    cdf = np.cumsum(np.bincount(b[fin], minlength=nbins))
    out[fin] = _ratio(cdf[b[fin]], n, x.dtype)
    return out


def equalize_sliding_tile(x: np.ndarray, nbins: int, tile_shape) -> np.ndarray:
    th, tw = (int(s) for s in tile_shape)
    b = bins(x, nbins)
    ny, nx = x.shape
    out = x.copy()
    for i in range(ny):
        r0, r1 = max(0, i - th // 2), min(ny, i - th // 2 + th)
        for j in range(nx):
            if b[i, j] < 0:
                continue
            c0, c1 = max(0, j - tw // 2), min(nx, j - tw // 2 + tw)
            win = b[r0:r1, c0:c1]
            valid = win >= 0
            num = int(np.count_nonzero(valid & (win <= b[i, j])))
            out[i, j] = _ratio(num, int(valid.sum()), x.dtype)
    return out


def _centres(n: int, t: int, dtype) -> np.ndarray:
    starts = np.arange(0, n, t)
    ends = np.minimum(starts + t, n)
    return ((starts + ends - 1).astype(dtype) / np.dtype(dtype).type(2)).astype(dtype)


def _interp_axis(idx: np.ndarray, centres: np.ndarray, dtype):
    """(a0, a1, f) for positions idx against the tile centres."""
    t = np.dtype(dtype).type
    pos = idx.astype(dtype)
    last = len(centres) - 1
    a0 = np.clip(np.searchsorted(centres, pos, side="right") - 1, 0, last)
    a1 = np.minimum(a0 + 1, last)
    inside = (pos > centres[0]) & (pos < centres[last])
    a1 = np.where(inside, a1, a0)
    f = np.zeros(idx.shape, dtype=dtype)
    num = (pos - centres[a0]).astype(dtype)
    den = (centres[a1] - centres[a0]).astype(dtype)
    f[inside] = (num[inside] / den[inside]).astype(dtype)
    return a0, a1, f.astype(dtype), t


def equalize_tile_interpolation(x: np.ndarray, nbins: int, tile_shape) -> np.ndarray:
    th, tw = (int(s) for s in tile_shape)
    dt = x.dtype
    b = bins(x, nbins)
    ny, nx = x.shape
    na, nc = -(-ny // th), -(-nx // tw)
    maps = np.zeros((na, nc, nbins), dtype=dt)
    for a in range(na):
        for c in range(nc):
            tb = b[a * th:(a + 1) * th, c * tw:(c + 1) * tw]
            tb = tb[tb >= 0]
            if tb.size:
                cdf = np.cumsum(np.bincount(tb, minlength=nbins))
                maps[a, c] = _ratio(cdf, tb.size, dt)
    ra0, ra1, fy, t = _interp_axis(np.arange(ny), _centres(ny, th, dt), dt)
    ca0, ca1, fx, _ = _interp_axis(np.arange(nx), _centres(nx, tw, dt), dt)
    out = x.copy()
    fin = b >= 0
    ii, jj = np.nonzero(fin)
    k = b[ii, jj]

    def lerp(u, w, f):
        return (u + (f * (w - u).astype(dt)).astype(dt)).astype(dt)

    m00 = maps[ra0[ii], ca0[jj], k]
    m01 = maps[ra0[ii], ca1[jj], k]
    m10 = maps[ra1[ii], ca0[jj], k]
    m11 = maps[ra1[ii], ca1[jj], k]
    top = lerp(m00, m01, fx[jj])
    bot = lerp(m10, m11, fx[jj])
    out[ii, jj] = lerp(top, bot, fy[ii])
    return out


def equalize(x: np.ndarray, nbins: int, strategy: str = "global", tile_shape=None) -> np.ndarray:
    if strategy == "global":
        return equalize_global(x, nbins)
    if strategy == "sliding_tile":
        return equalize_sliding_tile(x, nbins, tile_shape)
    if strategy == "tile_interpolation":
        return equalize_tile_interpolation(x, nbins, tile_shape)
    raise ValueError(strategy)
