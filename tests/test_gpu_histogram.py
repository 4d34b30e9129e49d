"""Histogram equalization on the GPU against its numpy definition, bit for bit.

Global, sliding-tile and tile-interpolation forms, float32 and float64,
through numpy (host copies) and CUDA tensors; odd shapes, ragged tiles,
tiles and windows larger than the image, non-finite pixels, constant
images, one bin and many bins; then an 8192^2 float32 image against
size-independent properties (the global form's value counts are the
histogram's).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import histogram as H
from rlic_gb300 import equalize as E

pytestmark = pytest.mark.gpu


def _bits(a):
    a = np.asarray(a)
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def assert_bitwise(got, want):
    got = got.cpu().numpy() if hasattr(got, "cpu") else np.asarray(got)
    assert got.dtype == want.dtype and got.shape == want.shape
    bad = _bits(got) != _bits(want)
    assert not bad.any(), (np.argwhere(bad)[:5], got[bad][:5], want[bad][:5])


def _image(rng, shape, dtype, specials=True):
    x = (rng.normal(size=shape) * 3 + rng.uniform(-2, 2)).astype(dtype)
    if specials and x.size > 8:
        flat = x.reshape(-1)
        k = rng.choice(x.size, 4, replace=False)
        flat[k[0]] = np.nan
        flat[k[1]] = np.inf
        flat[k[2]] = -np.inf
        flat[k[3]] = -0.0
    return x


CASES = [
    ((37, 53), 64, (8, 8)),
    ((64, 64), 256, (16, 16)),
    ((17, 90), 7, (5, 11)),     # ragged tiles
    ((1, 40), 16, (1, 7)),
    ((33, 1), 16, (4, 1)),
    ((20, 25), 1, (3, 3)),      # one bin
    ((30, 30), 5000, (64, 64)),  # many bins, tiles larger than the image
]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape, nbins, tile", CASES, ids=lambda c: str(c).replace(" ", ""))
def test_matches_definition(dtype, shape, nbins, tile) -> None:
    rng = np.random.default_rng(abs(hash((shape, nbins, tile))) % 2**32)
    x = _image(rng, shape, dtype)
    assert_bitwise(E.equalize_histogram(x, nbins), H.equalize_global(x, nbins))
    assert_bitwise(E.equalize_histogram_sliding_tile(x, nbins, tile),
                   H.equalize_sliding_tile(x, nbins, tile))
    assert_bitwise(E.equalize_histogram_tile_interpolation(x, nbins, tile),
                   H.equalize_tile_interpolation(x, nbins, tile))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_torch_tensors_and_stub_names(dtype) -> None:
    import torch

    rng = np.random.default_rng(3)
    x = _image(rng, (48, 40), dtype)
    t = torch.from_numpy(x).cuda()
    sfx = "f32" if dtype == np.float32 else "f64"
    g = getattr(E, f"equalize_histogram_{sfx}")(t, 32)
    assert g.is_cuda and g.dtype == t.dtype
    assert_bitwise(g, H.equalize_global(x, 32))
    assert_bitwise(getattr(E, f"equalize_histogram_sliding_tile_{sfx}")(t, 32, (9, 7)),
                   H.equalize_sliding_tile(x, 32, (9, 7)))
    assert_bitwise(getattr(E, f"equalize_histogram_tile_interpolation_{sfx}")(t, 32, (10, 6)),
                   H.equalize_tile_interpolation(x, 32, (10, 6)))


def test_constant_nonfinite_and_wide_range_images() -> None:
    c = np.full((9, 11), -2.25, dtype=np.float64)
    assert_bitwise(E.equalize_histogram(c, 16), H.equalize_global(c, 16))
    allnan = np.full((5, 5), np.nan, dtype=np.float32)
    assert_bitwise(E.equalize_histogram_tile_interpolation(allnan, 4, (2, 2)), allnan)
    wide = np.array([[-1e308, 0.0, 1e308, 5.0]])  # max - min overflows: one bin
    assert_bitwise(E.equalize_histogram(wide, 10), H.equalize_global(wide, 10))


def test_full_size_global_properties() -> None:
    import torch

    n, nbins = 8192, 256
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((n, n), generator=gen, device="cuda", dtype=torch.float32) ** 3
    out = E.equalize_histogram(x, nbins)
    # the output takes one value per non-empty bin: cdf / count, increasing
    vals, counts = torch.unique(out, return_counts=True)
    assert vals[-1].item() == 1.0
    cdf = torch.cumsum(counts, 0).to(torch.float64)
    torch.testing.assert_close(vals.double(), cdf / (n * n), rtol=1e-6, atol=0)
    assert len(vals) <= nbins


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("window", [(65, 65), (33, 17), (4, 9)], ids=str)
def test_sliding_tile_large_windows(dtype, window) -> None:
    """Windows of up to 65 x 65 cells on a 200 x 260 image (several CTA
    tiles of 32 x 32 pixels, rows below the last tile row), with and without
    non-finite pixels."""
    rng = np.random.default_rng(7)
    for specials in (False, True):
        x = _image(rng, (200, 260), dtype, specials=specials)
        assert_bitwise(E.equalize_histogram_sliding_tile(x, 256, window),
                       H.equalize_sliding_tile(x, 256, window))


def _sliding_by_box_sums(x, nbins, window):
    """The sliding-tile definition of oracle/histogram.py evaluated with box
    sums of indicator images (one per bin level): the same counts, so the
    same roundings, at a cost independent of the window size."""
    th, tw = window
    b = H.bins(x, nbins)
    ny, nx = x.shape

    def box(ind):
        c = np.zeros((ny + 1, nx + 1), dtype=np.int64)
        c[1:, 1:] = np.cumsum(np.cumsum(ind.astype(np.int64), 0), 1)
        i = np.arange(ny)[:, None]
        j = np.arange(nx)[None, :]
        r0, r1 = np.clip(i - th // 2, 0, ny), np.clip(i - th // 2 + th, 0, ny)
        c0, c1 = np.clip(j - tw // 2, 0, nx), np.clip(j - tw // 2 + tw, 0, nx)
        return c[r1, c1] - c[r0, c1] - c[r1, c0] + c[r0, c0]

    valid = box(b >= 0)
    below = np.zeros_like(valid)
    for k in range(nbins):
        below = np.where(b == k, box((b >= 0) & (b <= k)), below)
    out = x.copy()
    fin = b >= 0
    out[fin] = (below[fin].astype(x.dtype) / valid[fin].astype(x.dtype)).astype(x.dtype)
    return out


def test_box_sum_restatement_matches_definition() -> None:
    rng = np.random.default_rng(5)
    x = _image(rng, (40, 50), np.float32)
    for nbins, window in ((2, (9, 13)), (3, (64, 7))):
        assert_bitwise(_sliding_by_box_sums(x, nbins, window),
                       H.equalize_sliding_tile(x, nbins, window))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("nbins, window", [(2, (255, 257)), (1, (255, 257)), (2, (257, 257))],
                         ids=str)
def test_sliding_tile_histogram_limits(dtype, nbins, window) -> None:
    """Windows of 65535 cells, the most the running window histograms hold
    (with one or two bins a bin's count reaches the 16-bit limit), and one
    of 66049 cells, which counts every window cell per pixel instead, on a
    300 x 300 image with and without non-finite pixels."""
    rng = np.random.default_rng(11)
    for specials in (False, True):
        x = _image(rng, (300, 300), dtype, specials=specials)
        assert_bitwise(E.equalize_histogram_sliding_tile(x, nbins, window),
                       _sliding_by_box_sums(x, nbins, window))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sliding_tile_many_bins(dtype) -> None:
    """More than 256 bins: counted per window cell."""
    rng = np.random.default_rng(12)
    x = _image(rng, (60, 70), dtype)
    assert_bitwise(E.equalize_histogram_sliding_tile(x, 300, (9, 9)),
                   H.equalize_sliding_tile(x, 300, (9, 9)))
