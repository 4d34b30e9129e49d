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
