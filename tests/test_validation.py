"""Input validation of ``rlic.convolve``: same errors, texts and grouping as the
reference (tests/test_exceptions.py:14-205 of neutrinoceros/rlic).

Validation runs before any native call, so these tests need no GPU.  They go
through the ``rlic`` alias package to show that code written against the
reference imports and behaves the same.
"""

from __future__ import annotations

import numpy as np
import pytest
from pytest import RaisesExc, RaisesGroup

import rlic

img = np.eye(64)
u = img.copy()
v = img.copy()
kernel = np.linspace(0, 1, 10, dtype="float64")


def test_invalid_iterations() -> None:
    with pytest.raises(
        ValueError,
        match=r"^Invalid number of iterations: -1\nExpected a strictly positive integer\.$",
    ):
        rlic.convolve(img, u, v, kernel=kernel, iterations=-1)


def test_invalid_uv_mode() -> None:
    with pytest.raises(
        ValueError,
        match=r"^Invalid uv_mode 'astral'\. Expected one of \['velocity', 'polarization'\]$",
    ):
        rlic.convolve(img, u, v, kernel=kernel, uv_mode="astral")


def test_texture_ndim_and_shape_grouped() -> None:
    with RaisesGroup(
        RaisesExc(
            ValueError,
            match=r"^Expected a texture with exactly two dimensions\. Got texture\.ndim=3$",
        ),
        RaisesExc(
            ValueError,
            match=r"^Shape mismatch: expected texture, u and v with identical shapes\.",
        ),
        match=r"^Invalid inputs were received\.",
    ):
        rlic.convolve(np.ones((16, 16, 16)), u, v, kernel=kernel)


def test_negative_texture() -> None:
    with pytest.raises(
        ValueError,
        match=r"^Found invalid texture element\(s\)\. Expected only positive values\.$",
    ):
        rlic.convolve(-np.ones((64, 64)), v, v, kernel=kernel)


@pytest.mark.parametrize(
    "tshape, ushape, vshape",
    [((64, 64), (65, 64), (64, 64)), ((64, 64), (64, 64), (63, 64)), ((64, 66), (64, 64), (64, 64))],
)
def test_mismatched_shapes(tshape, ushape, vshape) -> None:
    rng = np.random.default_rng(0)
    t, uu, vv = rng.random(tshape), rng.random(ushape), rng.random(vshape)
    with pytest.raises(
        ValueError,
        match=(
            r"^Shape mismatch: expected texture, u and v with identical shapes\. "
            rf"Got texture.shape=\({tshape[0]}, {tshape[1]}\), "
            rf"u.shape=\({ushape[0]}, {ushape[1]}\), "
            rf"v.shape=\({vshape[0]}, {vshape[1]}\)$"
        ),
    ):
        rlic.convolve(t, uu, vv, kernel=kernel)


def test_kernel_ndim() -> None:
    with pytest.raises(
        ValueError, match=r"^Expected a kernel with exactly one dimension\. Got kernel\.ndim=2$"
    ):
        rlic.convolve(img, u, v, kernel=np.ones((5, 5)))


@pytest.mark.parametrize("bad", [-np.inf, np.inf, np.nan])
def test_non_finite_kernel(bad) -> None:
    k = np.ones(11)
    k[5] = bad
    with pytest.raises(ValueError, match=r"^Found non-finite value\(s\) in kernel\.$"):
        rlic.convolve(img, u, v, kernel=k)


def test_unsupported_texture_dtype() -> None:
    with RaisesGroup(
        RaisesExc(
            TypeError,
            match=(
                r"^Found unsupported data type\(s\): \[dtype\('complex128'\)\]\. "
                r"Expected texture, u, v and kernel with identical dtype, from "
                r"\[dtype\('float32'\), dtype\('float64'\)\]\. "
                r"Got texture\.dtype=dtype\('complex128'\), u\.dtype=dtype\('float64'\), "
                r"v\.dtype=dtype\('float64'\), kernel\.dtype=dtype\('float64'\)$"
            ),
        ),
        RaisesExc(TypeError, match=r"^Data types mismatch"),
        match=r"^Invalid inputs were received\.",
    ):
        rlic.convolve(np.ones((64, 64), dtype="complex128"), u, v, kernel=kernel)


def test_unsupported_kernel_dtype() -> None:
    with RaisesGroup(
        RaisesExc(TypeError, match=r"^Found unsupported data type\(s\): \[dtype\('complex128'\)\]"),
        RaisesExc(TypeError, match=r"^Data types mismatch"),
        match=r"^Invalid inputs were received\.",
    ):
        rlic.convolve(img, u, v, kernel=-np.ones(5, dtype="complex128"))


def test_mismatched_dtypes() -> None:
    with pytest.raises(
        TypeError,
        match=(
            r"^Data types mismatch. "
            r"Expected texture, u, v and kernel with identical dtype, from "
            r"\[dtype\('float32'\), dtype\('float64'\)\]\. "
            r"Got texture\.dtype=dtype\('float32'\), u\.dtype=dtype\('float64'\), "
            r"v\.dtype=dtype\('float64'\), kernel\.dtype=dtype\('float64'\)$"
        ),
    ):
        rlic.convolve(np.ones((64, 64), dtype="float32"), u, v, kernel=kernel)


def test_validators_run_before_zero_iteration_copy() -> None:
    with pytest.raises(ValueError, match=r"^Found non-finite value\(s\) in kernel\.$"):
        rlic.convolve(img, u, v, kernel=np.full(11, np.nan), iterations=0)


def test_invalid_boundary_type() -> None:
    with pytest.raises(TypeError, match=r"^Invalid boundary specification "):
        rlic.convolve(img, u, v, kernel=kernel, boundaries=None)


def test_invalid_boundary_names_grouped_with_other_errors() -> None:
    with RaisesGroup(
        RaisesExc(ValueError, match=r"^Invalid number of iterations"),
        RaisesExc(ValueError, match=r"^Unknown left x boundary 'wall'$"),
        RaisesExc(ValueError, match=r"^left y boundary 'periodic' cannot be combined"),
        match=r"^Invalid inputs were received\.",
    ):
        rlic.convolve(
            img, u, v, kernel=kernel, iterations=-2,
            boundaries={"x": ("wall", "closed"), "y": ("periodic", "closed")},
        )


def test_zero_iterations_returns_new_copy() -> None:
    t = np.random.default_rng(3).random((8, 9))
    out = rlic.convolve(t, t, t, kernel=np.ones(3), iterations=0)
    np.testing.assert_array_equal(out, t)
    assert out is not t and not np.shares_memory(out, t)


@pytest.mark.parametrize("shape", [(0, 5), (7, 0), (0, 0)])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("klen", [0, 3])
def test_image_without_pixels_gives_an_empty_result(shape, dtype, klen) -> None:
    # the native core's pixel loops run zero times (src/lib.rs:373-374), so the
    # call returns a new empty array, even for an empty kernel; needs the
    # library (loaded, never launched), not a GPU
    t = np.zeros(shape, dtype=dtype)
    out = rlic.convolve(t, t, t, kernel=np.ones(klen, dtype=dtype), iterations=3,
                        uv_mode="polarization", boundaries="periodic")
    assert out.shape == shape and out.dtype == np.dtype(dtype)
    assert out is not t


def test_alias_modules_match_package() -> None:
    import rlic._boundaries
    import rlic._typing
    import rlic_gb300._boundaries
    import rlic_gb300._typing

    assert rlic._boundaries.BoundarySet is rlic_gb300._boundaries.BoundarySet
    assert rlic._typing.F is rlic_gb300._typing.F
    assert rlic.convolve is rlic_gb300.convolve
