"""BoundarySet normalisation and validation (reference: tests/test_boundaries.py)."""

from __future__ import annotations

from dataclasses import replace
from itertools import permutations, product

import pytest
from pytest import RaisesExc, RaisesGroup

from rlic._boundaries import (
    COMBO_ALLOWED_BOUNDS,
    COMBO_DISALLOWED_BOUNDS,
    SUPPORTED_BOUNDS,
    BoundarySet,
)


@pytest.mark.parametrize(
    "spec, expected",
    [
        ("a", BoundarySet(x=("a", "a"), y=("a", "a"))),
        ({"x": "a", "y": "b"}, BoundarySet(x=("a", "a"), y=("b", "b"))),
        ({"x": ("a", "b"), "y": ("c", "w")}, BoundarySet(x=("a", "b"), y=("c", "w"))),
        ({"x": ["a", "b"], "y": ["c", "w"]}, BoundarySet(x=("a", "b"), y=("c", "w"))),
        ({"y": "b", "x": ("a", "c")}, BoundarySet(x=("a", "c"), y=("b", "b"))),
    ],
)
def test_from_spec(spec, expected) -> None:
    assert BoundarySet.from_spec(spec) == expected


@pytest.mark.parametrize(
    "spec",
    [123, None, ["a", "b"], {"x": "a"}, {"y": "b"}, {"x": "a", "y": "b", "z": "c"},
     {"x": ("a", "b", "c"), "y": "b"}, {"x": ("a", 1), "y": "b"}, {"x": b"ab", "y": "b"}],
)
def test_from_spec_invalid_structure(spec) -> None:
    assert BoundarySet.from_spec(spec) is None


@pytest.mark.parametrize("b1, b2", list(product(SUPPORTED_BOUNDS, SUPPORTED_BOUNDS)))
def test_uniform_axes_are_valid(b1, b2) -> None:
    bs = BoundarySet(x=(b1, b1), y=(b2, b2))
    assert not bs.collect_exceptions()
    assert bs.validate() is None


@pytest.mark.parametrize(
    "b1, b2", [(a, b) for a, b in product(COMBO_DISALLOWED_BOUNDS, SUPPORTED_BOUNDS) if a != b]
)
def test_periodic_facing_other_kind(b1, b2) -> None:
    bs = BoundarySet(x=(b1, b2), y=(b1, b1))
    with pytest.raises(ValueError, match=r"^left x boundary '\w+' cannot be combined"):
        bs.validate()
    with pytest.raises(ValueError, match=r"^right x boundary '\w+' cannot be combined"):
        replace(bs, x=reversed(bs.x)).validate()
    swapped = BoundarySet(x=bs.y, y=bs.x)
    with pytest.raises(ValueError, match=r"^left y boundary '\w+' cannot be combined"):
        swapped.validate()
    with pytest.raises(ValueError, match=r"^right y boundary '\w+' cannot be combined"):
        replace(swapped, y=reversed(swapped.y)).validate()


def test_combo_message_text() -> None:
    with pytest.raises(
        ValueError,
        match=r"^left x boundary 'periodic' cannot be combined with a different boundary \('closed'\)$",
    ):
        BoundarySet(x=("periodic", "closed"), y=("closed", "closed")).validate()


@pytest.mark.parametrize(
    "sides", sorted(set(permutations(("periodic", "periodic", "periodic", "unknown"))))
)
def test_unknown_name(sides) -> None:
    b1, b2, b3, b4 = sides
    with pytest.raises(ValueError, match=r"^Unknown (left|right) (x|y) boundary 'unknown'$"):
        BoundarySet(x=(b1, b2), y=(b3, b4)).validate()


def test_multiple_errors() -> None:
    with RaisesGroup(
        RaisesExc(ValueError, match=r"^Unknown left x boundary 'unknown'$"),
        RaisesExc(ValueError, match=r"^left y boundary 'periodic' cannot be combined"),
        match="Found multiple issues with boundary specifications",
    ):
        BoundarySet(x=("unknown", "periodic"), y=("periodic", "closed")).validate()


def test_codes() -> None:
    bs = BoundarySet.from_spec({"x": "periodic", "y": ("closed", "closed")})
    assert bs.codes() == (1, 1, 0, 0)
    assert COMBO_ALLOWED_BOUNDS | COMBO_DISALLOWED_BOUNDS == SUPPORTED_BOUNDS
