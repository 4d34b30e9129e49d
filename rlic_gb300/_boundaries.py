"""Boundary specifications: normalisation and validation.

Mirrors the reference's ``rlic._boundaries`` (src/rlic/_boundaries.py:1-114):
the same public names (``BoundarySet``, ``BoundarySpec``, ``BoundaryStr``,
``SUPPORTED_BOUNDS``, ``COMBO_ALLOWED_BOUNDS``, ``COMBO_DISALLOWED_BOUNDS``),
the same accepted spec shapes and the same error texts, because the
reference's tests import and exercise this module directly
(tests/test_boundaries.py:7-13).

A spec is either one boundary name for all four sides, or a mapping with
exactly the keys ``"x"`` and ``"y"`` whose values are a name or a
``(left, right)`` pair of names.
"""

from __future__ import annotations

__all__ = [
    "COMBO_ALLOWED_BOUNDS",
    "COMBO_DISALLOWED_BOUNDS",
    "SUPPORTED_BOUNDS",
    "BoundarySet",
]

from collections.abc import Mapping, Sequence
from dataclasses import dataclass
from typing import TYPE_CHECKING, Literal, TypeAlias, TypedDict

if TYPE_CHECKING:
    from rlic_gb300._typing import Pair, PairSpec

BoundaryStr: TypeAlias = Literal["closed", "periodic"]


class BoundaryDictSpec(TypedDict):
    x: PairSpec[BoundaryStr]
    y: PairSpec[BoundaryStr]


BoundarySpec: TypeAlias = BoundaryStr | BoundaryDictSpec

# a "closed" side may face any other kind (src/rlic/_boundaries.py:29-30)
COMBO_ALLOWED_BOUNDS: frozenset[str] = frozenset({"closed"})
# a "periodic" side must face another "periodic" side (src/rlic/_boundaries.py:31-32)
COMBO_DISALLOWED_BOUNDS: frozenset[str] = frozenset({"periodic"})
SUPPORTED_BOUNDS: frozenset[str] = COMBO_ALLOWED_BOUNDS | COMBO_DISALLOWED_BOUNDS

# numeric codes of the C ABI (include/rlic_gb300.h)
BOUNDARY_CODES: dict[str, int] = {"closed": 0, "periodic": 1}

_MSG_UNKNOWN = "Unknown {side} {ax} boundary {name!r}"
_MSG_COMBO = (
    "{side} {ax} boundary {name!r} cannot be combined with a different boundary ({other!r})"
)


def _side_pair(value: object) -> tuple[str, str] | None:
    """One axis of a spec: a name, or a 2-sequence of names (not a str)."""
    if isinstance(value, str):
        return (value, value)
    if (
        isinstance(value, Sequence)
        and not isinstance(value, (bytes, bytearray))
        and len(value) == 2
        and all(isinstance(b, str) for b in value)
    ):
        return (value[0], value[1])
    return None


def as_pair(b: PairSpec[BoundaryStr], /) -> Pair[BoundaryStr]:
    """Expand one axis spec to a ``(left, right)`` tuple (src/rlic/_boundaries.py:38-45)."""
    pair = _side_pair(b)
    if pair is None:
        raise AssertionError(f"not a boundary pair spec: {b!r}")
    return pair  # type: ignore[return-value]


@dataclass(frozen=True, slots=True, kw_only=True)
class BoundarySet:
    """Boundary kinds of both axes, as ``(left, right)`` pairs."""

    x: Pair[BoundaryStr]
    y: Pair[BoundaryStr]

    @staticmethod
    def from_spec(spec: BoundarySpec, /) -> BoundarySet | None:
        """Normalise a spec; ``None`` when its structure is invalid.

        Names are not checked here (src/rlic/_boundaries.py:53-67): any
        string passes, and collect_exceptions() reports unknown ones.
        """
        if isinstance(spec, str):
            return BoundarySet(x=(spec, spec), y=(spec, spec))  # type: ignore[arg-type]
        if isinstance(spec, Mapping) and len(spec) == 2 and "x" in spec and "y" in spec:
            bx = _side_pair(spec["x"])
            by = _side_pair(spec["y"])
            if bx is not None and by is not None:
                return BoundarySet(x=bx, y=by)  # type: ignore[arg-type]
        return None

    def collect_exceptions(self) -> list[Exception]:
        """Every problem with the names and combinations, in reference order.

        Per axis (x first): an axis of two combinable kinds is fine; when
        both names are known, a periodic side facing a different kind is
        reported (left first); otherwise each unknown name is reported
        (src/rlic/_boundaries.py:69-105).
        """
        found: list[Exception] = []
        for ax, sides in (("x", self.x), ("y", self.y)):
            left, right = sides
            names = {left, right}
            if names <= COMBO_ALLOWED_BOUNDS:
                continue
            if names <= SUPPORTED_BOUNDS:
                if left == right:
                    continue
                for side, name, other in (("left", left, right), ("right", right, left)):
                    if name in COMBO_DISALLOWED_BOUNDS:
                        found.append(
                            ValueError(
                                _MSG_COMBO.format(side=side, ax=ax, name=name, other=other)
                            )
                        )
            else:
                for side, name in (("left", left), ("right", right)):
                    if name not in SUPPORTED_BOUNDS:
                        found.append(
                            ValueError(_MSG_UNKNOWN.format(side=side, ax=ax, name=name))
                        )
        return found

    def validate(self) -> None:
        """Raise the single problem, or all of them as an ExceptionGroup."""
        found = self.collect_exceptions()
        if len(found) == 1:
            raise found[0]
        if found:
            raise ExceptionGroup("Found multiple issues with boundary specifications", found)

    def codes(self) -> tuple[int, int, int, int]:
        """(x_left, x_right, y_left, y_right) as C-ABI boundary codes."""
        (xl, xr), (yl, yr) = self.x, self.y
        return (
            BOUNDARY_CODES[xl],
            BOUNDARY_CODES[xr],
            BOUNDARY_CODES[yl],
            BOUNDARY_CODES[yr],
        )
