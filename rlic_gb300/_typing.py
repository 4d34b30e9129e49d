"""Type aliases of the public API.

Same names and meanings as the reference's ``rlic._typing``
(src/rlic/_typing.py:1-37), which its test-suite imports
(tests/test_convolution.py:11, tests/test_exceptions.py:6,
tests/test_regressions.py:17).
"""

from __future__ import annotations

__all__ = [
    "D1",
    "D2",
    "F",
    "FArray1D",
    "FArray2D",
    "Pair",
    "PairSpec",
    "UVMode",
    "UnsetType",
    "UNSET",
    "f32",
    "f64",
]

from enum import Enum, auto
from typing import Literal, TypeAlias, TypeVar

import numpy as np
from numpy import float32 as f32
from numpy import float64 as f64

_T = TypeVar("_T")
Pair: TypeAlias = tuple[_T, _T]
PairSpec: TypeAlias = _T | Pair[_T]

UVMode = Literal["velocity", "polarization"]


class UnsetType(Enum):
    UNSET = auto()


UNSET = UnsetType.UNSET

F = TypeVar("F", f32, f64)
D1 = tuple[int]
D2 = tuple[int, int]
FArray1D = np.ndarray[D1, np.dtype[F]]
FArray2D = np.ndarray[D2, np.dtype[F]]
