"""Alias of ``rlic_gb300._boundaries``."""

from rlic_gb300._boundaries import (
    COMBO_ALLOWED_BOUNDS,
    COMBO_DISALLOWED_BOUNDS,
    SUPPORTED_BOUNDS,
    BoundaryDictSpec,
    BoundarySet,
    BoundarySpec,
    BoundaryStr,
    as_pair,
)

__all__ = [
    "COMBO_ALLOWED_BOUNDS",
    "COMBO_DISALLOWED_BOUNDS",
    "SUPPORTED_BOUNDS",
    "BoundaryDictSpec",
    "BoundarySet",
    "BoundarySpec",
    "BoundaryStr",
    "as_pair",
]
