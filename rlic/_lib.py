"""Alias of ``rlic_gb300._lib``."""

from rlic_gb300._lib import convolve

__all__ = ["convolve"]
