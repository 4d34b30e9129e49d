"""``import rlic`` served by rlic_gb300.

This package lets code written against neutrinoceros/rlic (including its
own test-suite, which imports ``rlic``, ``rlic._typing`` and
``rlic._boundaries``) run unchanged on the GB300 implementation.
"""

from rlic_gb300._lib import convolve

__all__ = ["convolve"]
