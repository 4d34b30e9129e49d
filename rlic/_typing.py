"""Alias of ``rlic_gb300._typing``."""

from rlic_gb300._typing import *  # noqa: F403
from rlic_gb300._typing import __all__ as __all__
