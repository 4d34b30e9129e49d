"""rlic_gb300: line integral convolution on NVIDIA GB300 (sm_103a).

A drop-in replacement for ``rlic.convolve`` (neutrinoceros/rlic) whose
streamline arithmetic runs in hand-written CUDA kernels behind a C ABI
(``include/rlic_gb300.h``), loaded with ctypes.
"""

from rlic_gb300._lib import convolve

__all__ = ["convolve"]
__version__ = "0.1.0"
