"""Host-side behaviour of rlic_gb300.forms.ConvolvePlan (no GPU needed).

The plan validates its arguments with convolve's rules and messages before
touching a device, and takes only CUDA tensors: numpy arrays and CPU
tensors are refused with clear errors, invalid arguments raise what
convolve raises.
"""

from __future__ import annotations

import numpy as np
import pytest

from rlic_gb300.forms import ConvolvePlan


def _arrays(dtype=np.float32):
    x = np.ones((8, 9), dtype=dtype)
    return x, x.copy(), x.copy(), np.ones(5, dtype=dtype)


def test_numpy_inputs_are_refused() -> None:
    tex, u, v, k = _arrays()
    with pytest.raises(TypeError, match="CUDA tensors"):
        ConvolvePlan(tex, u, v, kernel=k)


def test_cpu_tensors_are_refused() -> None:
    torch = pytest.importorskip("torch")
    tex, u, v, k = (torch.from_numpy(a) for a in _arrays())
    with pytest.raises(ValueError, match="CUDA tensors"):
        ConvolvePlan(tex, u, v, kernel=k)


def test_invalid_arguments_raise_what_convolve_raises() -> None:
    tex, u, v, k = _arrays()
    with pytest.raises(ValueError, match="Invalid uv_mode"):
        ConvolvePlan(tex, u, v, kernel=k, uv_mode="sideways")
    with pytest.raises(ValueError, match="Invalid number of iterations"):
        ConvolvePlan(tex, u, v, kernel=k, iterations=-1)
    neg = tex.copy()
    neg[0, 0] = -1.0
    with pytest.raises(ValueError, match="invalid texture element"):
        ConvolvePlan(neg, u, v, kernel=k)
    with pytest.raises(ExceptionGroup):
        ConvolvePlan(neg, u, v, kernel=k, uv_mode="sideways")
