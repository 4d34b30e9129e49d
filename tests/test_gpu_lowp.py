"""Reduced-precision form: 16-bit storage between passes, FP32 compensated
accumulation, streamline cells traced in the input dtype.

Its results approximate the exact path, so these tests bound the error,
measured on outputs normalised by sum(|kernel|)^iterations: the form stores
exactly those normalised values.
"""

from __future__ import annotations

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300.forms import convolve_lowp
from rlic_gb300.workloads import readme_case

pytestmark = pytest.mark.gpu

# max-abs error bounds on normalised outputs: FP16 keeps 11 significant bits
# (relative 2^-11 = 4.9e-4 per rounding), BF16 8 (3.9e-3)
BOUND = {"fp16": 1e-3, "bf16": 8e-3}


def _normalised_error(approx, exact, kernel, iterations):
    scale = np.sum(np.abs(kernel.astype(np.float64))) ** iterations
    d = (approx.astype(np.float64) - exact.astype(np.float64)) / scale
    return float(np.max(np.abs(d))), float(np.sqrt(np.mean(d * d)))


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_precision_form_error_bound(storage, dtype) -> None:
    c = readme_case(n=384, klen=129, dtype=dtype, seed=2)
    kw = dict(kernel=c["kernel"], boundaries="periodic", iterations=10)
    exact = rlic_gb300.convolve(c["texture"], c["u"], c["v"], **kw)
    approx = convolve_lowp(c["texture"], c["u"], c["v"], storage=storage, **kw)
    assert approx.dtype == exact.dtype and approx.shape == exact.shape
    max_abs, rms = _normalised_error(approx, exact, c["kernel"], 10)
    assert max_abs <= BOUND[storage], (max_abs, rms)
    assert rms <= BOUND[storage] / 4


def test_precision_form_polarization_closed_and_nan_stops() -> None:
    rng = np.random.default_rng(5)
    n = 200
    u = (rng.random((n, n)) - 0.5).astype(np.float32)
    v = (rng.random((n, n)) - 0.5).astype(np.float32)
    u[rng.random((n, n)) < 0.01] = np.nan  # streamlines stop here
    tex = rng.random((n, n)).astype(np.float32)
    k = np.hanning(33).astype(np.float32)
    kw = dict(kernel=k, uv_mode="polarization", boundaries={"x": "closed", "y": "periodic"},
              iterations=3)
    exact = rlic_gb300.convolve(tex, u, v, **kw)
    approx = convolve_lowp(tex, u, v, storage="fp16", **kw)
    max_abs, _ = _normalised_error(approx, exact, k, 3)
    assert max_abs <= BOUND["fp16"]


def test_precision_form_torch_inputs_and_zero_iterations() -> None:
    import torch

    c = readme_case(n=64, klen=17, dtype=np.float32)
    t = [torch.from_numpy(np.ascontiguousarray(c[x])).cuda() for x in ("texture", "u", "v", "kernel")]
    out = convolve_lowp(t[0], t[1], t[2], kernel=t[3], iterations=2)
    assert out.is_cuda and out.dtype == torch.float32
    ref = convolve_lowp(c["texture"], c["u"], c["v"], kernel=c["kernel"], iterations=2)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    same = convolve_lowp(c["texture"], c["u"], c["v"], kernel=c["kernel"], iterations=0)
    np.testing.assert_array_equal(same, c["texture"])


def test_precision_form_validates_like_convolve() -> None:
    c = readme_case(n=16, klen=5)
    with pytest.raises(ValueError, match="Invalid storage"):
        convolve_lowp(c["texture"], c["u"], c["v"], kernel=c["kernel"], storage="fp8")
    with pytest.raises(ValueError, match=r"^Invalid number of iterations"):
        convolve_lowp(c["texture"], c["u"], c["v"], kernel=c["kernel"], iterations=-1)
