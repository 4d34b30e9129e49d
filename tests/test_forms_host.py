"""Host-side behaviour of the precision and differentiable forms
(rlic_gb300.forms.convolve_lowp, convolve_autograd), no GPU needed.

Both validate with convolve's rules and messages before touching a device;
zero iterations return a copy of the texture, as convolve does; the
precision form names its storage choices and the differentiable form takes
CUDA tensors only.
"""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from rlic_gb300.forms import convolve_autograd, convolve_lowp  # noqa: E402


def _arrays(dtype=np.float64):
    rng = np.random.default_rng(3)
    x = rng.random((8, 9)).astype(dtype)
    return x, x.copy(), x.copy(), np.ones(5, dtype=dtype)


def test_lowp_names_its_storage_choices() -> None:
    tex, u, v, k = _arrays()
    with pytest.raises(ValueError, match=r"^Invalid storage 'fp8'\. Expected one of \['fp16', 'bf16'\]$"):
        convolve_lowp(tex, u, v, kernel=k, storage="fp8")


def test_lowp_validates_like_convolve() -> None:
    tex, u, v, k = _arrays()
    with pytest.raises(ValueError, match=r"^Invalid uv_mode 'sideways'"):
        convolve_lowp(tex, u, v, kernel=k, uv_mode="sideways")
    bad = tex.copy()
    bad[2, 2] = -1.0
    with pytest.raises(ValueError, match=r"^Found invalid texture element\(s\)"):
        convolve_lowp(bad, u, v, kernel=k)
    with pytest.raises(ExceptionGroup) as info:
        convolve_lowp(bad, u, v, kernel=k, iterations=-1)
    assert [type(e) for e in info.value.exceptions] == [ValueError, ValueError]
    with pytest.raises(TypeError, match="Data types mismatch"):
        convolve_lowp(tex, u.astype(np.float32), v, kernel=k)


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_lowp_zero_iterations_copy_the_texture(storage) -> None:
    tex, u, v, k = _arrays(np.float32)
    out = convolve_lowp(tex, u, v, kernel=k, iterations=0, storage=storage)
    assert out is not tex and out.dtype == tex.dtype
    np.testing.assert_array_equal(out, tex)
    t = torch.from_numpy(tex)
    out_t = convolve_lowp(t, torch.from_numpy(u), torch.from_numpy(v),
                          kernel=torch.from_numpy(k), iterations=0, storage=storage)
    assert out_t.data_ptr() != t.data_ptr() and torch.equal(out_t, t)


def test_autograd_takes_tensors_only() -> None:
    tex, u, v, k = _arrays()
    with pytest.raises(TypeError, match="torch CUDA tensors"):
        convolve_autograd(tex, u, v, kernel=k)


def test_autograd_refuses_cpu_tensors() -> None:
    tex, u, v, k = (torch.from_numpy(a) for a in _arrays())
    with pytest.raises(ValueError, match="CUDA tensors"):
        convolve_autograd(tex, u, v, kernel=k, iterations=2)


def test_autograd_validates_like_convolve() -> None:
    tex, u, v, k = (torch.from_numpy(a) for a in _arrays())
    with pytest.raises(ValueError, match=r"^Invalid number of iterations: -1"):
        convolve_autograd(tex, u, v, kernel=k, iterations=-1)
    with pytest.raises(TypeError, match="Boundary|boundar"):
        convolve_autograd(tex, u, v, kernel=k, boundaries=3)
