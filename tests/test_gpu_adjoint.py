"""Differentiable form: forward bit-identical to convolve; backward checked
against a dense transpose built from impulse responses of the oracle (the
reference's restated core) and against central finite differences in
float64 (h = 1e-6, perturbing only texture entries >= 2h, since validation
rejects negative textures).
"""

from __future__ import annotations

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300.forms import convolve_autograd
from rlic_gb300.workloads import readme_case

pytestmark = pytest.mark.gpu


def _tensors(c, dtype):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(c[x], dtype=dtype)).cuda()
            for x in ("texture", "u", "v", "kernel")]


def test_forward_is_bit_identical_to_convolve() -> None:
    c = readme_case(n=200, klen=33, dtype=np.float32, seed=4)
    tex, u, v, k = _tensors(c, np.float32)
    out = convolve_autograd(tex, u, v, kernel=k, boundaries="periodic", iterations=3)
    ref = rlic_gb300.convolve(tex, u, v, kernel=k, boundaries="periodic", iterations=3)
    assert out.equal(ref)


@pytest.mark.parametrize("uv_mode, bnd", [("velocity", "periodic"),
                                           ("polarization", {"x": "closed", "y": "periodic"})])
def test_gradient_matches_dense_transpose(oracle, uv_mode, bnd) -> None:
    import torch

    n, klen, iters = 48, 17, 3
    rng = np.random.default_rng(4)
    c = readme_case(n=n, klen=klen, dtype=np.float64, seed=4)
    u = np.ascontiguousarray(c["u"]) + 0.3 * (rng.random((n, n)) - 0.5)
    v = np.ascontiguousarray(c["v"]) + 0.3 * (rng.random((n, n)) - 0.5)
    k = c["kernel"]
    # dense one-pass operator from impulse responses of the oracle
    A = np.empty((n * n, n * n))
    for j in range(n * n):
        e = np.zeros(n * n)
        e[j] = 1.0
        A[:, j] = oracle.convolve(e.reshape(n, n), u, v, k, uv_mode=uv_mode, boundaries=bnd).ravel()
    W = rng.normal(size=(n, n))
    want = W.ravel()
    for _ in range(iters):
        want = A.T @ want
    tex = torch.from_numpy(c["texture"]).cuda().requires_grad_(True)
    out = convolve_autograd(tex, torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda(),
                            kernel=torch.from_numpy(k).cuda(), uv_mode=uv_mode, boundaries=bnd,
                            iterations=iters)
    (out * torch.from_numpy(W).cuda()).sum().backward()
    got = tex.grad.cpu().numpy().ravel()
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-10 * np.abs(want).max())
    # the forward agrees with the dense operator too
    fwd = c["texture"].ravel()
    for _ in range(iters):
        fwd = A @ fwd
    np.testing.assert_allclose(out.detach().cpu().numpy().ravel(), fwd, rtol=1e-12)


def test_gradients_match_finite_differences() -> None:
    import torch

    n, klen, iters, h = 96, 33, 3, 1e-6
    c = readme_case(n=n, klen=klen, dtype=np.float64, seed=4)
    rng = np.random.default_rng(4)
    tex0 = torch.from_numpy(c["texture"]).cuda()
    u, v = (torch.from_numpy(np.ascontiguousarray(c[x])).cuda() for x in ("u", "v"))
    k0 = torch.from_numpy(c["kernel"]).cuda()
    W = torch.from_numpy(rng.normal(size=(n, n))).cuda()
    kw = dict(boundaries="periodic", iterations=iters)

    def loss(tex, k):
        return float((rlic_gb300.convolve(tex, u, v, kernel=k, **kw) * W).sum())

    tex = tex0.clone().requires_grad_(True)
    k = k0.clone().requires_grad_(True)
    (convolve_autograd(tex, u, v, kernel=k, **kw) * W).sum().backward()
    gt, gk = tex.grad.cpu().numpy(), k.grad.cpu().numpy()
    flat = np.flatnonzero(c["texture"].ravel() >= 2 * h)
    for idx in rng.choice(flat, size=12, replace=False):
        i, j = divmod(int(idx), n)
        tp, tm = tex0.clone(), tex0.clone()
        tp[i, j] += h
        tm[i, j] -= h
        fd = (loss(tp, k0) - loss(tm, k0)) / (2 * h)
        assert fd == pytest.approx(gt[i, j], rel=1e-5, abs=1e-4)
    for q in range(klen):
        kp, km = k0.clone(), k0.clone()
        kp[q] += h
        km[q] -= h
        fd = (loss(tex0, kp) - loss(tex0, km)) / (2 * h)
        assert fd == pytest.approx(gk[q], rel=1e-5, abs=1e-6 * np.abs(gk).max())


def test_float32_gradients_track_float64() -> None:
    import torch

    c = readme_case(n=160, klen=33, dtype=np.float64, seed=4)
    W = np.random.default_rng(4).normal(size=(160, 160))
    grads = {}
    for dt in (np.float32, np.float64):
        tex, u, v, k = _tensors(c, dt)
        tex.requires_grad_(True)
        k.requires_grad_(True)
        out = convolve_autograd(tex, u, v, kernel=k, boundaries="periodic", iterations=3)
        (out * torch.from_numpy(W.astype(dt)).cuda()).sum().backward()
        grads[dt] = (tex.grad.cpu().numpy().astype(np.float64), k.grad.cpu().numpy().astype(np.float64))
    for a, b in zip(grads[np.float32], grads[np.float64]):
        np.testing.assert_allclose(a, b, rtol=2e-4, atol=2e-4 * np.abs(b).max())
