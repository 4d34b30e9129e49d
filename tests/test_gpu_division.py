"""The screened float64 division of the streamline step against IEEE division.

float64 steps whose time comparison the float32 screen settles divide once,
by a short Newton-Raphson sequence whose result is used only under a
remainder certificate; refused operands fall back to the IEEE division
(rlic_check_quotients_f64 exposes the sequence).  Every certified quotient
must equal numpy's correctly rounded |a / b| bit for bit: random operands
across the screened exponent range, exact quotients, and operands built to
sit next to rounding ties.  Ordinary operands must nearly all be certified,
or the short path would not pay.
"""

from __future__ import annotations

import numpy as np
import pytest

from rlic_gb300 import _native

pytestmark = pytest.mark.gpu


def _screened(a: np.ndarray, b: np.ndarray):
    import torch

    ta = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).cuda()
    q = torch.empty_like(ta)
    cert = torch.empty(ta.shape, dtype=torch.int32, device="cuda")
    _native.check(_native.lib().rlic_check_quotients_f64(
        ta.data_ptr(), tb.data_ptr(), ta.numel(), q.data_ptr(), cert.data_ptr(), None))
    torch.cuda.synchronize()
    return q.cpu().numpy(), cert.cpu().numpy().astype(bool)


def _operands(rng, n, lo=-60, hi=60):
    mant = rng.uniform(1.0, 2.0, n)
    return np.ldexp(mant, rng.integers(lo, hi + 1, n)) * rng.choice([-1.0, 1.0], n)


def _assert_certified_exact(a, b, q, cert):
    want = np.abs(a / b)
    bad = cert & (q.view(np.int64) != want.view(np.int64))
    assert not bad.any(), (a[bad][:5], b[bad][:5], q[bad][:5], want[bad][:5])


def test_random_operands_over_the_screened_range() -> None:
    rng = np.random.default_rng(0)
    n = 4_000_000
    a, b = _operands(rng, n), _operands(rng, n)
    q, cert = _screened(a, b)
    _assert_certified_exact(a, b, q, cert)
    assert cert.mean() > 0.999


def test_exact_and_power_of_two_quotients() -> None:
    rng = np.random.default_rng(1)
    n = 200_000
    # b with few significant bits, so b * k is exact for small odd k
    b = np.ldexp(rng.integers(1, 1 << 20, n).astype(np.float64), rng.integers(-70, -20, n))
    k = rng.choice([1.0, 3.0, 5.0, 7.0, 0.5, 0.75, 1.5, 2.0, 1024.0], n)
    a = b * k
    q, cert = _screened(a, b)
    _assert_certified_exact(a, b, q, cert)
    # powers of two are refused (their lower neighbour is half an ulp away);
    # the other exact quotients have a zero remainder and are certified
    pow2 = np.isin(k, [1.0, 0.5, 2.0, 1024.0])
    assert not cert[pow2].any()
    assert cert[~pow2].all()


def test_operands_next_to_rounding_ties() -> None:
    rng = np.random.default_rng(2)
    n = 2_000_000
    b = _operands(rng, n, -30, 30)
    q = np.abs(_operands(rng, n, -30, 30))
    # a / b lands within a few units of 2^-53 (relative) of q (1 + 2^-53),
    # the midpoint between q and its upper neighbour, for mantissas near 1
    a = b * (q * (1.0 + 2.0**-52)) * 0.5 + b * q * 0.5
    a = a + rng.integers(-2, 3, n) * np.spacing(a)
    qs, cert = _screened(a, b)
    _assert_certified_exact(a, b, qs, cert)
    assert cert.mean() > 0.5
