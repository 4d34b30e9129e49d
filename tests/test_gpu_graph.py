"""One convolve call recorded into a CUDA graph (rlic_gb300.forms.ConvolvePlan).

The device call (field packing, the traced first pass, replayed passes
ping-ponging between the output and a workspace buffer) is recorded once
and replayed; each replay must give the bits of ``convolve`` on the values
the plan's buffers hold at that moment: new textures written in place,
a new field, several replays in a row, both dtypes, the paired pass of a
small image and the TMA-staged replays of a larger one, and zero passes.
"""

from __future__ import annotations

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300.forms import ConvolvePlan

pytestmark = pytest.mark.gpu


def _same(a, b) -> bool:
    import torch

    it = torch.int32 if a.dtype == torch.float32 else torch.int64
    return bool(torch.equal(a.view(it), b.view(it)))


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("shape, klen, iters", [((256, 256), 65, 1), ((300, 340), 33, 3),
                                                ((1024, 1040), 65, 5)], ids=str)
def test_graph_replays_equal_convolve(dtype, shape, klen, iters) -> None:
    import torch

    from rlic_gb300.workloads import fourier_vortex_case

    n = max(shape)
    c = fourier_vortex_case(n=n, as_numpy=True, iterations=iters)
    dt = getattr(torch, dtype)
    t = {k: torch.from_numpy(np.ascontiguousarray(c[k][:shape[0], :shape[1]])).to("cuda", dt)
         for k in ("texture", "u", "v")}
    k = torch.from_numpy(np.hanning(klen)).to("cuda", dt)
    kw = dict(kernel=k, uv_mode="polarization", boundaries={"x": "periodic", "y": "closed"},
              iterations=iters)
    plan = ConvolvePlan(t["texture"], t["u"], t["v"], **kw)
    plan.capture()
    want = rlic_gb300.convolve(t["texture"], t["u"], t["v"], **kw)
    assert _same(plan.replay(), want)
    assert _same(plan.replay(), want)  # a second replay, same bits
    gen = torch.Generator(device="cuda").manual_seed(3)
    for _ in range(2):  # new textures written in place
        new = torch.rand(shape, generator=gen, device="cuda", dtype=dt)
        plan.texture.copy_(new)
        got = plan.replay()
        assert _same(got, rlic_gb300.convolve(new, t["u"], t["v"], **kw))
    # a new field: the recorded packing reads the plan's u and v again
    plan.u.copy_(-t["v"])
    plan.v.copy_(t["u"])
    got = plan.replay()
    assert _same(got, rlic_gb300.convolve(plan.texture, -t["v"], t["u"], **kw))


def test_zero_passes_copy_the_texture() -> None:
    import torch

    tex = torch.rand((64, 80), device="cuda")
    uv = torch.ones((64, 80), device="cuda")
    plan = ConvolvePlan(tex, uv, uv, kernel=torch.ones(5, device="cuda"), iterations=0)
    plan.capture()
    assert torch.equal(plan.replay(), tex)


def test_plan_validates_like_convolve() -> None:
    import torch

    tex = torch.rand((32, 32), device="cuda")
    with pytest.raises(ValueError):
        ConvolvePlan(tex, tex, tex, kernel=torch.ones(5, device="cuda"), uv_mode="nope")
    with pytest.raises(TypeError):
        ConvolvePlan(tex.cpu().numpy(), tex.cpu().numpy(), tex.cpu().numpy(),
                     kernel=np.ones(5, dtype=np.float32))
