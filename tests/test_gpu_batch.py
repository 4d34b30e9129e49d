"""Batched form: one call for many instances of uneven sizes, kernels,
boundaries, uv modes and iteration counts, bit-identical to one convolve
call per instance, also when replayed from a captured CUDA graph, both in
with one launch per level and in one persistent launch from a work queue."""

from __future__ import annotations

import numpy as np
import pytest

import rlic_gb300
from rlic_gb300.batch import BatchPlan, autotune_tiles
from rlic_gb300.workloads import batch_case

pytestmark = pytest.mark.gpu


def _reference(items):
    return [
        rlic_gb300.convolve(it["texture"], it["u"], it["v"], kernel=it["kernel"],
                            uv_mode=it["uv_mode"], boundaries=it["boundaries"],
                            iterations=it["iterations"])
        for it in items
    ]


def _mixed_items():
    import torch

    items = batch_case(count=14, seed=11, min_side=24, max_side=320)
    rng = np.random.default_rng(12)
    for k, it in enumerate(items):
        it["tile_x"] = [0, 8, 16, 32, 64, 128, 256][k % 7]
        if k % 5 == 0:
            it["iterations"] = 0  # zeros from the native core; the Python layer copies
        if k % 4 == 1:  # rough field with zeros, -0 and NaN stops
            ny, nx = it["texture"].shape
            u = (rng.random((ny, nx)) - 0.5).astype(np.float32)
            v = (rng.random((ny, nx)) - 0.5).astype(np.float32)
            u[rng.random((ny, nx)) < 0.03] = 0.0
            v[u == 0] = -0.0
            u[rng.random((ny, nx)) < 0.005] = np.nan
            it["u"], it["v"] = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    return items


@pytest.mark.parametrize("queue", [False, True], ids=["per-level", "queue"])
def test_batch_matches_individual_calls(queue) -> None:
    import torch

    items = _mixed_items()
    for k, it in enumerate(items):
        it["replay_tiles"] = [0, 1, 3, 64][k % 4]
    plan = BatchPlan(items, queue=queue)
    outs = plan.run()
    for it, got, want in zip(items, outs, _reference(items)):
        if it["iterations"] == 0:
            assert not got.any()
            continue
        assert torch.equal(got.view(torch.int32), want.view(torch.int32))
    assert plan.status()


def test_batch_queue_many_small_instances() -> None:
    """300 instances of 16-96 pixels a side in one queue: thousands of
    segments (beyond the 2048 the kernel keeps in shared memory), so the
    segment search runs in global memory; every level waits for its
    previous one."""
    import torch

    items = batch_case(count=300, seed=13, min_side=16, max_side=96)
    for it in items:
        it["iterations"] = 10
    plan = BatchPlan(items, queue=True)
    outs = plan.run()
    for got, want in zip(outs, _reference(items)):
        assert torch.equal(got.view(torch.int32), want.view(torch.int32))
    assert plan.status()


@pytest.mark.parametrize("queue", [False, True], ids=["per-level", "queue"])
def test_batch_graph_replay_with_new_textures(queue) -> None:
    import torch

    items = _mixed_items()
    for it in items:
        it["iterations"] = max(it["iterations"], 1)
    plan = BatchPlan(items, queue=queue)
    plan.capture()
    for round_ in range(2):
        gen = torch.Generator(device="cuda").manual_seed(round_)
        for t in plan.inputs:
            t["texture"].copy_(torch.rand(t["texture"].shape, generator=gen, device="cuda"))
        outs = plan.replay()
        torch.cuda.synchronize()
        want = _reference([{**it, "texture": t["texture"]} for it, t in zip(items, plan.inputs)])
        for got, w in zip(outs, want):
            assert torch.equal(got.view(torch.int32), w.view(torch.int32))


def test_autotune_sets_tiles() -> None:
    items = batch_case(count=3, seed=5, min_side=64, max_side=200)
    for it in items:
        it["iterations"] = 3
    choice = autotune_tiles(items, repeats=1)
    assert choice and all(it["tile_x"] in (64, 32, 16) for it in items)
    assert all(it["replay_tiles"] in (2, 4, 8) for it in items)


def test_batch_validates_items() -> None:
    items = batch_case(count=2, seed=5, min_side=32, max_side=40)
    items[1]["uv_mode"] = "astral"
    with pytest.raises(ValueError, match=r"^Invalid uv_mode 'astral'"):
        BatchPlan(items)


def test_large_items_run_as_their_own_calls() -> None:
    """Items above the solo size run as single calls beside the batched call
    of the others: the same bits as batching every item, also from a graph."""
    import torch

    items = batch_case(count=6, seed=17, min_side=96, max_side=400)
    solo = BatchPlan(items, solo_pixels=150 * 150)
    assert 0 < len(solo.solo) < len(items)
    every = BatchPlan(items, solo_pixels=0)
    a, b = solo.run(), every.run()
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))
    solo.capture()
    for x, y in zip(solo.replay(), b):
        torch.cuda.synchronize()
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_batch_covers_every_item(world) -> None:
    """A batch split by instance across `world` ranks, each rank's share run
    in turn on this GPU (shares never wait on one another): every item's
    output once, bit-identical to its own convolve call."""
    import torch

    from rlic_gb300.batch import convolve_batch_sharded

    items = batch_case(count=10, seed=23, min_side=24, max_side=200)
    got = {}
    for rank in range(world):
        share = convolve_batch_sharded(items, rank, world)
        assert not set(share) & set(got)
        got.update(share)
    assert sorted(got) == list(range(len(items)))
    for k, want in enumerate(_reference(items)):
        assert torch.equal(got[k].view(torch.int32), want.view(torch.int32))
