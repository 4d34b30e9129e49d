"""Host-side behaviour of rlic_gb300.batch.BatchPlan (no GPU needed).

A plan validates every item with convolve's rules and messages before it
allocates anything on a device: an empty batch, arrays that are not
tensors, tensors that are not float32 CUDA tensors and invalid arguments
are refused, naming the item at fault.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from rlic_gb300.batch import BatchPlan, _validate_item  # noqa: E402


def _item(dtype=torch.float32, **kw) -> dict:
    x = torch.ones((8, 9), dtype=dtype)
    item = {"texture": x, "u": x.clone(), "v": x.clone(),
            "kernel": torch.ones(5, dtype=dtype), "iterations": 2}
    item.update(kw)
    return item


def test_empty_batch_is_refused() -> None:
    with pytest.raises(ValueError, match="empty batch"):
        BatchPlan([])


def test_numpy_items_are_refused_with_their_index() -> None:
    a = np.ones((8, 9), dtype=np.float32)
    bad = {"texture": a, "u": a, "v": a, "kernel": np.ones(5, dtype=np.float32)}
    with pytest.raises(TypeError, match=r"^batch item 0: .*torch tensors"):
        BatchPlan([bad, _item()])
    with pytest.raises(TypeError, match=r"^batch item 3: .*torch tensors"):
        _validate_item(3, bad)


def test_cpu_tensors_are_refused() -> None:
    with pytest.raises(TypeError, match=r"^batch item 0: .*float32 CUDA tensors"):
        BatchPlan([_item()])


def test_float64_items_are_refused() -> None:
    with pytest.raises(TypeError, match=r"^batch item 0: .*float32 CUDA tensors"):
        BatchPlan([_item(dtype=torch.float64)])


def test_one_problem_raises_convolves_error_with_a_note() -> None:
    with pytest.raises(ValueError, match=r"^Invalid uv_mode 'astral'") as info:
        BatchPlan([_item(uv_mode="astral"), _item()])
    assert "in batch item 0" in info.value.__notes__
    with pytest.raises(ValueError, match=r"^Invalid uv_mode 'astral'") as info:
        _validate_item(2, _item(uv_mode="astral"))
    assert "in batch item 2" in info.value.__notes__


def test_several_problems_are_grouped_per_item() -> None:
    with pytest.raises(ExceptionGroup, match=r"batch item 1") as info:
        _validate_item(1, _item(uv_mode="astral", iterations=-1))
    assert [type(e) for e in info.value.exceptions] == [ValueError, ValueError]


def test_mismatched_dtypes_raise_convolves_type_error() -> None:
    item = _item()
    item["u"] = item["u"].double()
    with pytest.raises(TypeError, match="Data types mismatch"):
        BatchPlan([item])


# ------------------------------------------------------- instance sharding --

def _sized_items(sides_klens_iters) -> list[dict]:
    items = []
    for ny, nx, klen, n in sides_klens_iters:
        items.append({"texture": np.zeros((ny, nx)), "u": None, "v": None,
                      "kernel": np.zeros(klen), "iterations": n})
    return items


@pytest.mark.parametrize("world", [1, 2, 3, 5, 8])
def test_shard_items_is_a_balanced_partition(world) -> None:
    from rlic_gb300.batch import item_samples, shard_items

    rng = np.random.default_rng(world)
    items = _sized_items(
        (int(rng.integers(8, 300)), int(rng.integers(8, 300)), int(rng.integers(1, 65)) * 2 + 1,
         int(rng.integers(1, 11))) for _ in range(37))
    shares = shard_items(items, world)
    assert len(shares) == world
    flat = sorted(k for s in shares for k in s)
    assert flat == list(range(len(items)))
    assert all(s == sorted(s) for s in shares)
    loads = [sum(item_samples(items[k]) for k in s) for s in shares]
    assert max(loads) - min(loads) <= max(item_samples(i) for i in items)
    # the same items give the same assignment on every rank
    assert shard_items(items, world) == shares


def test_shard_items_edge_cases() -> None:
    from rlic_gb300.batch import convolve_batch_sharded, shard_items

    items = _sized_items([(4, 4, 3, 1), (64, 64, 9, 2), (8, 8, 5, 1)])
    # more ranks than items: the largest items first, each to an idle rank
    assert shard_items(items, 5) == [[1], [2], [0], [], []]
    assert shard_items([], 3) == [[], [], []]
    assert shard_items(items, 1) == [[0, 1, 2]]
    with pytest.raises(ValueError, match="world size"):
        shard_items(items, 0)
    with pytest.raises(ValueError, match="outside a world"):
        convolve_batch_sharded(items, 2, 2)
    # an idle rank runs nothing
    assert convolve_batch_sharded(items, 4, 5, run=lambda its: 1 / 0) == {}


def _oracle_item(oracle, it: dict) -> np.ndarray:
    return oracle.convolve(it["texture"].numpy(), it["u"].numpy(), it["v"].numpy(),
                           it["kernel"].numpy(), uv_mode=it["uv_mode"],
                           boundaries=it["boundaries"], iterations=it["iterations"])


def _batch_worker(rank, world, port, outdir, seed) -> None:
    import os

    import torch.distributed as dist

    from oracle import oracle
    from rlic_gb300.batch import convolve_batch_sharded
    from rlic_gb300.workloads import batch_case

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        items = batch_case(count=9, seed=seed, min_side=16, max_side=48, device="cpu")

        def run(share):
            return [_oracle_item(oracle, it) for it in share]

        mine = convolve_batch_sharded(items, rank, world, run=run)
        # the ranks' shares partition the batch without any exchange before
        # this check
        every = [None] * world
        dist.all_gather_object(every, sorted(mine))
        assert sorted(k for s in every for k in s) == list(range(len(items)))
        np.savez(Path(outdir) / f"rank{rank}.npz",
                 **{f"item{k}": out for k, out in mine.items()})
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_batch_on_gloo_ranks(tmp_path, oracle, world) -> None:
    """A batch sharded by instance over gloo ranks (the oracle standing in
    for each rank's GPU): every item's output exactly once, equal to the
    item run alone."""
    import socket

    import torch.multiprocessing as mp

    from rlic_gb300.workloads import batch_case

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    seed = 11
    mp.spawn(_batch_worker, nprocs=world, join=True, args=(world, port, str(tmp_path), seed))
    items = batch_case(count=9, seed=seed, min_side=16, max_side=48, device="cpu")
    got = {}
    for r in range(world):
        with np.load(tmp_path / f"rank{r}.npz") as z:
            for name in z.files:
                k = int(name[4:])
                assert k not in got
                got[k] = z[name]
    assert sorted(got) == list(range(len(items)))
    for k, it in enumerate(items):
        np.testing.assert_array_equal(got[k], _oracle_item(oracle, it))


def test_autotune_times_one_item_per_bucket(monkeypatch) -> None:
    """The tuner's choices, with the timing replaced by a fixed cost table:
    one probe per bucket (side, kernel length in steps of 32 taps, uv mode),
    probes of at most two iterations, the fastest tile shape, then the
    fastest tiles per replay item with it, and no replay choice for
    single-pass probes."""
    from rlic_gb300 import batch

    probes = []

    class FakePlan:
        def __init__(self, items, queue=False, solo_pixels=batch.SOLO_PIXELS) -> None:
            assert len(items) == 1 and solo_pixels == 0
            self.item, self.queue = items[0], queue

    def fake_time(plan, repeats) -> float:
        it = plan.item
        probes.append((it["texture"].shape, it["iterations"], it["tile_x"],
                       it.get("replay_tiles"), plan.queue))
        cost = {64: 3.0, 32: 1.0, 16: 2.0}[it["tile_x"]]
        if plan.queue:
            cost += {2: 2.0, 4: 1.0, 8: 3.0}[it["replay_tiles"]]
        return cost

    monkeypatch.setattr(batch, "BatchPlan", FakePlan)
    monkeypatch.setattr(batch, "_time_plan", fake_time)
    items = _sized_items([(256, 256, 65, 5), (256, 256, 63, 9), (64, 64, 9, 1),
                          (256, 256, 65, 3)])
    for it in items:
        it["uv_mode"] = "velocity"
    items[3]["uv_mode"] = "polarization"
    choice = batch.autotune_tiles(items)
    # buckets: items 0 and 1 share one (same side, 33-64 taps, velocity)
    assert len(choice) == 3
    assert [(it["tile_x"], it["replay_tiles"]) for it in items] == [
        (32, 4), (32, 4), (32, 0), (32, 4)]
    # 3 tile shapes per bucket, plus 3 replay choices where the probe has a replay
    assert len(probes) == 3 * 3 + 2 * 3
    assert all(n <= 2 for _, n, _, _, _ in probes)
    assert not any(q for shape, _, _, _, q in probes if shape == (64, 64))
