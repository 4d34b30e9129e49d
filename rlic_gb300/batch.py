"""The batched form: many independent float32 convolutions in one call.

``BatchPlan`` takes a list of items (dicts with the arguments of
``convolve``: ``texture``, ``u``, ``v``, ``kernel`` as float32 CUDA tensors,
plus ``uv_mode``, ``boundaries``, ``iterations`` and optionally ``tile_x``),
validates every item with the rules and messages of ``convolve``, and
preallocates the outputs and one workspace.  ``run()`` makes one pack
launch and one launch per pass level over all items
(rlic_convolve_batch_f32), or, with ``queue=True``, one persistent kernel
launch that runs the whole batch from a work queue (pack, traced pass and
replays of every item, each level of an item waiting for its previous
one).  ``capture()``
records a run into a CUDA graph so that ``replay()`` re-runs the whole
batch with a single graph launch; write new textures into the plan's input
tensors in place between replays.  ``status()`` reports whether the last
work-queue run's bounded waits all ended.

Items of at least ``SOLO_PIXELS`` pixels run as their own
rlic_convolve_f32 calls in the same stream (and graph): such an item fills
the GPU alone, and a single call replays from TMA-staged boxes, which the
batched kernels do not (``solo_pixels=0`` batches every item).

``autotune_tiles`` picks, per bucket of similar items (side, kernel length,
uv mode), the CTA tile shape (``tile_x`` x 256 / ``tile_x`` pixels) and the
tiles per replay work item (``replay_tiles``) by timing the candidates on
the bucket's first item.  Results are bit-identical to one ``convolve`` call
per item, whatever the tile shapes.

On several GPUs a batch shards by instance: ``shard_items`` gives each rank
whole items, balanced by samples, and ``convolve_batch_sharded`` runs one
rank's share; the instances are independent, so no data moves between
ranks.
"""

from __future__ import annotations

__all__ = ["BatchPlan", "autotune_tiles", "convolve_batch", "convolve_batch_sharded",
           "item_samples", "shard_items"]

import ctypes
import math
from typing import Any

from rlic_gb300 import _native
from rlic_gb300._lib import _collect_problems, _Ops

TILE_CANDIDATES = (64, 32, 16)
# items of at least this many pixels (1448^2) run as their own calls
SOLO_PIXELS = 1 << 21
REPLAY_TILE_CANDIDATES = (2, 4, 8)


def _validate_item(k: int, item: dict) -> tuple:
    import torch

    tex, u, v, kern = (item[x] for x in ("texture", "u", "v", "kernel"))
    if not all(isinstance(a, torch.Tensor) for a in (tex, u, v, kern)):
        raise TypeError(f"batch item {k}: texture, u, v and kernel must be torch tensors")
    problems, bs = _collect_problems(
        _Ops(True), tex, u, v, kern, item.get("uv_mode", "velocity"),
        item.get("boundaries", "closed"), item.get("iterations", 1),
    )
    if len(problems) == 1:
        # convolve's message, with the item's index as a note
        problems[0].add_note(f"in batch item {k}")
        raise problems[0]
    if problems:
        raise ExceptionGroup(f"Invalid inputs were received (batch item {k}).", problems)
    if tex.dtype != torch.float32 or not tex.is_cuda:
        raise TypeError(f"batch item {k}: the batched form takes float32 CUDA tensors")
    return bs


class BatchPlan:
    """Preallocated batch of convolutions (see the module docstring).

    Items of at least ``solo_pixels`` pixels fill the GPU on their own, and
    one call each (whose replays read TMA-staged boxes) runs them faster
    than the batched kernels: those items run as their own
    rlic_convolve_f32 calls, in the same stream (and the same captured
    graph) as the batched call of the others.  ``solo_pixels=0`` batches
    every item.
    """

    def __init__(self, items: list[dict], queue: bool = False,
                 solo_pixels: int = SOLO_PIXELS) -> None:
        import torch

        if not items:
            raise ValueError("empty batch")
        self.queue = queue
        self.lib = _native.lib()
        self.device = items[0]["texture"].device
        self.inputs: list[dict] = []
        self.outputs: list[Any] = []
        batched, self.solo, total = [], [], 0
        for k, item in enumerate(items):
            bs = _validate_item(k, item)
            t = {x: item[x].to(device=self.device).contiguous() for x in ("texture", "u", "v", "kernel")}
            out = torch.empty_like(t["texture"])
            self.inputs.append(t)
            self.outputs.append(out)
            ny, nx = t["texture"].shape
            klen, iters = int(t["kernel"].shape[0]), int(item.get("iterations", 1))
            total += ny * nx * klen * iters
            mode = _native.UV_MODE_CODES[item.get("uv_mode", "velocity")]
            if solo_pixels and ny * nx >= solo_pixels and iters >= 1:
                self.solo.append((t, out, ny, nx, klen, iters, mode, bs.codes()))
                continue
            xl, xr, yl, yr = bs.codes()
            batched.append(_native.BatchItemF32(
                t["texture"].data_ptr(), t["u"].data_ptr(), t["v"].data_ptr(),
                t["kernel"].data_ptr(), out.data_ptr(), ny, nx, klen, iters, mode, xl, xr, yl,
                yr, int(item.get("tile_x", 0)), int(item.get("replay_tiles", 0)),
            ))
        self.total_samples = total
        self.count = len(batched)
        self.items = (_native.BatchItemF32 * max(self.count, 1))(*batched)
        nbytes = self.lib.rlic_batch_workspace_bytes_f32(self.items, self.count) \
            if self.count else 0
        self.workspace = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
        self.nbytes = nbytes
        self.solo_bytes = max((self.lib.rlic_workspace_bytes(ny, nx, klen, iters, 4, 0)
                               for _, _, ny, nx, klen, iters, _, _ in self.solo), default=0)
        self.solo_ws = torch.empty(max(self.solo_bytes, 1), dtype=torch.uint8,
                                   device=self.device)
        self.prepared = False
        self.graph = None

    def samples(self) -> int:
        return self.total_samples

    def run(self) -> list:
        """Launch the batch on the current stream; returns the output tensors."""
        import torch

        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        for t, out, ny, nx, klen, iters, mode, bc in self.solo:
            _native.check(self.lib.rlic_convolve_f32(
                t["texture"].data_ptr(), t["u"].data_ptr(), t["v"].data_ptr(), ny, nx,
                t["kernel"].data_ptr(), klen, mode, *bc, iters, out.data_ptr(),
                self.solo_ws.data_ptr(), self.solo_bytes, stream, 0))
        if self.count:
            flags = _native.RLIC_FLAG_BATCH_PREPARED if self.prepared else 0
            if self.queue:
                flags |= _native.RLIC_FLAG_BATCH_QUEUE
            _native.check(self.lib.rlic_convolve_batch_f32(
                self.items, self.count, self.workspace.data_ptr(), self.nbytes, stream, flags))
        self.prepared = True
        return self.outputs

    def status(self) -> bool:
        """True if every bounded wait of the last work-queue run ended
        (synchronises the device)."""
        if not self.count:
            return True
        rc = self.lib.rlic_batch_status_f32(self.items, self.count, self.workspace.data_ptr())
        if rc < 0:
            _native.check(-rc)
        return rc == 0

    def capture(self) -> None:
        """Record one prepared run into a CUDA graph (replay() re-runs it)."""
        import torch

        if not self.prepared:
            self.run()
            torch.cuda.synchronize(self.device)
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(side), torch.cuda.graph(graph, stream=side):
            self.run()
        torch.cuda.current_stream(self.device).wait_stream(side)
        self.graph = graph

    def replay(self) -> list:
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()
        return self.outputs


def convolve_batch(items: list[dict]) -> list:
    """One-shot batch: validate, run, and return the outputs."""
    return BatchPlan(items).run()


def item_samples(item: dict) -> int:
    """Samples of one item: pixels x kernel length x iterations."""
    ny, nx = item["texture"].shape
    return int(ny) * int(nx) * int(item["kernel"].shape[0]) * int(item.get("iterations", 1))


def shard_items(items: list[dict], world: int) -> list[list[int]]:
    """The item indices each of `world` ranks runs, for one batch on several
    GPUs.

    Instances are independent, so each goes whole to one rank and no data
    moves between ranks.  Largest first (by samples), each item goes to the
    rank with the fewest samples so far (the lowest rank on a tie), so that
    the ranks' totals differ by at most the samples of one item (Graham's
    longest-processing-time rule).  The assignment depends on the items
    alone: every rank computes the same one without a message.
    """
    if world <= 0:
        raise ValueError("world size must be positive")
    load = [0] * world
    shares: list[list[int]] = [[] for _ in range(world)]
    for k in sorted(range(len(items)), key=lambda k: (-item_samples(items[k]), k)):
        r = min(range(world), key=lambda r: (load[r], r))
        shares[r].append(k)
        load[r] += item_samples(items[k])
    return [sorted(s) for s in shares]


def convolve_batch_sharded(items: list[dict], rank: int, world: int, run=None) -> dict:
    """This rank's share of a batch run on `world` ranks (``shard_items``):
    {item index: output}.  ``run`` maps a list of items to their outputs
    (default ``convolve_batch``, on this rank's GPU); the union over ranks
    holds every item's output once."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    mine = shard_items(items, world)[rank]
    if not mine:
        return {}
    outs = (run or convolve_batch)([items[k] for k in mine])
    return dict(zip(mine, outs))


def _bucket(item: dict) -> tuple:
    ny, nx = item["texture"].shape
    klen = int(item["kernel"].shape[0])
    return (round(math.log2(max(ny * nx, 1)) / 2), (klen + 15) // 32,
            item.get("uv_mode", "velocity"))


def _time_plan(plan: "BatchPlan", repeats: int) -> float:
    import torch

    plan.run()
    torch.cuda.synchronize(plan.device)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(repeats):
        plan.run()
    b.record()
    torch.cuda.synchronize(plan.device)
    return a.elapsed_time(b) / repeats


def autotune_tiles(items: list[dict], candidates: tuple = TILE_CANDIDATES,
                   replay_candidates: tuple = REPLAY_TILE_CANDIDATES,
                   repeats: int = 2) -> dict:
    """Sets item["tile_x"] and item["replay_tiles"] to the fastest candidates
    for each bucket of similar items (side, kernel length in steps of 32 taps,
    uv mode).

    Each bucket is timed on its first item, as a one-item batch of at most
    two iterations (a traced pass and a replay): first the tile shapes, then,
    with the best shape, the tiles per replay work item of the work-queue
    form.  Returns the choice per bucket.
    """
    choice: dict = {}
    for item in items:
        key = _bucket(item)
        if key not in choice:
            probe = {**item, "iterations": min(int(item.get("iterations", 1)), 2)}
            best_tx = min(candidates, key=lambda tx: _time_plan(
                BatchPlan([{**probe, "tile_x": tx}], solo_pixels=0), repeats))
            best_rt = 0
            if probe["iterations"] >= 2:  # tiles per replay item of the work queue
                best_rt = min(replay_candidates, key=lambda rt: _time_plan(
                    BatchPlan([{**probe, "tile_x": best_tx, "replay_tiles": rt}], queue=True,
                              solo_pixels=0), repeats))
            choice[key] = (best_tx, best_rt)
        item["tile_x"], item["replay_tiles"] = choice[key]
    return choice
