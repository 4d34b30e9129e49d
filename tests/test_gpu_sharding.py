"""Row-band sharding with the GPU pass: two ranks (processes) on one GPU,
exchanging halo rows over a `gloo` group between passes, give the full
image's bits.

The ranks' kernels never wait on each other: every exchange happens on the
host between passes.
"""

from __future__ import annotations

import socket
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    from rlic_gb300.workloads import fourier_vortex_case

    c = fourier_vortex_case(n=512, klen=33, iterations=3)
    return c


def _worker(rank, world, port, outdir):
    import os

    import torch.distributed as dist

    from rlic_gb300.sharding import convolve_row_sharded

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c = _case()
        r0, r1, rows = convolve_row_sharded(
            c["texture"], c["u"], c["v"], kernel=c["kernel"], uv_mode=c["uv_mode"],
            boundaries=c["boundaries"], iterations=c["iterations"], rank=rank, world=world)
        np.savez(Path(outdir) / f"rank{rank}.npz", r0=r0, r1=r1, rows=rows)
    finally:
        dist.destroy_process_group()


def test_two_gpu_ranks_equal_full_image(tmp_path) -> None:
    import torch.multiprocessing as mp

    import rlic_gb300

    world = 2
    mp.spawn(_worker, nprocs=world, join=True, args=(world, _free_port(), str(tmp_path)))
    c = _case()
    want = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"],
                               uv_mode=c["uv_mode"], boundaries=c["boundaries"],
                               iterations=c["iterations"])
    got = np.empty_like(want)
    for r in range(world):
        z = np.load(tmp_path / f"rank{r}.npz")
        got[int(z["r0"]):int(z["r1"])] = z["rows"]
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
