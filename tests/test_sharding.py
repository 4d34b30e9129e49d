"""Row-band sharding (rlic_gb300.sharding) on CPU ranks.

The GPU pool gives one GPU per machine, so the multi-rank path is tested
here with `gloo` process groups of 2 and 3 ranks, the oracle standing in for
the per-band GPU pass.  Every rank's rows must equal the full-image result
bit for bit, over several iterations (so the halo exchange between passes
is exercised), for closed and periodic y axes, including bands thinner than
the halo (rows then come from several ranks).
"""

from __future__ import annotations

import os
import socket
from pathlib import Path

import numpy as np
import pytest

from rlic_gb300.sharding import ShardPlan, row_bands


def test_row_bands_cover_and_balance() -> None:
    for ny, world in [(10, 3), (7, 7), (100, 8), (5, 1)]:
        bands = row_bands(ny, world)
        assert bands[0][0] == 0 and bands[-1][1] == ny
        assert all(a[1] == b[0] for a, b in zip(bands, bands[1:]))
        sizes = [b - a for a, b in bands]
        assert max(sizes) - min(sizes) <= 1


def test_plan_rows_and_transfers() -> None:
    plan = ShardPlan(ny=20, world=2, radius=3, periodic_y=True)
    assert list(plan.ext_rows[0]) == [17, 18, 19] + list(range(0, 10)) + [10, 11, 12]
    assert plan.owned_offset == [3, 3]
    t = plan.transfers()
    assert set(t) == {(0, 1), (1, 0)}
    assert list(t[(1, 0)]) == [17, 18, 19, 10, 11, 12]
    closed = ShardPlan(ny=20, world=2, radius=3, periodic_y=False)
    assert list(closed.ext_rows[0]) == list(range(0, 13))
    assert closed.owned_offset == [0, 3]
    assert closed.local_boundaries({"x": ("periodic", "periodic"), "y": ("closed", "closed")}) == {
        "x": ("periodic", "periodic"), "y": ("closed", "closed")}


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(ny, nx, klen, seed):
    rng = np.random.default_rng(seed)
    u = (rng.random((ny, nx)) - 0.5)
    v = (rng.random((ny, nx)) - 0.5)
    u[rng.random((ny, nx)) < 0.03] = 0.0
    return rng.random((ny, nx)), u, v, rng.random(klen)


def _worker(rank, world, port, outdir, ny, nx, klen, boundaries, uv_mode, iterations):
    import torch.distributed as dist

    from oracle import oracle
    from rlic_gb300.sharding import convolve_row_sharded

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tex, u, v, k = _case(ny, nx, klen, seed=ny * 100 + klen)

        def compute(tex_ext, u_ext, v_ext, kernel, mode, spec):
            return oracle.convolve(tex_ext, u_ext, v_ext, kernel, uv_mode=mode,
                                   boundaries=spec, iterations=1)

        r0, r1, rows = convolve_row_sharded(
            tex, u, v, kernel=k, uv_mode=uv_mode, boundaries=boundaries,
            iterations=iterations, rank=rank, world=world, compute=compute)
        np.savez(Path(outdir) / f"rank{rank}.npz", r0=r0, r1=r1, rows=rows)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize(
    "world, ny, nx, klen, boundaries, uv_mode",
    [
        (2, 40, 37, 17, "periodic", "velocity"),
        (2, 41, 30, 17, {"x": "periodic", "y": "closed"}, "polarization"),
        (3, 12, 25, 17, "periodic", "polarization"),   # bands of 4 rows, halo of 8
        (3, 13, 20, 9, {"x": "closed", "y": "closed"}, "velocity"),
    ],
)
def test_sharded_equals_full_image(tmp_path, oracle, world, ny, nx, klen, boundaries, uv_mode):
    import torch.multiprocessing as mp

    iterations = 3
    mp.spawn(_worker, nprocs=world, join=True,
             args=(world, _free_port(), str(tmp_path), ny, nx, klen, boundaries, uv_mode,
                   iterations))
    tex, u, v, k = _case(ny, nx, klen, seed=ny * 100 + klen)
    want = oracle.convolve(tex, u, v, k, uv_mode=uv_mode, boundaries=boundaries,
                           iterations=iterations)
    got = np.empty_like(want)
    for r in range(world):
        z = np.load(tmp_path / f"rank{r}.npz")
        got[int(z["r0"]):int(z["r1"])] = z["rows"]
    np.testing.assert_array_equal(got, want)


def test_single_rank_band_wraps_onto_itself(oracle) -> None:
    """One rank, periodic y: the extended band holds copies of the rank's own
    rows at both ends (no process group is needed), over 3 passes."""
    from rlic_gb300.sharding import convolve_row_sharded

    tex, u, v, k = _case(20, 24, 9, seed=7)

    def compute(tex_ext, u_ext, v_ext, kernel, mode, spec):
        return oracle.convolve(tex_ext, u_ext, v_ext, kernel, uv_mode=mode, boundaries=spec,
                               iterations=1)

    r0, r1, rows = convolve_row_sharded(tex, u, v, kernel=k, uv_mode="polarization",
                                        boundaries="periodic", iterations=3, rank=0, world=1,
                                        compute=compute)
    want = oracle.convolve(tex, u, v, k, uv_mode="polarization", boundaries="periodic",
                           iterations=3)
    assert (r0, r1) == (0, 20)
    np.testing.assert_array_equal(rows, want)
