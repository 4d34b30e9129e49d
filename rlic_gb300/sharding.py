"""Row-band sharding of one convolution across ranks.

Pixels are independent within a pass and a streamline moves at most one
cell per step, so every cell a pixel's streamlines sample lies within
R = klen // 2 rows of it.  Rank r owns the rows [r0, r1) of the output and
works on an *extended band*: its rows plus R rows above and below (wrapped
for a periodic y axis, clipped at a closed edge).  A pass over the extended
band gives exact results for the owned rows, because

* at a global closed edge the extended band starts or ends at that edge, so
  the local closed rule is the global one;
* at an artificial edge (inside the image, or a periodic seam unrolled into
  the band) no streamline from an owned row can reach it.

Between passes the ranks exchange halos point to point: each rank receives
the owned rows of the ranks that hold its halo rows (its ring neighbours
when bands are at least R rows high) and sends its own rows to the ranks
that need them.  No collective touches the data path.

``ShardPlan`` holds the row bookkeeping (pure host logic); ``HaloExchange``
moves rows with torch.distributed point-to-point calls; and
``convolve_row_sharded`` drives the passes with a pluggable per-band compute
(the GPU path by default).
"""

from __future__ import annotations

__all__ = ["ShardPlan", "HaloExchange", "convolve_row_sharded", "row_bands"]

from dataclasses import dataclass, field

import numpy as np


def row_bands(ny: int, world: int) -> list[tuple[int, int]]:
    """Balanced contiguous row ranges [r0, r1) for `world` ranks."""
    if world <= 0:
        raise ValueError("world size must be positive")
    base, extra = divmod(ny, world)
    bands, r0 = [], 0
    for r in range(world):
        r1 = r0 + base + (1 if r < extra else 0)
        bands.append((r0, r1))
        r0 = r1
    return bands


@dataclass
class ShardPlan:
    """Extended-band rows of every rank for an ny-row image."""

    ny: int
    world: int
    radius: int
    periodic_y: bool
    bands: list[tuple[int, int]] = field(init=False)
    ext_rows: list[np.ndarray] = field(init=False)  # global row of each extended-band row
    owned_offset: list[int] = field(init=False)     # first owned row inside the extended band

    def __post_init__(self) -> None:
        self.bands = row_bands(self.ny, self.world)
        self.ext_rows, self.owned_offset = [], []
        for r0, r1 in self.bands:
            if self.periodic_y:
                rows = np.arange(r0 - self.radius, r1 + self.radius) % self.ny
                off = self.radius
            else:
                lo, hi = max(0, r0 - self.radius), min(self.ny, r1 + self.radius)
                rows = np.arange(lo, hi)
                off = r0 - lo
            self.ext_rows.append(rows)
            self.owned_offset.append(off)

    def owner(self, row: int) -> int:
        for r, (r0, r1) in enumerate(self.bands):
            if r0 <= row < r1:
                return r
        raise ValueError(f"row {row} outside the image")

    def local_boundaries(self, boundaries: dict) -> dict:
        """Boundary spec of an extended band: x unchanged, y closed (see the module)."""
        return {"x": boundaries["x"], "y": ("closed", "closed")}

    def transfers(self) -> dict[tuple[int, int], np.ndarray]:
        """(source, destination) -> global rows the source sends to the destination."""
        out: dict[tuple[int, int], list[int]] = {}
        for dst, rows in enumerate(self.ext_rows):
            for row in dict.fromkeys(int(x) for x in rows):  # unique, in order
                src = self.owner(row)
                if src != dst:
                    out.setdefault((src, dst), []).append(row)
        return {k: np.asarray(v, dtype=np.int64) for k, v in out.items()}


class HaloExchange:
    """Rebuilds every rank's extended band from the ranks' owned rows."""

    def __init__(self, plan: ShardPlan, rank: int, group=None) -> None:
        self.plan, self.rank, self.group = plan, rank, group
        self.transfers = plan.transfers()

    def extended(self, owned: np.ndarray) -> np.ndarray:
        """owned: this rank's rows [r0, r1) (2-D).  Returns the extended band."""
        import torch
        import torch.distributed as dist

        plan, rank = self.plan, self.rank
        r0, r1 = plan.bands[rank]
        rows = {}
        for row in range(r0, r1):
            rows[row] = owned[row - r0]
        reqs, recv_bufs = [], {}
        # post receives and sends in a fixed global order: no deadlock for
        # any pattern of pairs
        for (src, dst), glob in sorted(self.transfers.items()):
            if dst == rank:
                buf = torch.empty((len(glob), owned.shape[1]), dtype=torch.from_numpy(owned).dtype)
                reqs.append(dist.irecv(buf, src=src, group=self.group))
                recv_bufs[(src, dst)] = (glob, buf)
            elif src == rank:
                payload = torch.from_numpy(np.ascontiguousarray(owned[glob - r0]))
                reqs.append(dist.isend(payload, dst=dst, group=self.group))
        for req in reqs:
            req.wait()
        for glob, buf in recv_bufs.values():
            arr = buf.numpy()
            for k, row in enumerate(glob):
                rows[int(row)] = arr[k]
        return np.stack([rows[int(row)] for row in plan.ext_rows[rank]])


def _gpu_band_pass(tex_ext, u_ext, v_ext, kernel, uv_mode, boundaries):
    import rlic_gb300

    return rlic_gb300.convolve(tex_ext, u_ext, v_ext, kernel=kernel, uv_mode=uv_mode,
                               boundaries=boundaries, iterations=1)


def convolve_row_sharded(texture, u, v, *, kernel, uv_mode="velocity", boundaries="closed",
                         iterations=1, rank: int, world: int, group=None, compute=None):
    """This rank's rows of convolve(texture, u, v, ...), computed on its band.

    texture, u, v: the full image (numpy); only this rank's extended band is
    read.  compute(tex_ext, u_ext, v_ext, kernel, uv_mode, boundaries)
    performs one pass over an extended band (default: the GPU path).  Returns
    (r0, r1, rows) with rows the output rows [r0, r1).
    """
    from rlic_gb300._boundaries import BoundarySet

    bs = BoundarySet.from_spec(boundaries)
    if bs is None:
        raise TypeError(f"Invalid boundary specification {boundaries}")
    bs.validate()
    ny = texture.shape[0]
    periodic_y = bs.y[0] == "periodic"
    plan = ShardPlan(ny, world, len(kernel) // 2, periodic_y)
    spec = plan.local_boundaries({"x": bs.x, "y": bs.y})
    compute = compute or _gpu_band_pass
    rows = plan.ext_rows[rank]
    off = plan.owned_offset[rank]
    r0, r1 = plan.bands[rank]
    u_ext = np.ascontiguousarray(u[rows])
    v_ext = np.ascontiguousarray(v[rows])
    owned = np.ascontiguousarray(texture[r0:r1])
    if iterations == 0:
        return r0, r1, owned.copy()
    halo = HaloExchange(plan, rank, group)
    tex_ext = np.ascontiguousarray(texture[rows])
    for it in range(iterations):
        out_ext = compute(tex_ext, u_ext, v_ext, kernel, uv_mode, spec)
        owned = np.ascontiguousarray(out_ext[off:off + (r1 - r0)])
        if it + 1 < iterations:
            tex_ext = halo.extended(owned)
    return r0, r1, owned
