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

With the GPU engine everything stays on the rank's device: the extended
band's field is uploaded and packed once, the first pass traces the band
and records its path cache, and every later pass replays the band from the
cache; between passes only the halo rows move, device to device over NCCL
(through host memory when the process group is `gloo`).  No kernel waits on
another rank: each exchange completes between passes.

``ShardPlan`` holds the row bookkeeping (pure host logic); ``HaloExchange``
moves rows with torch.distributed point-to-point calls; ``GpuBandEngine``
runs a rank's passes; and ``convolve_row_sharded`` drives them (any object
with the engine's ``first``/``next`` methods, or a per-pass ``compute``
function, can stand in for the GPU engine).
"""

from __future__ import annotations

__all__ = ["GpuBandEngine", "HaloExchange", "ShardPlan", "convolve_row_sharded",
           "row_bands"]

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
    """Rebuilds every rank's extended band from the ranks' owned rows.

    The rows a rank needs from each other rank, and where they go in its
    extended band, are fixed by the plan, so they are computed once as index
    arrays; ``fill`` then moves them with one isend/irecv per pair of ranks
    (in a fixed global order, so no pattern of pairs can deadlock) and
    gathers/scatters rows with index_select/index_copy_ on the tensors'
    device.  With a `gloo` group, device tensors are staged through host
    memory (gloo moves host tensors only).
    """

    def __init__(self, plan: ShardPlan, rank: int, group=None) -> None:
        self.plan, self.rank, self.group = plan, rank, group
        self.transfers = plan.transfers()
        ext = plan.ext_rows[rank]
        r0, _ = plan.bands[rank]
        # this rank's own rows inside its extended band (several copies when
        # a periodic band wraps onto itself)
        own = [(q, int(g) - r0) for q, g in enumerate(ext) if plan.owner(int(g)) == rank]
        off = plan.owned_offset[rank]
        n_own = plan.bands[rank][1] - r0
        # the copies outside the owned block (q != off + k)
        copies = [(q, k) for q, k in own if q != off + k]
        assert all(0 <= k < n_own for _, k in own)
        self.copy_dst = np.array([q for q, _ in copies], dtype=np.int64)
        self.copy_src = np.array([k for _, k in copies], dtype=np.int64)
        # per source rank: extended-band positions of its rows, in the order
        # of the rows it sends
        self.recv: dict[int, tuple[np.ndarray, np.ndarray]] = {}
        self.send: dict[int, np.ndarray] = {}
        for (src, dst), glob in self.transfers.items():
            if dst == rank:
                pos = {}
                for q, g in enumerate(ext):
                    pos.setdefault(int(g), []).append(q)
                dst_pos, order = [], []
                for k, g in enumerate(glob):
                    for q in pos[int(g)]:
                        dst_pos.append(q)
                        order.append(k)
                self.recv[src] = (np.array(dst_pos, dtype=np.int64),
                                  np.array(order, dtype=np.int64))
            elif src == rank:
                self.send[dst] = np.asarray(glob, dtype=np.int64) - r0

    def _staged(self, t):
        import torch.distributed as dist

        backend = dist.get_backend(self.group)
        return t.is_cuda and backend != "nccl"

    def fill(self, owned, ext) -> None:
        """Writes the extended band `ext` (rows x nx torch tensor, in place)
        from `owned`, this rank's rows [r0, r1), and the other ranks' rows."""
        off = self.plan.owned_offset[self.rank]
        ext[off:off + owned.shape[0]].copy_(owned)
        self.refresh(ext)

    def refresh(self, ext) -> None:
        """Rewrites the halo rows of the extended band `ext` in place, its
        owned rows (at the plan's owned offset) being current: the copies of
        owned rows a periodic band holds twice, and the other ranks' rows.
        A pass's output band becomes the next pass's input this way, with no
        copy of the owned rows."""
        import torch
        import torch.distributed as dist

        off = self.plan.owned_offset[self.rank]
        r0, r1 = self.plan.bands[self.rank]
        owned = ext[off:off + (r1 - r0)]
        dev = ext.device
        idx = lambda a: torch.from_numpy(a).to(dev)  # noqa: E731
        if self.copy_dst.size:
            ext.index_copy_(0, idx(self.copy_dst), owned.index_select(0, idx(self.copy_src)))
        if not self.transfers:  # a single rank: its band holds only its own rows
            return
        staged = self._staged(owned)
        reqs, recv_bufs = [], {}
        for (src, dst), glob in sorted(self.transfers.items()):
            if dst == self.rank:
                shape = (len(glob), owned.shape[1])
                buf = torch.empty(shape, dtype=owned.dtype,
                                  device="cpu" if staged else dev)
                reqs.append(dist.irecv(buf, src=src, group=self.group))
                recv_bufs[src] = buf
            elif src == self.rank:
                payload = owned.index_select(0, idx(self.send[dst])).contiguous()
                if staged:
                    payload = payload.cpu()
                reqs.append(dist.isend(payload, dst=dst, group=self.group))
        for req in reqs:
            req.wait()
        for src, buf in recv_bufs.items():
            dst_pos, order = self.recv[src]
            rows = buf.to(dev).index_select(0, idx(order))
            ext.index_copy_(0, idx(dst_pos), rows)

    def extended(self, owned: np.ndarray) -> np.ndarray:
        """owned: this rank's rows [r0, r1) (2-D numpy).  Returns the extended band."""
        import torch

        own = torch.from_numpy(np.ascontiguousarray(owned))
        ext = torch.empty((len(self.plan.ext_rows[self.rank]), owned.shape[1]), dtype=own.dtype)
        self.fill(own, ext)
        return ext.numpy()


class GpuBandEngine:
    """One rank's passes over its extended band, on its GPU.

    The band's (u, v) field is packed once; ``first`` traces the band
    (rlic_sweep_*, recording the path cache when more passes follow) and
    ``next`` replays it from the cache (rlic_replay_*).  Textures are torch
    tensors on `device`; results are new tensors there.  Every call is
    asynchronous on the current stream.
    """

    def __init__(self, u_ext, v_ext, kernel, uv_mode: str, boundaries: dict, iterations: int,
                 device=None) -> None:
        import torch

        from rlic_gb300 import _native
        from rlic_gb300._boundaries import BoundarySet

        self.lib = _native.lib()
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        as_t = lambda a: torch.as_tensor(np.ascontiguousarray(a) if isinstance(a, np.ndarray)  # noqa: E731
                                          else a).to(self.device).contiguous()
        self.u, self.v, self.kernel = as_t(u_ext), as_t(v_ext), as_t(kernel)
        self.dtype = self.u.dtype
        if self.dtype not in (torch.float32, torch.float64):
            raise TypeError("the GPU band engine takes float32 or float64 arrays")
        self.sfx = "f32" if self.dtype == torch.float32 else "f64"
        self.ny, self.nx = self.u.shape
        self.klen = int(self.kernel.shape[0])
        self.uv_code = _native.UV_MODE_CODES[uv_mode]
        self.bcodes = BoundarySet.from_spec(boundaries).codes()
        self.record = iterations >= 2 and self.klen > 1
        self.uv = torch.empty((self.ny, self.nx, 2), dtype=self.dtype, device=self.device)
        self._call("rlic_pack_field", self.u.data_ptr(), self.v.data_ptr(), self.ny, self.nx,
                   self.uv.data_ptr(), self._stream())
        nbytes = self.lib.rlic_path_code_bytes(self.ny, self.nx, self.klen) if self.record else 1
        self.codes = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=self.device)
        # the field's NaN-free promise spares the replays their stop-code tests
        self.flags = 0 if bool(torch.isnan(self.uv).any()) else _native.RLIC_FLAG_FIELD_NAN_FREE

    def _stream(self):
        import ctypes

        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _call(self, name: str, *args) -> None:
        from rlic_gb300 import _native

        _native.check(getattr(self.lib, f"{name}_{self.sfx}")(*args))

    def first(self, tex_ext):
        import torch

        out = torch.empty_like(tex_ext)
        self._call("rlic_sweep", tex_ext.data_ptr(), self.uv.data_ptr(), self.ny, self.nx,
                   self.kernel.data_ptr(), self.klen, self.uv_code, *self.bcodes,
                   out.data_ptr(), self.codes.data_ptr() if self.record else None,
                   self._stream(), self.flags)
        return out

    def next(self, tex_ext):
        import torch

        if not self.record:
            return self.first(tex_ext)
        out = torch.empty_like(tex_ext)
        self._call("rlic_replay", tex_ext.data_ptr(), self.codes.data_ptr(), self.ny, self.nx,
                   self.kernel.data_ptr(), self.klen, out.data_ptr(), self._stream(),
                   self.flags)
        return out


class _PassEngine:
    """A per-pass compute(tex_ext, u_ext, v_ext, kernel, uv_mode, boundaries)
    function on host arrays, as an engine (every pass traced)."""

    def __init__(self, compute, u_ext, v_ext, kernel, uv_mode, spec) -> None:
        self.compute, self.args = compute, (u_ext, v_ext, kernel, uv_mode, spec)

    def first(self, tex_ext):
        import torch

        u_ext, v_ext, kernel, uv_mode, spec = self.args
        return torch.from_numpy(np.ascontiguousarray(
            self.compute(tex_ext.numpy(), u_ext, v_ext, kernel, uv_mode, spec)))

    next = first


def convolve_row_sharded(texture, u, v, *, kernel, uv_mode="velocity", boundaries="closed",
                         iterations=1, rank: int, world: int, group=None, compute=None,
                         engine=None, device=None):
    """This rank's rows of convolve(texture, u, v, ...), computed on its band.

    texture, u, v: the full image (numpy arrays or torch tensors); only this
    rank's extended band is read.  By default the band's passes run on this
    rank's GPU (``GpuBandEngine`` on `device`, the current CUDA device if
    None), device-resident with the path cache.  ``engine(u_ext, v_ext,
    kernel, uv_mode, boundaries, iterations)`` may build another engine, or
    ``compute(tex_ext, u_ext, v_ext, kernel, uv_mode, boundaries)`` perform
    one pass over an extended band on host arrays.  Returns (r0, r1, rows)
    with rows the output rows [r0, r1) as a numpy array.
    """
    import torch

    from rlic_gb300._boundaries import BoundarySet

    bs = BoundarySet.from_spec(boundaries)
    if bs is None:
        raise TypeError(f"Invalid boundary specification {boundaries}")
    bs.validate()
    ny = texture.shape[0]
    periodic_y = bs.y[0] == "periodic"
    plan = ShardPlan(ny, world, len(kernel) // 2, periodic_y)
    spec = plan.local_boundaries({"x": bs.x, "y": bs.y})
    rows = plan.ext_rows[rank]
    off = plan.owned_offset[rank]
    r0, r1 = plan.bands[rank]

    def host(a):
        return a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)

    texture, u, v, kernel = host(texture), host(u), host(v), host(kernel)
    if iterations == 0:
        return r0, r1, np.ascontiguousarray(texture[r0:r1]).copy()
    u_ext = np.ascontiguousarray(u[rows])
    v_ext = np.ascontiguousarray(v[rows])
    tex_ext = torch.from_numpy(np.ascontiguousarray(texture[rows]))
    if compute is not None:
        eng = _PassEngine(compute, u_ext, v_ext, kernel, uv_mode, spec)
    elif engine is not None:
        eng = engine(u_ext, v_ext, kernel, uv_mode, spec, iterations)
    else:
        eng = GpuBandEngine(u_ext, v_ext, kernel, uv_mode, spec, iterations, device=device)
        tex_ext = tex_ext.to(eng.device)
    halo = HaloExchange(plan, rank, group)
    out_ext = None
    for it in range(iterations):
        out_ext = eng.first(tex_ext) if it == 0 else eng.next(tex_ext)
        if it + 1 < iterations:
            halo.refresh(out_ext)  # the output band, halo refreshed, is the next input
            tex_ext = out_ext
    return r0, r1, out_ext[off:off + (r1 - r0)].cpu().numpy().copy()
