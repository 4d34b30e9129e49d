"""Benchmark: line integral convolution throughput on GB300.

Workload (one "step"): rlic.convolve on the at-scale case, 8192 x 8192
float32, 65-tap Hann kernel, polarization mode, boundaries
{x: periodic, y: closed}, 5 iterations (rlic_gb300.workloads.
fourier_vortex_case).  Metric: Gsamples/s = H * W * K * iterations / time.

  value     device-resident inputs, rlic_convolve_f32 on device pointers in
            its default (path-cache) form: pack, one traced pass that records
            every streamline step, four replayed passes; CUDA events on the
            launching stream.  "forms" also gives the plain form (every pass
            traced, RLIC_FLAG_NO_PATH_CACHE) on the same workload;
  e2e       the public API rlic_gb300.convolve on ordinary (pageable) host
            numpy arrays, as a reference caller passes them: validation,
            host->device transfer, compute, device->host transfer of the
            result, all inside the timed region ("pinned" beside it: the
            same call on page-locked arrays);
  roofline  the kernel with the largest share of a step, timed per launch:
            its algorithmic bytes per pixel (cache-less gather model) over
            its duration, against the measured HBM copy bandwidth; "kernels"
            lists every kernel of the step the same way;
  cpu_baseline  the CPU oracle (a restatement of the reference's Rust
            core) timed on a bounded band of rows of the same workload.

--impl reference times the CPU restatement of the reference's
implementation on all host threads (the reference's Rust core cannot be
built here), with the same metric and config.

Multi-GPU (torchrun, one rank per GPU): every rank convolves its own full
instance (the image does not need to be split to fill a GPU), so the work
per GPU is fixed and value = total samples / max time over ranks.  With
--shard one image is split into row bands instead, and with --workload
batched the 64-instance batch is split by instance; both are strong
scaling (the work is fixed).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

N_DEFAULT = 8192
KLEN = 65
ITERS = 5
METRIC = "Gsamples/s (px x kernel x iters)"
UNIT = "Gsamples/s"


def parse_args() -> argparse.Namespace:
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--size", type=int, default=N_DEFAULT, help="image side (default 8192)")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="target CPU time of the oracle baseline sample")
    p.add_argument("--e2e-steps", type=int, default=None)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--shard", action="store_true",
                   help="strong scaling: split one image into row bands across the ranks")
    p.add_argument("--replay", choices=["auto", "l1", "staged"], default="auto",
                   help="how replayed passes gather: the library's default, through L1, or "
                        "from TMA-staged shared-memory boxes")
    p.add_argument("--workload",
                   choices=["fourier", "readme", "precision", "adjoint", "batched", "equalize"],
                   default="fourier",
                   help="fourier: the headline 8192^2 float32 case (default); readme: the "
                        "reference's README case, 256^2 float64; precision: 8192^2 float64, "
                        "K=129, 10 iterations, exact vs FP16/BF16 storage forms; adjoint: "
                        "1024^2 float32, K=33, 3 iterations, forward + backward; batched: 64 "
                        "instances of sides 256-4096, K 17-129, 1-10 iterations; equalize: "
                        "histogram equalization of an 8192^2 float32 image")
    return p.parse_args()


def _replay_modes():
    from rlic_gb300 import _native

    return {"auto": _native.RLIC_REPLAY_AUTO, "l1": _native.RLIC_REPLAY_L1,
            "staged": _native.RLIC_REPLAY_STAGED}


# the replay kernel each --replay choice runs in a step (the library's
# default stages the texture in shared memory)
STEP_REPLAY = {"auto": "staged", "l1": "l1", "staged": "staged"}


def config(n: int, replay: str = "auto") -> dict:
    return {
        "workload": f"fourier_vortex_{n}x{n}_f32_hann{KLEN}_polarization_xperiodic_yclosed_n{ITERS}",
        "size": [n, n],
        "klen": KLEN,
        "kernel": "hann",
        "uv_mode": "polarization",
        "boundaries": {"x": "periodic", "y": "closed"},
        "iterations": ITERS,
        "form": "path cache (pass 1 traces and records 4-bit step codes, passes 2-5 replay"
                + (" from TMA-staged shared-memory boxes)" if STEP_REPLAY[replay] == "staged"
                   else " through L1)"),
        "l2": "inputs larger than L2 (texture 256 MiB, packed field 512 MiB at 8192^2)",
    }


# ------------------------------------------------------------ distributed --

class Dist:
    def __init__(self) -> None:
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None

    def init(self, backend: str) -> None:
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self) -> None:
        if self.pg is not None:
            self.pg.barrier()

    def max(self, x: float, device) -> float:
        if self.pg is None:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64, device=device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.pg is not None:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------- clocks --

class ClockSampler:
    """nvidia-smi samples every 100 ms while the timed region runs.

    Entering starts nvidia-smi and returns once its first sample is written
    (or after STARTUP_S), so that a short timed region is not over before
    sampling begins; the samples written up to then precede the region and
    are left out of the summary (used only when none falls inside it).
    """

    FIELDS = ("pci.bus_id,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
    STARTUP_S = 5.0

    def __init__(self, pci: tuple[int, int, int] | None) -> None:
        self.pci = pci
        self.proc = None
        self.skip = 0
        fd, name = tempfile.mkstemp(prefix="rlic_clocks_", suffix=".csv")
        os.close(fd)
        self.path = Path(name)

    def _complete_lines(self) -> int:
        try:
            return self.path.read_text().count("\n")
        except OSError:
            return 0

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return self
        deadline = time.monotonic() + self.STARTUP_S
        while (time.monotonic() < deadline and self.proc.poll() is None
               and self._complete_lines() == 0):
            time.sleep(0.02)
        self.skip = self._complete_lines()
        return self

    def __exit__(self, *exc) -> None:
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    @staticmethod
    def _pci(text: str) -> tuple[int, int, int] | None:
        try:
            dom, bus, rest = text.strip().split(":")
            return int(dom, 16), int(bus, 16), int(rest.split(".")[0], 16)
        except ValueError:
            return None

    def summary(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        lines = self.path.read_text().splitlines()
        self.path.unlink(missing_ok=True)
        window = "timed region"
        if len(lines) > self.skip:
            lines = lines[self.skip:]
        elif lines:
            window = "just before the timed region (none fell inside it)"
        rows = [[x.strip() for x in line.split(",")] for line in lines]
        rows = [r for r in rows if len(r) == 8]
        if self.pci is not None and any(self._pci(r[0]) == self.pci for r in rows):
            rows = [r for r in rows if self._pci(r[0]) == self.pci]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x: str) -> float | None:
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        reasons = sorted({self.REASONS[i] for r in rows for i in range(4) if r[4 + i] == "Active"})
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": reasons,
            "samples": len(rows),
            "window": window,
        }


# ------------------------------------------------------------ roofline --

def compulsory_roofline(px: int, iters: int, elem: int, ms_step: float, peak: float) -> dict:
    """The compulsory-traffic figure of a whole step.

    Whatever the caches do, every pass reads the texture, u and v and writes
    its output once: 4 * elem bytes per pixel per iteration (16 B for
    float32).  Its rate over the measured step time bounds how far below
    the HBM roofline a step sits if nothing were re-read.
    """
    nbytes = 4 * elem * px * iters
    gbs = nbytes / (ms_step / 1e3) / 1e9
    return {"bytes_per_px_per_iter": 4 * elem, "bytes_per_step": nbytes,
            "achieved": gbs, "unit": "GB/s", "frac": gbs / peak}


# -------------------------------------------------------------- CPU legs --

def cpu_sample(case_np: dict, seconds: float, threads: int) -> dict:
    """Times the oracle on a band of rows of one pass, sized to ~`seconds`."""
    from oracle import oracle

    tex, u, v, k = (case_np[x] for x in ("texture", "u", "v", "kernel"))
    ny, nx = tex.shape
    kw = dict(uv_mode=case_np["uv_mode"], boundaries=case_np["boundaries"], nthreads=threads)
    rows = max(threads, 8)
    r0 = ny // 2
    t0 = time.perf_counter()
    oracle.sweep_rows(tex, u, v, k, r0, min(ny, r0 + rows), **kw)
    dt = time.perf_counter() - t0
    rows = int(min(ny, max(rows, rows * seconds / max(dt, 1e-6))))
    r0 = max(0, ny // 2 - rows // 2)
    t0 = time.perf_counter()
    oracle.sweep_rows(tex, u, v, k, r0, r0 + rows, **kw)
    dt = time.perf_counter() - t0
    samples = rows * nx * k.size
    return {
        "value": samples / dt / 1e9,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"rows [{r0}, {r0 + rows}) of one pass over the {ny}x{nx} workload "
                  f"({samples:.3e} samples, {dt:.2f} s) with the C oracle, {threads} threads",
        "seconds": dt,
    }


def run_reference(args, dist: Dist) -> None:
    """The CPU restatement of the reference's implementation, timed on the host."""
    if dist.rank != 0:
        return
    from oracle import oracle
    from rlic_gb300.workloads import fourier_vortex_case

    threads = oracle.env_threads()
    case = fourier_vortex_case(n=args.size, device="cpu")
    per_step = max(2.0, 150.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_sample(case, min(per_step, 3.0), threads)
    vals, times = [], []
    for _ in range(args.steps):
        r = cpu_sample(case, per_step, threads)
        vals.append(r["value"])
        times.append(r["seconds"])
    value = float(statistics.median(vals))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * float(statistics.median(times)),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Fourier modes + point vortices, 1% zero cells)",
        "config": config(args.size),
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": r["sample"] + "; the reference's Rust core cannot be built here "
                      "(no Rust toolchain), so its C restatement is timed",
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU leg --

def run_gb300(args, dist: Dist) -> None:
    import torch

    import rlic_gb300
    from rlic_gb300 import _native
    from rlic_gb300.workloads import fourier_vortex_case

    dist.init("nccl")
    dev = torch.device("cuda", dist.local_rank)
    torch.cuda.set_device(dev)
    lib = _native.lib()
    _native.set_replay_mode(_replay_modes()[args.replay])
    n = args.size
    case = fourier_vortex_case(n=n, device=str(dev), as_numpy=False)
    tex, u, v, k = (case[x].contiguous() for x in ("texture", "u", "v", "kernel"))
    bcodes = (1, 1, 0, 0)
    uv_code = 1
    samples = n * n * KLEN * ITERS
    out = torch.empty_like(tex)
    nbytes = lib.rlic_workspace_bytes(n, n, KLEN, ITERS, 4, 0)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step() -> None:
        _native.check(lib.rlic_convolve_f32(
            tex.data_ptr(), u.data_ptr(), v.data_ptr(), n, n, k.data_ptr(), KLEN, uv_code,
            *bcodes, ITERS, out.data_ptr(), ws.data_ptr(), nbytes, sp, 0))

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize(dev)
    props = torch.cuda.get_device_properties(dev)
    pci = None
    if all(hasattr(props, a) for a in ("pci_domain_id", "pci_bus_id", "pci_device_id")):
        pci = (props.pci_domain_id, props.pci_bus_id, props.pci_device_id)

    launches0 = _native.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(pci) as clocks:
        dist.barrier()
        torch.cuda.synchronize(dev)
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        dist.barrier()
    launches = _native.launch_count() - launches0
    ms_local = ev0.elapsed_time(ev1)
    ms_total = dist.max(ms_local, dev)
    ms_step = ms_total / args.steps
    value = dist.world * samples * args.steps / (ms_total / 1e3) / 1e9

    # ---- the plain form (every pass traced) on the same workload
    plain_steps = max(3, min(args.steps, 8))
    flags_plain = _native.RLIC_FLAG_NO_PATH_CACHE

    def step_plain() -> None:
        _native.check(lib.rlic_convolve_f32(
            tex.data_ptr(), u.data_ptr(), v.data_ptr(), n, n, k.data_ptr(), KLEN, uv_code,
            *bcodes, ITERS, out.data_ptr(), ws.data_ptr(), nbytes, sp, flags_plain))

    step_plain()
    torch.cuda.synchronize(dev)
    ev0.record(stream)
    for _ in range(plain_steps):
        step_plain()
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    plain_ms = dist.max(ev0.elapsed_time(ev1), dev) / plain_steps
    plain_value = dist.world * samples / (plain_ms / 1e3) / 1e9

    # ---- per-kernel timing on the launching stream (each launch bracketed)
    uv = torch.empty((n, n, 2), dtype=torch.float32, device=dev)
    _native.check(lib.rlic_pack_field_f32(u.data_ptr(), v.data_ptr(), n, n, uv.data_ptr(), sp))
    codes = torch.empty(lib.rlic_path_code_bytes(n, n, KLEN), dtype=torch.uint8, device=dev)
    tmp = torch.empty_like(tex)
    reps = max(6, min(args.steps, 12))

    def timed(launch) -> float:
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(reps + 2)]
        for a, b in evs:
            a.record(stream)
            launch()
            b.record(stream)
        torch.cuda.synchronize(dev)
        return statistics.mean(a.elapsed_time(b) for a, b in evs[2:])

    # as in the timed steps, whose pack finds the field free of NaN samples
    nan_free = not bool(torch.isnan(uv).any())
    sweep_flags = _native.RLIC_FLAG_FIELD_NAN_FREE if nan_free else 0

    def sweep(code_ptr):
        return lambda: _native.check(lib.rlic_sweep_f32(
            tex.data_ptr(), uv.data_ptr(), n, n, k.data_ptr(), KLEN, uv_code, *bcodes,
            tmp.data_ptr(), code_ptr, sp, sweep_flags))

    ms_trace_rec = timed(sweep(codes.data_ptr()))
    ms_trace = timed(sweep(None))
    def replay():
        _native.check(lib.rlic_replay_f32(
            tex.data_ptr(), codes.data_ptr(), n, n, k.data_ptr(), KLEN, tmp.data_ptr(), sp,
            sweep_flags))

    replay_ms = {}
    for name, mode in (("l1", _native.RLIC_REPLAY_L1), ("staged", _native.RLIC_REPLAY_STAGED)):
        _native.set_replay_mode(mode)
        replay_ms[name] = timed(replay)
    _native.set_replay_mode(_replay_modes()[args.replay])
    ms_replay = replay_ms[STEP_REPLAY[args.replay]]
    ms_pack = timed(lambda: _native.check(lib.rlic_pack_field_f32(
        u.data_ptr(), v.data_ptr(), n, n, uv.data_ptr(), sp)))
    del uv, tmp, codes

    peaks_path = REPO / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peak = float(json.loads(peaks_path.read_text())["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    px = n * n
    code_b = lib.rlic_path_code_bytes(n, n, KLEN) / px
    # algorithmic bytes per pixel of each kernel (cache-less gather model)
    alg = {
        "trace_record": 4 * (3 * KLEN - 1) + code_b,  # u, v, tex per step + centre + out + codes
        "trace": 4 * (3 * KLEN - 1),
        "replay": code_b + 4 * KLEN + 4,              # codes + tex per tap + out
        "pack": 16,                                    # u, v in, (u, v) out
    }
    alg["replay_l1"] = alg["replay_staged"] = alg["replay"]
    times = {"trace_record": ms_trace_rec, "trace": ms_trace, "replay": ms_replay,
             "replay_l1": replay_ms["l1"], "replay_staged": replay_ms["staged"],
             "pack": ms_pack}
    kernels = {}
    for name, ms in times.items():
        gbs = alg[name] * px / (ms / 1e3) / 1e9
        kernels[name] = {"ms": ms, "alg_bytes_per_px": alg[name], "achieved_gbs": gbs,
                         "frac": gbs / peak}
    per_step = {"trace_record": ms_trace_rec, "replay": (ITERS - 1) * ms_replay,
                "pack": ms_pack}
    dominant = max(per_step, key=per_step.get)
    for name, ms in per_step.items():
        kernels[name]["share_of_step"] = ms / sum(per_step.values())
    traffic = None
    tfile = REPO / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            t = json.loads(tfile.read_text())
            traffic = float(t[dominant]["dram_bytes_per_px"]) * px
        except Exception:
            traffic = None

    # ---- end to end through the public API on host numpy arrays: ordinary
    # pageable arrays, as a reference caller passes them (the headline e2e),
    # and the same data in page-locked buffers
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 10))

    def e2e_leg(host: dict) -> tuple[float, float]:
        kw = dict(kernel=host["kernel"], uv_mode="polarization",
                  boundaries={"x": "periodic", "y": "closed"}, iterations=ITERS)
        # warm-up as timed: each result is held while the next call runs, so
        # the pinned result cache holds two buffers before timing starts
        for _ in range(max(3, args.warmup)):
            res = rlic_gb300.convolve(host["texture"], host["u"], host["v"], **kw)
        dist.barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            res = rlic_gb300.convolve(host["texture"], host["u"], host["v"], **kw)
        torch.cuda.synchronize(dev)
        secs = dist.max(time.perf_counter() - t0, dev)
        dist.barrier()
        assert res.shape == (n, n) and isinstance(res, np.ndarray)
        return dist.world * samples * e2e_steps / secs / 1e9, 1e3 * secs / e2e_steps

    pageable = {name: t.cpu().numpy().copy()
                for name, t in (("texture", tex), ("u", u), ("v", v), ("kernel", k))}
    e2e_value, e2e_ms = e2e_leg(pageable)
    del pageable
    pinned = {}
    for name, t in (("texture", tex), ("u", u), ("v", v), ("kernel", k)):
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t)
        pinned[name] = h.numpy()
    e2e_pinned_value, e2e_pinned_ms = e2e_leg(pinned)
    del pinned

    line = None
    if dist.rank == 0:
        clk = clocks.summary()
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": dist.world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded Fourier modes + point vortices, 1% zero cells)",
            "config": config(n, args.replay),
            "gpu_launches": int(launches),
            "clocks": clk,
            "e2e": {
                "value": e2e_value,
                "unit": UNIT,
                "h2d_bytes_per_step": int(3 * n * n * 4 + KLEN * 4),
                "d2h_bytes_per_step": int(n * n * 4),
                "ms_per_step": e2e_ms,
                "path": "rlic_gb300.convolve(numpy arrays in ordinary pageable host memory) "
                        "-> rlic_convolve_f32 host-memory",
                "pinned": {"value": e2e_pinned_value, "ms_per_step": e2e_pinned_ms,
                           "path": "the same call on page-locked numpy arrays"},
            },
            "roofline": {
                "bound": "hbm",
                "kernel": {"trace_record": "lic_pass_kernel<float, fma, branchless, pol, record>",
                           "replay": ("lic_gather_staged_kernel<float, fma>"
                                      if STEP_REPLAY[args.replay] == "staged"
                                      else "lic_gather_kernel<float, fma>"),
                           "pack": "pack_uv_kernel<float>"}[dominant],
                "achieved": kernels[dominant]["achieved_gbs"],
                "peak": peak,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs, burst)",
                "unit": "GB/s",
                "frac": kernels[dominant]["frac"],
                "traffic": traffic,
                "algorithmic_bytes_per_launch": alg[dominant] * px,
                "launch_ms": times[dominant],
                "compulsory": compulsory_roofline(px, ITERS, 4, ms_step, peak),
            },
            "kernels": kernels,
            "forms": {
                "path_cache": {"value": value, "ms_per_step": ms_step},
                "plain": {"value": plain_value, "ms_per_step": plain_ms},
            },
        }
        # the CPU baseline is a single-GPU figure: at N > 1 the host cores
        # are shared with the other ranks' processes, so it is left out
        if not args.no_cpu_baseline and dist.world == 1:
            from oracle import oracle

            case_np = {x: case[x].cpu().numpy() for x in ("texture", "u", "v", "kernel")}
            case_np.update(uv_mode="polarization", boundaries={"x": "periodic", "y": "closed"})
            cb = cpu_sample(case_np, args.cpu_seconds, oracle.env_threads())
            cb.pop("seconds", None)
            line["cpu_baseline"] = cb
        print(json.dumps(line), flush=True)
    dist.close()


# ------------------------------------------------------- other workloads --

def _time_calls(fn, steps: int, warmup: int, stream) -> float:
    """Mean ms per call of fn() (CUDA events on `stream`)."""
    import torch

    for _ in range(max(1, warmup)):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def run_readme(args) -> None:
    """The reference's README case: 256^2 float64, K=65, periodic, velocity, n=1."""
    import torch

    import rlic_gb300
    from oracle import oracle
    from rlic_gb300 import _native
    from rlic_gb300.workloads import readme_case

    c = readme_case()
    lib = _native.lib()
    n, klen = 256, 65
    dev = torch.device("cuda", 0)
    t = {x: torch.from_numpy(np.ascontiguousarray(c[x])).to(dev) for x in ("texture", "u", "v", "kernel")}
    out = torch.empty_like(t["texture"])
    nbytes = lib.rlic_workspace_bytes(n, n, klen, 1, 8, 0)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def call():
        _native.check(lib.rlic_convolve_f64(
            t["texture"].data_ptr(), t["u"].data_ptr(), t["v"].data_ptr(), n, n,
            t["kernel"].data_ptr(), klen, 0, 1, 1, 1, 1, 1, out.data_ptr(), ws.data_ptr(),
            nbytes, sp, 0))

    steps = max(args.steps, 50)
    ms = _time_calls(call, steps, args.warmup, stream)
    # the same calls with one thread per pixel (no paired pass), for comparison
    _native.set_split_pixels(0)
    ms_one_thread = _time_calls(call, steps, args.warmup, stream)
    _native.set_split_pixels(-1)
    # the call recorded into a CUDA graph (rlic_gb300.forms.ConvolvePlan)
    from rlic_gb300.forms import ConvolvePlan

    plan = ConvolvePlan(t["texture"], t["u"], t["v"], kernel=t["kernel"], boundaries="periodic")
    plan.capture()
    ms_graph = _time_calls(plan.replay, steps, args.warmup, stream)
    samples = n * n * klen
    for _ in range(max(3, args.warmup)):
        res = rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"],
                                  boundaries="periodic")
    t0 = time.perf_counter()
    for _ in range(steps):
        rlic_gb300.convolve(c["texture"], c["u"], c["v"], kernel=c["kernel"], boundaries="periodic")
    e2e_ms = (time.perf_counter() - t0) * 1e3 / steps
    res = {}
    for threads in () if args.no_cpu_baseline else (1, oracle.env_threads()):
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            oracle.convolve(c["texture"], c["u"], c["v"], c["kernel"], boundaries="periodic",
                            nthreads=threads)
        res[threads] = samples * reps / (time.perf_counter() - t0) / 1e9
    print(json.dumps({
        "metric": METRIC, "unit": UNIT, "workload": "readme_256x256_f64_triangle65_periodic_velocity_n1",
        "value": samples / (ms / 1e3) / 1e9, "ms_per_call": ms, "dtype": "f64", "steps": steps,
        "forms": {"paired": {"ms_per_call": ms}, "one_thread_per_pixel": {"ms_per_call": ms_one_thread},
                  "graph_replay": {"ms_per_call": ms_graph}},
        "e2e": {"value": samples / (e2e_ms / 1e3) / 1e9, "ms_per_call": e2e_ms},
        "cpu_oracle_gsamples": {f"{k}_threads": v for k, v in res.items()},
    }), flush=True)


def run_precision(args) -> None:
    """8192^2 float64 (README recipe, seed 2), K=129 triangle, periodic, n=10:
    the exact plain and path-cache forms against the FP16 / BF16 storage forms."""
    import torch

    from rlic_gb300 import _native
    from rlic_gb300.workloads import readme_case

    n, klen, iters = args.size, 129, 10
    c = readme_case(n=n, klen=klen, dtype=np.float64, seed=2)
    dev = torch.device("cuda", 0)
    t = {x: torch.from_numpy(np.ascontiguousarray(c[x])).to(dev) for x in ("texture", "u", "v", "kernel")}
    lib = _native.lib()
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    samples = n * n * klen * iters
    outs, times = {}, {}
    for name, flags in (("f64_plain", _native.RLIC_FLAG_NO_PATH_CACHE), ("f64_path_cache", 0)):
        out = torch.empty_like(t["texture"])
        nbytes = lib.rlic_workspace_bytes(n, n, klen, iters, 8, flags)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)

        def call(out=out, ws=ws, nbytes=nbytes, flags=flags):
            _native.check(lib.rlic_convolve_f64(
                t["texture"].data_ptr(), t["u"].data_ptr(), t["v"].data_ptr(), n, n,
                t["kernel"].data_ptr(), klen, 0, 1, 1, 1, 1, iters, out.data_ptr(),
                ws.data_ptr(), nbytes, sp, flags))

        times[name] = _time_calls(call, 2 if "plain" in name else 3, 1, stream)
        outs[name] = out
        del ws
    for name, st in (("fp16", _native.RLIC_STORAGE_FP16), ("bf16", _native.RLIC_STORAGE_BF16)):
        out = torch.empty_like(t["texture"])
        nbytes = lib.rlic_lowp_workspace_bytes(n, n, klen, 8)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)

        def call(out=out, ws=ws, nbytes=nbytes, st=st):
            _native.check(lib.rlic_convolve_lowp_f64(
                t["texture"].data_ptr(), t["u"].data_ptr(), t["v"].data_ptr(), n, n,
                t["kernel"].data_ptr(), klen, 0, 1, 1, 1, 1, iters, st, out.data_ptr(),
                ws.data_ptr(), nbytes, sp, 0))

        times[name] = _time_calls(call, 3, 1, stream)
        outs[name] = out
        del ws
    exact = outs["f64_plain"]
    assert torch.equal(exact, outs["f64_path_cache"]), "path-cache form differs from plain"
    scale = float(torch.sum(torch.abs(t["kernel"]))) ** iters
    errs = {}
    for name in ("fp16", "bf16"):
        d = (outs[name] - exact) / scale
        errs[name] = {"max_abs": float(d.abs().max()), "rms": float(torch.sqrt((d * d).mean()))}
    forms = {k: {"ms_per_step": v, "value": samples / (v / 1e3) / 1e9} for k, v in times.items()}
    for k in ("fp16", "bf16"):
        forms[k]["error_vs_f64_normalised"] = errs[k]
        forms[k]["speedup_vs_f64_plain"] = times["f64_plain"] / times[k]
        forms[k]["speedup_vs_f64_path_cache"] = times["f64_path_cache"] / times[k]
    print(json.dumps({
        "metric": METRIC, "unit": UNIT,
        "workload": f"readme_recipe_{n}x{n}_f64_triangle{klen}_periodic_velocity_n{iters}",
        "value": forms["fp16"]["value"], "dtype": "f64 in, fp16 storage",
        "forms": forms, "error_normalisation": "outputs divided by sum(|kernel|)^iterations",
    }), flush=True)


def run_adjoint(args) -> None:
    """1024^2 float32 (README recipe, seed 4), K=33 triangle, periodic, n=3;
    loss = sum(W * out), W ~ N(0, 1): forward + backward through
    rlic_gb300.forms.convolve_autograd."""
    import torch

    from rlic_gb300.forms import convolve_autograd
    from rlic_gb300.workloads import readme_case

    n, klen, iters = 1024, 33, 3
    c = readme_case(n=n, klen=klen, dtype=np.float32, seed=4)
    dev = torch.device("cuda", 0)
    t = {x: torch.from_numpy(np.ascontiguousarray(c[x])).to(dev) for x in ("texture", "u", "v", "kernel")}
    W = torch.from_numpy(np.random.default_rng(4).normal(size=(n, n)).astype(np.float32)).to(dev)
    stream = torch.cuda.current_stream(dev)

    def fwd_bwd():
        tex = t["texture"].detach().requires_grad_(True)
        k = t["kernel"].detach().requires_grad_(True)
        out = convolve_autograd(tex, t["u"], t["v"], kernel=k, boundaries="periodic",
                                iterations=iters)
        (out * W).sum().backward()
        return tex.grad, k.grad

    def fwd():
        with torch.no_grad():
            convolve_autograd(t["texture"], t["u"], t["v"], kernel=t["kernel"],
                              boundaries="periodic", iterations=iters)

    steps = max(args.steps, 20)
    ms_fb = _time_calls(fwd_bwd, steps, args.warmup, stream)
    ms_f = _time_calls(fwd, steps, args.warmup, stream)
    samples = n * n * klen * iters
    print(json.dumps({
        "metric": METRIC, "unit": UNIT,
        "workload": f"readme_recipe_{n}x{n}_f32_triangle{klen}_periodic_velocity_n{iters}_fwd_bwd",
        "value": samples / (ms_fb / 1e3) / 1e9, "ms_per_step": ms_fb, "dtype": "f32",
        "forward_only": {"ms": ms_f, "value": samples / (ms_f / 1e3) / 1e9},
        "note": "value = forward samples per second of forward + backward (d/dtexture, d/dkernel)",
    }), flush=True)


def run_equalize(args) -> None:
    """Histogram equalization of an 8192^2 float32 LIC-like image (uniform^3,
    seed 0), 256 bins: global, sliding tile (65 x 65 windows) and tile
    interpolation (64 x 64 tiles), device-resident."""
    import torch

    from rlic_gb300 import equalize as E

    n, nbins = args.size, 256
    dev = torch.device("cuda", 0)
    gen = torch.Generator(device=dev).manual_seed(0)
    x = torch.rand((n, n), generator=gen, device=dev, dtype=torch.float32) ** 3
    stream = torch.cuda.current_stream(dev)
    forms = {
        "global": lambda: E.equalize_histogram(x, nbins),
        "sliding_tile_65x65": lambda: E.equalize_histogram_sliding_tile(x, nbins, (65, 65)),
        "tile_interpolation_64x64": lambda: E.equalize_histogram_tile_interpolation(
            x, nbins, (64, 64)),
    }
    res = {}
    for name, fn in forms.items():
        ms = _time_calls(fn, max(3, min(args.steps, 10)), args.warmup, stream)
        res[name] = {"ms": ms, "gpx_per_s": n * n / (ms / 1e3) / 1e9}
    print(json.dumps({
        "metric": "Gpixels/s", "unit": "Gpx/s", "workload": f"equalize_{n}x{n}_f32_bins{nbins}",
        "value": res["global"]["gpx_per_s"], "dtype": "f32", "forms": res,
        "note": "post-processing of the LIC output; no counterpart implemented in the reference",
    }), flush=True)


def run_batched(args) -> None:
    """Two batched mixes (rlic_gb300.workloads.batch_case): the 64-instance
    workload (sides 256-4096, seed 3) and 256 small instances (sides
    128-512, seed 5), each with kernels of 17-129 taps and 1-10 iterations.
    Per mix: the batched call (items of 2^21 pixels and more as their own
    calls, the rest in one launch per level with tuned tiles; also replayed
    from a CUDA graph), every item batched per level, every item in the
    persistent work-queue launch, and one rlic_convolve_f32 call per
    instance in its path-cache and plain forms."""
    import torch

    from rlic_gb300 import _native
    from rlic_gb300._boundaries import BoundarySet
    from rlic_gb300.batch import BatchPlan, autotune_tiles
    from rlic_gb300.workloads import batch_case

    lib = _native.lib()
    steps = max(3, min(args.steps, 10))

    def gs(samples, ms):
        return samples / (ms / 1e3) / 1e9

    def measure(items) -> dict:
        dev = items[0]["texture"].device
        stream = torch.cuda.current_stream(dev)
        sp = ctypes.c_void_p(stream.cuda_stream)
        t0 = time.perf_counter()
        choice = autotune_tiles(items)
        tune_s = time.perf_counter() - t0
        plan = BatchPlan(items)
        samples = plan.samples()
        ms_levels = _time_calls(plan.run, steps, args.warmup, stream)
        plan.capture()
        ms_graph = _time_calls(plan.replay, steps, args.warmup, stream)
        every = BatchPlan(items, solo_pixels=0)
        ms_every = _time_calls(every.run, steps, args.warmup, stream)
        queue = BatchPlan(items, queue=True, solo_pixels=0)
        ms_queue = _time_calls(queue.run, steps, args.warmup, stream)
        assert queue.status(), "a bounded wait of the work queue gave up"
        seq = []
        for it, t in zip(items, plan.inputs):
            ny, nx = t["texture"].shape
            bc = BoundarySet.from_spec(it["boundaries"]).codes()
            seq.append((t, ny, nx, t["kernel"].shape[0], it["iterations"],
                        _native.UV_MODE_CODES[it["uv_mode"]], bc, torch.empty_like(t["texture"])))
        wsmax = max(lib.rlic_workspace_bytes(ny, nx, klen, n, 4, 0)
                    for _, ny, nx, klen, n, _, _, _ in seq)
        ws = torch.empty(wsmax, dtype=torch.uint8, device=dev)

        def sequential(flags):
            def go():
                for t, ny, nx, klen, n, mode, bc, out in seq:
                    _native.check(lib.rlic_convolve_f32(
                        t["texture"].data_ptr(), t["u"].data_ptr(), t["v"].data_ptr(), ny, nx,
                        t["kernel"].data_ptr(), klen, mode, *bc, n, out.data_ptr(),
                        ws.data_ptr(), wsmax, sp, flags))
            return go

        ms_seq = _time_calls(sequential(0), steps, args.warmup, stream)
        ms_seq_plain = _time_calls(sequential(_native.RLIC_FLAG_NO_PATH_CACHE), 2, 1, stream)
        for (_, _, _, _, _, _, _, out), a, b, c in zip(seq, plan.outputs, queue.outputs,
                                                      every.outputs):
            assert torch.equal(out, a) and torch.equal(out, b) and torch.equal(out, c), \
                "batched result differs"
        return {
            "instances": len(items),
            "pixels": int(sum(int(i["texture"].numel()) for i in items)),
            "samples_per_step": samples,
            "forms": {
                "batched_graph_replay": {"ms": ms_graph, "value": gs(samples, ms_graph)},
                "batched_call": {"ms": ms_levels, "value": gs(samples, ms_levels)},
                "every_item_batched_per_level": {"ms": ms_every, "value": gs(samples, ms_every)},
                "every_item_batched_queue": {"ms": ms_queue, "value": gs(samples, ms_queue)},
                "sequential_path_cache_calls": {"ms": ms_seq, "value": gs(samples, ms_seq)},
                "sequential_plain_calls": {"ms": ms_seq_plain,
                                           "value": gs(samples, ms_seq_plain)},
            },
            "autotune": {"seconds": tune_s,
                         "choices": {str(k): list(v) for k, v in choice.items()}},
        }

    mixes = {
        "batch_64_instances_seed3": measure(batch_case(count=64, seed=3)),
        "batch_256_small_instances_seed5": measure(
            batch_case(count=256, seed=5, min_side=128, max_side=512)),
    }
    head = mixes["batch_64_instances_seed3"]["forms"]["batched_graph_replay"]["value"]
    print(json.dumps({
        "metric": METRIC, "unit": UNIT, "workload": "batch_64_instances_seed3",
        "value": head, "dtype": "f32", "mixes": mixes,
    }), flush=True)


def run_batched_sharded(args, dist: Dist) -> None:
    """The 64-instance batch (seed 3) split by instance across the ranks
    (rlic_gb300.batch.shard_items: whole instances, balanced by samples, no
    data exchanged).  Each rank tunes and records its share as a CUDA graph
    and replays it; value = the whole batch's samples per second over the
    slowest rank (strong scaling: the batch is fixed)."""
    import torch

    from rlic_gb300.batch import BatchPlan, autotune_tiles, item_samples, shard_items
    from rlic_gb300.workloads import batch_case

    dist.init("nccl")
    dev = torch.device("cuda", dist.local_rank)
    torch.cuda.set_device(dev)
    items = batch_case(count=64, seed=3, device="cpu")
    total = sum(item_samples(it) for it in items)
    mine = shard_items(items, dist.world)[dist.rank]
    share = [{**items[k], **{x: items[k][x].to(dev) for x in ("texture", "u", "v", "kernel")}}
             for k in mine]
    plan = None
    if share:
        autotune_tiles(share)
        plan = BatchPlan(share)
        plan.capture()
    stream = torch.cuda.current_stream(dev)
    steps = max(3, min(args.steps, 10))
    for _ in range(max(3, args.warmup)):
        if plan is not None:
            plan.replay()
    torch.cuda.synchronize(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize(dev)
    ev0.record(stream)
    for _ in range(steps):
        if plan is not None:
            plan.replay()
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    dist.barrier()
    ms = dist.max(ev0.elapsed_time(ev1), dev) / steps
    if dist.rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": total / (ms / 1e3) / 1e9, "unit": UNIT,
            "n_gpus": dist.world, "steps": steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (batch_case: 64 instances, seed 3)",
            "workload": "batch_64_instances_seed3",
            "config": {"workload": "batch_64_instances_seed3", "instances": len(items),
                       "sharding": f"{dist.world} ranks, whole instances balanced by samples, "
                                   "no exchange"},
        }), flush=True)
    dist.close()


def run_shard(args, dist: Dist) -> None:
    """Strong scaling of one image: the 8192^2 workload split into row bands,
    one per rank (rlic_gb300.sharding), each band device-resident with its
    own path cache, halo rows exchanged over NCCL between passes.  value =
    the image's samples per second over the slowest rank."""
    import torch

    from rlic_gb300.sharding import GpuBandEngine, HaloExchange, ShardPlan
    from rlic_gb300.workloads import fourier_vortex_case

    dist.init("nccl")
    dev = torch.device("cuda", dist.local_rank)
    torch.cuda.set_device(dev)
    n = args.size
    case = fourier_vortex_case(n=n, device="cpu")
    plan = ShardPlan(n, dist.world, KLEN // 2, periodic_y=False)
    spec = plan.local_boundaries({"x": ("periodic", "periodic"), "y": ("closed", "closed")})
    rows = plan.ext_rows[dist.rank]
    eng = GpuBandEngine(case["u"][rows], case["v"][rows], case["kernel"], "polarization", spec,
                        ITERS, device=dev)
    halo = HaloExchange(plan, dist.rank)
    tex0 = torch.from_numpy(np.ascontiguousarray(case["texture"][rows])).to(dev)

    def step():
        t = tex0
        for it in range(ITERS):
            out = eng.first(t) if it == 0 else eng.next(t)
            if it + 1 < ITERS:
                halo.refresh(out)  # halo rows of the output band, in place
                t = out
        return out

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize(dev)
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize(dev)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    dist.barrier()
    ms = dist.max(ev0.elapsed_time(ev1), dev) / args.steps
    samples = n * n * KLEN * ITERS
    if dist.rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": samples / (ms / 1e3) / 1e9, "unit": UNIT,
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Fourier modes + point vortices, 1% zero cells)",
            "config": {**config(n, args.replay),
                       "sharding": f"{dist.world} row bands with a {KLEN // 2}-row halo, "
                                   "halo rows exchanged between passes"},
        }), flush=True)
    dist.close()


def main() -> None:
    args = parse_args()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
        return
    if args.workload == "readme":
        run_readme(args)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "equalize":
        run_equalize(args)
    elif args.workload == "batched":
        if dist.world > 1:
            run_batched_sharded(args, dist)
        else:
            run_batched(args)
    elif args.shard:
        run_shard(args, dist)
    else:
        run_gb300(args, dist)


if __name__ == "__main__":
    main()
