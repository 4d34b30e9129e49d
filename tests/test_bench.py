"""Host-side helpers of bench.py, without a GPU: the roofline arithmetic,
the workload description and the parsing of nvidia-smi clock samples."""

from __future__ import annotations

import os
import textwrap
import time

import pytest

import bench


def test_compulsory_roofline_arithmetic() -> None:
    # 8192^2 float32, 5 passes: 16 B per pixel per pass
    r = bench.compulsory_roofline(8192 * 8192, 5, 4, 20.0, 6790.3)
    assert r["bytes_per_px_per_iter"] == 16
    assert r["bytes_per_step"] == 16 * 5 * 8192 * 8192
    assert r["achieved"] == pytest.approx(16 * 5 * 8192 * 8192 / 0.020 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6790.3)
    assert r["unit"] == "GB/s"


def test_config_names_the_workload() -> None:
    c = bench.config(8192)
    assert c["workload"] == "fourier_vortex_8192x8192_f32_hann65_polarization_xperiodic_yclosed_n5"
    assert c["boundaries"] == {"x": "periodic", "y": "closed"}
    assert (c["klen"], c["iterations"]) == (bench.KLEN, bench.ITERS)
    assert "L2" in c["l2"]


class _Running:
    """Stands in for the nvidia-smi process once sampling has ended."""


def _summary(lines: list[str], pci=None) -> dict:
    clocks = bench.ClockSampler(pci)
    clocks.path.write_text("\n".join(lines) + "\n")
    clocks.proc = _Running()
    return clocks.summary()


def test_clock_summary_median_and_reasons() -> None:
    rows = [
        "00000009:01:00.0, 1965, 2070, 900.1, Not Active, Not Active, Not Active, Not Active",
        "00000009:01:00.0, 2070, 2070, 1100.0, Not Active, Not Active, Not Active, Active",
        "00000009:01:00.0, 2010, 2070, 1000.0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    s = _summary(rows)
    assert s["sm_mhz"] == 2010
    assert s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 3


def test_clock_summary_keeps_this_gpu_only() -> None:
    rows = [
        "00000009:01:00.0, 2070, 2070, 900, Not Active, Not Active, Not Active, Not Active",
        "00000019:01:00.0, 1200, 2070, 900, Active, Not Active, Not Active, Not Active",
    ]
    s = _summary(rows, pci=(9, 1, 0))
    assert s["sm_mhz"] == 2070 and s["reasons"] == [] and s["samples"] == 1
    # without a PCI match every row counts
    s = _summary(rows, pci=(0x30, 1, 0))
    assert s["samples"] == 2 and s["reasons"] == ["hw_slowdown"]


def test_clock_summary_without_samples() -> None:
    assert _summary([])["reasons"] == ["no samples"]
    clocks = bench.ClockSampler(None)
    assert clocks.summary()["reasons"] == ["nvidia-smi unavailable"]
    clocks.path.unlink(missing_ok=True)


_ROW = "00000009:01:00.0, {mhz}, 2070, 900, Not Active, Not Active, Not Active, Not Active"


def _fake_smi(tmp_path, monkeypatch, body: str) -> None:
    """An executable named nvidia-smi, first on PATH, running `body`."""
    exe = tmp_path / "nvidia-smi"
    exe.write_text("#!/usr/bin/env python3\n" + textwrap.dedent(body))
    exe.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")


def test_sampler_starts_before_the_region_and_skips_earlier_samples(tmp_path, monkeypatch):
    # the first sample (idle clock) precedes the region; later ones are under load
    _fake_smi(tmp_path, monkeypatch, f"""
        import time
        k = 0
        while True:
            print({_ROW!r}.format(mhz=1000 if k == 0 else 2070), flush=True)
            k += 1
            time.sleep(0.05)
    """)
    with bench.ClockSampler(None) as clocks:
        assert clocks.skip >= 1
        time.sleep(0.4)
    s = clocks.summary()
    assert s["window"] == "timed region"
    assert s["sm_mhz"] == 2070 and s["samples"] >= 2


def test_sampler_falls_back_to_samples_before_a_short_region(tmp_path, monkeypatch):
    _fake_smi(tmp_path, monkeypatch, f"""
        import time
        print({_ROW!r}.format(mhz=1980), flush=True)
        time.sleep(60)
    """)
    with bench.ClockSampler(None) as clocks:
        time.sleep(0.05)
    s = clocks.summary()
    assert s["window"].startswith("just before")
    assert s["sm_mhz"] == 1980 and s["samples"] == 1


def test_sampler_does_not_wait_for_a_silent_exit(tmp_path, monkeypatch):
    _fake_smi(tmp_path, monkeypatch, "raise SystemExit(9)\n")
    t0 = time.monotonic()
    with bench.ClockSampler(None) as clocks:
        pass
    assert time.monotonic() - t0 < bench.ClockSampler.STARTUP_S
    assert clocks.summary()["reasons"] == ["no samples"]
