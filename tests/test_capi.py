"""The C ABI library loads, exports every declared symbol, and rejects bad
arguments with status codes -- all without touching a GPU (argument checks
run before any CUDA call)."""

from __future__ import annotations

import re
from pathlib import Path

import pytest

from rlic_gb300 import _native

HEADER = Path(__file__).resolve().parents[1] / "include" / "rlic_gb300.h"


def declared_symbols() -> list[str]:
    text = HEADER.read_text()
    return re.findall(r"RLIC_API\s+[\w\s\*]+?\b(rlic_\w+)\s*\(", text)


def test_header_declares_the_binding_table() -> None:
    assert sorted(declared_symbols()) == sorted(_native.SIGNATURES)


def test_integration_guide_lists_every_entry_point() -> None:
    guide = (HEADER.parents[1] / "INTEGRATION.md").read_text()
    for name in declared_symbols():
        assert f"`{name}`" in guide or f"`{name[:-4]}" in guide, name


def test_library_exports_every_declared_symbol(native) -> None:
    for name in declared_symbols():
        assert hasattr(native, name), name


def test_version(native) -> None:
    assert native.rlic_version().decode().startswith("rlic_gb300")


def test_workspace_bytes(native) -> None:
    ws = native.rlic_workspace_bytes
    n = 8192 * 8192
    # one pass: packed (u, v) + kernel copy + the field's NaN flag
    assert ws(8192, 8192, 65, 1, 4, 0) == 2 * n * 4 + 512 + 256
    # five passes: + ping-pong buffer + path cache (8 words of 8 steps per pixel)
    assert ws(8192, 8192, 65, 5, 4, 0) == 3 * n * 4 + 8 * 4 * n + 512 + 256
    assert ws(8192, 8192, 65, 5, 4, 0x8) == 3 * n * 4 + 512 + 256
    assert ws(10, 10, 3, 2, 8, 0) == 1792 + 1024 + 1024 + 256 + 256
    assert ws(10, 10, 3, 2, 8, 0x8) == 1792 + 1024 + 256 + 256
    assert ws(0, 10, 3, 1, 4, 0) == 0
    assert ws(10, 10, 3, 1, 2, 0) == 0
    # a small image traced by the paired pass keeps no path cache for one
    # pass, whatever the paired threshold
    for split in (1 << 40, 0, -1):
        assert native.rlic_set_split_pixels(split) == 0
        assert ws(256, 256, 65, 1, 8, 0) == 2 * 65536 * 8 + 768 + 256


def test_path_code_bytes(native) -> None:
    pc = native.rlic_path_code_bytes
    assert pc(8192, 8192, 65) == 8 * 4 * 8192 * 8192  # 32 + 32 steps
    assert pc(10, 10, 129) == 16 * 4 * 100  # 64 + 64 steps
    assert pc(10, 10, 2) == 1 * 4 * 100  # 0 forward + 1 backward step
    assert pc(10, 10, 18) == (1 + 2) * 4 * 100  # 8 forward + 9 backward steps
    assert pc(0, 10, 3) == 0


def _call(native, **over):
    args = dict(texture=1, u=1, v=1, ny=4, nx=4, kernel=1, klen=3, uv_mode=0, bxl=0, bxr=0,
                byl=0, byr=0, iterations=1, out=1, ws=None, wsb=0, stream=None, flags=0)
    args.update(over)
    return native.rlic_convolve_f32(*args.values())


@pytest.mark.parametrize(
    "over, text",
    [
        (dict(ny=0), "dimensions"),
        (dict(nx=-3), "dimensions"),
        (dict(klen=0), "at least one tap"),
        (dict(uv_mode=2), "uv_mode"),
        (dict(bxr=2), "boundaries"),
        (dict(iterations=-1), "iterations"),
        (dict(texture=None), "null"),
        (dict(flags=0x100), "flag"),
        (dict(klen=1 << 21), "too long"),
    ],
)
def test_argument_errors(native, over, text) -> None:
    rc = _call(native, **over)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT
    assert text in native.rlic_last_error().decode()


def test_check_raises(native) -> None:
    _call(native, ny=0)
    with pytest.raises(_native.NativeLibraryError, match="dimensions"):
        _native.check(_native.RLIC_ERR_INVALID_ARGUMENT)


def test_trace_argument_errors(native) -> None:
    rc = native.rlic_trace_cells_f64(1, 1, 4, 4, 3, 0, 0, 0, 0, 0, -1, 1, 1, None, 0)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT


def test_sweep_and_replay_argument_errors(native) -> None:
    # host-memory flag is not accepted by the device-only building blocks
    rc = native.rlic_sweep_f32(1, 1, 4, 4, 1, 3, 0, 0, 0, 0, 0, 1, None, None, 0x1)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT
    rc = native.rlic_replay_f32(1, 1, 4, 4, 1, 3, 1, None, 0x4)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT
    rc = native.rlic_replay_f64(1, None, 4, 4, 1, 3, 1, None, 0)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT
    rc = native.rlic_pack_field_f32(1, 1, 4, 4, 3, None)  # misaligned pair array
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT


def test_batch_argument_errors(native) -> None:
    assert native.rlic_convolve_batch_f32(None, 0, None, 0, None, 0) == _native.RLIC_ERR_INVALID_ARGUMENT
    items = (_native.BatchItemF32 * 1)()
    items[0] = _native.BatchItemF32(1, 1, 1, 1, 1, 8, 8, 5, 1, 0, 0, 0, 0, 0, 24)
    rc = native.rlic_convolve_batch_f32(items, 1, 256, 1 << 20, None, 0)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT
    assert "tile_x" in native.rlic_last_error().decode()
    items[0] = _native.BatchItemF32(1, 1, 1, 1, 1, 8, 8, 2049, 1, 0, 0, 0, 0, 0, 0)
    rc = native.rlic_convolve_batch_f32(items, 1, 256, 1 << 20, None, 0)
    assert rc == _native.RLIC_ERR_INVALID_ARGUMENT
    assert "1025 taps" in native.rlic_last_error().decode()
    items[0] = _native.BatchItemF32(1, 1, 1, 1, 1, 8, 8, 5, 1, 0, 0, 0, 0, 0, 0)
    assert native.rlic_batch_workspace_bytes_f32(items, 1) > 0
    rc = native.rlic_convolve_batch_f32(items, 1, 256, 16, None, 0)
    assert rc == _native.RLIC_ERR_WORKSPACE_TOO_SMALL


def test_block_shape_validation(native) -> None:
    assert native.rlic_set_block_shape(0, 4) == _native.RLIC_ERR_INVALID_ARGUMENT
    assert native.rlic_set_block_shape(64, 64) == _native.RLIC_ERR_INVALID_ARGUMENT
    assert native.rlic_set_block_shape(64, 4) == _native.RLIC_OK
    assert native.rlic_set_block_shape(0, 0) == _native.RLIC_OK  # back to the defaults
    assert native.rlic_set_split_pixels(-2) == _native.RLIC_ERR_INVALID_ARGUMENT
    assert native.rlic_set_split_pixels(-1) == _native.RLIC_OK  # the default threshold
    assert native.rlic_set_replay_mode(7, 0) == _native.RLIC_ERR_INVALID_ARGUMENT
    assert native.rlic_set_replay_mode(_native.RLIC_REPLAY_STAGED, 6) == \
        _native.RLIC_ERR_INVALID_ARGUMENT
    assert native.rlic_set_replay_mode(_native.RLIC_REPLAY_AUTO, 0) == _native.RLIC_OK


def test_missing_library_fails_loudly(monkeypatch, tmp_path) -> None:
    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "LIB_PATH", tmp_path / "librlic_gb300.so")
    with pytest.raises(_native.NativeLibraryError, match="not built"):
        _native.lib()
