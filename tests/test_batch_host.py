"""Host-side behaviour of rlic_gb300.batch.BatchPlan (no GPU needed).

A plan validates every item with convolve's rules and messages before it
allocates anything on a device: an empty batch, arrays that are not
tensors, tensors that are not float32 CUDA tensors and invalid arguments
are refused, naming the item at fault.
"""

from __future__ import annotations

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
