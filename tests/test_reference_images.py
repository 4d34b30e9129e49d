"""The oracle and the GPU path against the reference's own published outputs.

The reference's Rust core cannot run here, but its repository ships the
figures of its README, drawn from results of that core: the README example
after 1, 5 and 100 iterations (``static/base_example_out.png``) and the
polarization example in both uv modes (``static/polarization_example.png``).
``tests/golden/figures/reference_images.npz`` holds their LIC panels (made by
``tests/golden/make_reference_images.py``): 340 x 340 pixels of viridis'
green channel, which rises monotonically with the mapped value.

To compare, a 256 x 256 result is drawn the way ``imshow`` drew it: the
image spans the 342-pixel axes frame, each frame pixel takes the two nearest
image pixels per axis with raised-cosine (Hann) weights, and the outermost
frame pixel, covered by the frame line, is cut.  The colour map is monotone,
so the rank (Spearman) correlation of the drawn result with the panel is
the measure.

The results match their panels to a rank correlation of 0.999 (the rest is
the colour map's 8-bit quantisation), while results that differ from the
reference's in any visible way (another iteration count, swapped or negated
components, other boundaries, the other uv mode) fall well below.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "figures" / "reference_images.npz"
MATCH = 0.998  # rank correlation of a result with its own panel


def draw(result: np.ndarray, frame: int) -> np.ndarray:
    """A square result drawn into a frame of `frame` pixels, frame line cut."""
    n = result.shape[0]
    t = np.clip((np.arange(frame) + 0.5) * n / frame - 0.5, 0, n - 1)
    i0 = np.floor(t).astype(np.int64)
    i1 = np.minimum(i0 + 1, n - 1)
    w1 = 0.5 - 0.5 * np.cos(np.pi * (t - i0))
    rows = result[i0] * (1 - w1)[:, None] + result[i1] * w1[:, None]
    out = rows[:, i0] * (1 - w1)[None, :] + rows[:, i1] * w1[None, :]
    return out[1:-1, 1:-1]


def rank_correlation(a: np.ndarray, b: np.ndarray) -> float:
    def ranks(x):
        r = np.empty(x.size)
        r[np.argsort(x.ravel(), kind="stable")] = np.arange(x.size)
        return r - r.mean()

    ra, rb = ranks(np.asarray(a, dtype=np.float64)), ranks(np.asarray(b, dtype=np.float64))
    return float((ra * rb).sum() / np.sqrt((ra * ra).sum() * (rb * rb).sum()))


def readme_inputs():
    """README.md:49-56 and 78 (the example the figures were drawn from)."""
    shape = (256, 256)
    texture = np.random.default_rng(0).random(shape)
    x = np.linspace(0, np.pi, 256)
    u = np.broadcast_to(np.cos(2 * x), shape)
    v = np.broadcast_to(np.sin(x).T, shape)
    kernel = 1 - np.abs(np.linspace(-1, 1, 65))
    return texture, u, v, kernel


def polarization_inputs():
    """README.md:115-124: u = -1 left of the middle column, +1 right of it."""
    shape = (256, 256)
    texture = np.random.default_rng(0).random(shape)
    kernel = 1 - np.abs(np.linspace(-1, 1, 65, dtype="float64"))
    ii = np.broadcast_to(np.arange(256), shape)
    u = np.where(ii < 128, -np.ones(shape), np.ones(shape))
    v = np.zeros(shape)
    return texture, u, v, kernel


POL_BOUNDARIES = {"x": "periodic", "y": "closed"}


@pytest.fixture(scope="module")
def panels():
    return np.load(GOLDEN)


def _check_readme_figure(conv, panels) -> None:
    texture, u, v, kernel = readme_inputs()
    frame = int(panels["frame"][0])
    drawn = {n: draw(conv(texture, u, v, kernel, "velocity", "periodic", n), frame)
             for n in (1, 5, 100)}
    for n in (1, 5, 100):
        panel = panels[f"base_n{n}"]
        corr = {m: rank_correlation(drawn[m], panel) for m in (1, 5, 100)}
        assert corr[n] > MATCH, corr
        # each panel is told apart from the other iteration counts
        assert max(c for m, c in corr.items() if m != n) < 0.8, corr
    # results that differ visibly from the reference's fall well below
    panel = panels["base_n1"]
    wrong = {
        "u and v swapped": conv(texture, v, u, kernel, "velocity", "periodic", 1),
        "u negated": conv(texture, -np.asarray(u), v, kernel, "velocity", "periodic", 1),
        "closed boundaries": conv(texture, u, v, kernel, "velocity", "closed", 1),
        "texture transposed": conv(np.ascontiguousarray(texture.T), u, v, kernel, "velocity",
                                   "periodic", 1),
    }
    for name, res in wrong.items():
        assert rank_correlation(draw(res, frame), panel) < 0.95, name


def _check_polarization_figure(conv, panels) -> None:
    texture, u, v, kernel = polarization_inputs()
    frame = int(panels["frame"][0])
    res = {m: conv(texture, u, v, kernel, m, POL_BOUNDARIES, 1)
           for m in ("velocity", "polarization")}
    drawn = {m: draw(r, frame) for m, r in res.items()}
    # where the two modes' results differ (along the sign changes of u)
    differ = draw((res["velocity"] != res["polarization"]).astype(np.float64), frame) > 0.99
    assert differ.sum() > 10_000
    for mode, other in (("velocity", "polarization"), ("polarization", "velocity")):
        panel = panels[f"pol_{mode}"]
        assert rank_correlation(drawn[mode], panel) > MATCH
        own = rank_correlation(drawn[mode][differ], panel[differ])
        cross = rank_correlation(drawn[other][differ], panel[differ])
        assert own > MATCH and cross < 0.8, (mode, own, cross)


def _oracle_conv(oracle):
    def conv(texture, u, v, kernel, uv_mode, boundaries, iterations):
        return oracle.convolve(texture, u, v, kernel, uv_mode=uv_mode, boundaries=boundaries,
                               iterations=iterations, nthreads=oracle.max_threads())
    return conv


def test_oracle_draws_the_readme_figure(oracle, panels) -> None:
    _check_readme_figure(_oracle_conv(oracle), panels)


def test_oracle_draws_the_polarization_figure(oracle, panels) -> None:
    _check_polarization_figure(_oracle_conv(oracle), panels)


def _gpu_conv(texture, u, v, kernel, uv_mode, boundaries, iterations):
    import rlic_gb300

    return rlic_gb300.convolve(texture, u, v, kernel=kernel, uv_mode=uv_mode,
                               boundaries=boundaries, iterations=iterations)


@pytest.mark.gpu
def test_gpu_draws_the_readme_figure(panels) -> None:
    _check_readme_figure(_gpu_conv, panels)


@pytest.mark.gpu
def test_gpu_draws_the_polarization_figure(panels) -> None:
    _check_polarization_figure(_gpu_conv, panels)
