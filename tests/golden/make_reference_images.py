"""Extracts the reference's published output images into a test fixture.

The reference repository ships the figures of its README
(``static/base_example_out.png``, ``static/polarization_example.png``,
drawn from ``README.md:68-96`` and ``README.md:107-145``).  They are the
only outputs of the reference's own Rust core that exist here: the core
cannot be built or run in this environment.  Each figure is a row of three
matplotlib axes; every LIC panel is a 256 x 256 result drawn with
``imshow`` (default viridis colour map, scaled to the result's own min and
max) into an axes frame 342 pixels wide.

This script decodes the two PNG files (zlib and the five PNG row filters,
no imaging library needed), cuts out the drawing area of every LIC panel
inside its frame lines, and stores its green channel (viridis' green rises
monotonically with the mapped value, so it orders pixels as the results
do) in ``figures/reference_images.npz``:

  base_n1, base_n5, base_n100   README example, 1, 5 and 100 iterations
  pol_velocity, pol_polarization  polarization example, both uv modes

Run from the repository root, with the reference checked out:
    python tests/golden/make_reference_images.py <path to the reference>
"""

from __future__ import annotations

import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

# Frame geometry of both figures (found from their frame lines): the axes
# frames span rows [32, 374) and columns [c0, c0 + 342) for c0 below, and
# the frame lines cover the outermost pixel on every side.
FRAME_ROWS = (32, 374)
FRAME_COLS = (10, 420, 831)
FRAME = 342


def read_png(path: Path) -> np.ndarray:
    """8-bit, non-interlaced PNG -> (h, w, channels) uint8."""
    data = path.read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat = 8, []
    width = height = channels = None
    while pos < len(data):
        length, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if kind == b"IHDR":
            width, height, depth, colour, _, _, interlace = struct.unpack(">IIBBBBB", body)
            if depth != 8 or interlace != 0:
                raise ValueError(f"{path}: only 8-bit non-interlaced PNG is supported")
            channels = {0: 1, 2: 3, 4: 2, 6: 4}[colour]
        elif kind == b"IDAT":
            idat.append(body)
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), dtype=np.uint8)
    stride = width * channels
    raw = raw.reshape(height, stride + 1)
    out = np.zeros((height, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int64)
    for y in range(height):
        kind, line = int(raw[y, 0]), raw[y, 1:].astype(np.int64)
        if kind == 0:
            cur = line
        elif kind == 2:
            cur = (line + prev) & 255
        else:  # Sub, Average and Paeth depend on the pixel to the left
            cur = np.zeros(stride, dtype=np.int64)
            for x in range(stride):
                a = int(cur[x - channels]) if x >= channels else 0
                c = int(prev[x - channels]) if x >= channels else 0
                b = int(prev[x])
                if kind == 1:
                    pred = a
                elif kind == 3:
                    pred = (a + b) >> 1
                else:
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (int(line[x]) + pred) & 255
        out[y] = cur
        prev = cur
    return out.reshape(height, width, channels)


def panels(img: np.ndarray) -> list[np.ndarray]:
    r0, r1 = FRAME_ROWS
    return [np.ascontiguousarray(img[r0 + 1:r1 - 1, c0 + 1:c0 + FRAME - 1, 1])
            for c0 in FRAME_COLS]


def main(reference: Path) -> None:
    base = panels(read_png(reference / "static" / "base_example_out.png"))
    pol = panels(read_png(reference / "static" / "polarization_example.png"))
    np.savez_compressed(
        HERE / "figures" / "reference_images.npz",
        base_n1=base[0], base_n5=base[1], base_n100=base[2],
        pol_velocity=pol[1], pol_polarization=pol[2],
        frame=np.array([FRAME], dtype=np.int64),
    )


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(Path(sys.argv[1]))
