"""Seeded Radiance RGBE pictures in every scanline coding the reference's HDRLoader reads
(src/loader/HDRLoader.cpp:84-152): flat pixels, flat pixels with (1, 1, 1, n) repeat pixels (the
older run-length form, including consecutive repeats whose counts scale by 256), adaptive
run-length scanlines (2, 2, width header, per-component run and literal packets), a narrow
picture whose flat pixels begin with the RLE marker bytes, and a picture mixing codings row by row.
`truncated()` writes a picture whose data ends inside a run-length scanline (this decoder stops
there; the reference's decoder keeps writing past its scanline buffer, so it has no golden). Used by tests/test_rgbe.py and tests/golden/make_rgbe_golden.py."""
from __future__ import annotations

from pathlib import Path

import numpy as np

HEADER = b"#?RADIANCE\n# seeded test picture\nFORMAT=32-bit_rle_rgbe\n\n"


def _pixels(rng, w: int, h: int) -> np.ndarray:
    px = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    px[..., 3] = rng.integers(100, 150, (h, w))  # exponents near the bias
    px[..., 0] = np.where(px[..., 0] < 3, 3, px[..., 0])  # no pixel reads as a repeat or RLE marker
    return px


def _flat_row(row: np.ndarray) -> bytes:
    return row.tobytes()


def _flat_row_with_repeats(rng, row: np.ndarray) -> bytes:
    """Pixels with runs of the previous pixel written as repeat pixels (never at the row start)."""
    out, x, w, after_repeat = bytearray(row[0].tobytes()), 1, row.shape[0], False
    while x < w:
        left = w - x
        if left > 3 and not after_repeat and rng.random() < 0.3:
            n = int(rng.integers(1, min(left, 255) + 1))
            out += bytes([1, 1, 1, n])
            row[x:x + n] = row[x - 1]
            x += n
            after_repeat = True  # a second repeat right after would scale its count by 256
        else:
            out += row[x].tobytes()
            x += 1
            after_repeat = False
    return bytes(out)


def _rle_row(rng, row: np.ndarray) -> bytes:
    w = row.shape[0]
    out = bytearray([2, 2, w >> 8, w & 255])
    for c in range(4):
        comp = row[:, c].copy()
        x = 0
        while x < w:
            left = w - x
            if left >= 2 and rng.random() < 0.4:  # a run packet
                n = int(rng.integers(1, min(left, 127) + 1))
                comp[x:x + n] = comp[x]
                out += bytes([128 + n, int(comp[x])])
            else:  # a literal packet
                n = int(rng.integers(1, min(left, 128) + 1))
                out += bytes([n]) + comp[x:x + n].tobytes()
            x += n
        row[:, c] = comp
    return bytes(out)


def write_all(d: Path) -> dict[str, Path]:
    rng = np.random.default_rng(2024)
    files = {}

    def put(name, w, h, rows):
        p = d / f"{name}.hdr"
        p.write_bytes(HEADER + f"-Y {h} +X {w}\n".encode() + b"".join(rows))
        files[name] = p

    px = _pixels(rng, 13, 5)
    put("flat", 13, 5, [_flat_row(r) for r in px])
    px = _pixels(rng, 300, 4)
    rows = [_flat_row_with_repeats(rng, r) for r in px]
    # two consecutive repeat pixels: 1 + (1 << 8) = 257 copies of the pixel before them
    rows[2] = px[2, 0].tobytes() + px[2, 1].tobytes() + bytes([1, 1, 1, 1, 1, 1, 1, 1]) + px[2, 259:].tobytes()
    put("flat_repeat", 300, 4, rows)
    px = _pixels(rng, 40, 6)
    put("rle", 40, 6, [_rle_row(rng, r) for r in px])
    px = _pixels(rng, 5, 3)
    px[:, 0] = [2, 2, 0, 5]  # flat: narrower than 8, so the RLE marker bytes are a pixel
    put("narrow", 5, 3, [_flat_row(r) for r in px])
    px = _pixels(rng, 24, 6)
    put("mixed", 24, 6, [(_rle_row(rng, r) if i % 2 else _flat_row(r)) for i, r in enumerate(px)])
    return files


def truncated(d: Path) -> tuple[Path, np.ndarray]:
    """A 32 x 5 run-length picture cut inside its fourth scanline, and its first three rows."""
    rng = np.random.default_rng(77)
    px = _pixels(rng, 32, 5)
    rows = [_rle_row(rng, r) for r in px]
    data = b"".join(rows[:3]) + rows[3][:len(rows[3]) // 2]
    p = d / "truncated.hdr"
    p.write_bytes(HEADER + b"-Y 5 +X 32\n" + data)
    return p, px[:3]
