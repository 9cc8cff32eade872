"""Generates the golden fixtures in tests/golden/*.npz from the REFERENCE
ITSELF: the reference's src/eikonal_fim.cpp and src/eikonal_fmm.cpp compiled
unmodified from their sources (oracle/Makefile target `ref`).

    python tests/golden/make_golden.py [REF_SRC_DIR]

Each fixture holds the cost field, the seeds and the reference's FIM fields
(at eps 1e-5 and 1e-3, the harness value of src/test_runner.cpp:17) and FMM
field. Inputs are the seeded synthetic generators of ghcm_gb300.fields plus
the reference's own binary ring images data/7_ring_32_2d.png and
data/7_ring_256_2d.png, decoded here as the reference's loader does (stb grey
conversion y = (77 r + 150 g + 29 b) >> 8, then (y / 255)^2.2 as the LDR->float
mapping; the images are pure 0/255, so speed is exactly 0 or 1; cost = 1/speed,
src/test_runner.cpp:38-45; seed (0, 0), src/test_runner.cpp:314).

Test infrastructure only; needs the reference sources, so it runs in the
development container, never on the GPU machine (which only reads the .npz files).
"""
from __future__ import annotations

import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from ghcm_gb300 import fields  # noqa: E402
from oracle import oracle  # noqa: E402


def decode_png_rgba8(path: Path) -> np.ndarray:
    """Minimal decoder for non-interlaced 8-bit RGBA PNGs: returns [H, W, 4] uint8."""
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", path
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype, _, _, interlace = hdr
    assert depth == 8 and ctype == 6 and interlace == 0, hdr
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8)
    bpp, stride = 4, w * 4
    out = np.zeros((h, stride), dtype=np.int32)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        line = raw[y * (stride + 1):(y + 1) * (stride + 1)]
        ftype, cur = int(line[0]), line[1:].astype(np.int32)
        rec = np.zeros(stride, dtype=np.int32)
        for i in range(stride):
            a = rec[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ftype == 0:
                pred = 0
            elif ftype == 1:
                pred = a
            elif ftype == 2:
                pred = b
            elif ftype == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            rec[i] = (cur[i] + pred) & 0xFF
        out[y] = rec
        prev = rec
    return out.reshape(h, w, 4).astype(np.uint8)


def image_cost(path: Path) -> np.ndarray:
    rgba = decode_png_rgba8(path).astype(np.int32)
    grey = (rgba[..., 0] * 77 + rgba[..., 1] * 150 + rgba[..., 2] * 29) >> 8
    assert set(np.unique(grey).tolist()) <= {0, 255}, "expected a binary image"
    speed = np.where(grey == 255, np.float32(1.0), np.float32(0.0)).astype(np.float32)
    return fields.cost_from_speed(speed)


def cases(ref_data: Path):
    speed, seeds = fields.ring7(64, 4.0, 30.0, 2.0, 0.01, 4.0, seed=3)
    yield "ring7_64", fields.cost_from_speed(speed), seeds
    speed, seeds = fields.value_noise(40, seed=11, base_period=16.0, sources=3, w=48)
    yield "noise_48x40", fields.cost_from_speed(speed), seeds
    yield "constant_33x17", np.ones((17, 33), dtype=np.float32), np.array([[3, 5]], dtype=np.uint32)
    speed, seeds = fields.ring7(40, 3.0, 18.0, 2.0, 0.0, 3.0, seed=5)  # walls of speed 0: impassable
    yield "walls_inf_40", fields.cost_from_speed(speed), seeds
    speed, seeds = fields.value_noise(50, seed=23, base_period=8.0, sources=6, w=50)
    yield "multi_seed_50", fields.cost_from_speed(speed), seeds
    yield "single_row_1x29", np.full((1, 29), 2.0, dtype=np.float32), np.array([[4, 0]], dtype=np.uint32)
    yield "single_col_23x1", np.full((23, 1), 0.5, dtype=np.float32), np.array([[0, 22]], dtype=np.uint32)
    for name in ("7_ring_32_2d", "7_ring_256_2d"):
        p = ref_data / f"{name}.png"
        if p.exists():
            yield f"ref_{name}", image_cost(p), np.array([[0, 0]], dtype=np.uint32)


def main() -> None:
    ref_src = Path(sys.argv[1]) if len(sys.argv) > 1 else oracle.REF_SRC
    oracle.build(with_reference=True)
    ref = oracle.Reference()
    for name, cost, seeds in cases(ref_src.parent / "data"):
        fim5, _ = ref.fim(cost, seeds, 1e-5)
        fim3, _ = ref.fim(cost, seeds, 1e-3)
        fmm, _ = ref.fmm(cost, seeds)
        np.savez_compressed(HERE / f"{name}.npz", cost=cost, seeds=seeds, fim_1e5=fim5, fim_1e3=fim3, fmm=fmm)
        print(f"{name}: {cost.shape}, seeds {len(seeds)}, finite {np.isfinite(fim5).mean():.3f}")


if __name__ == "__main__":
    main()
