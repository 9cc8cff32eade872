"""Seeded synthetic speed fields and seed cells for the eikonal workloads.

The reference benchmarks on images it loads from disk (src/test_runner.cpp:310-322);
two of them are not shipped (.MISSING_LARGE_BLOBS). The workloads here are
seeded synthetic fields with the shapes, sizes and value ranges of the
benchmark configurations this package is measured on:

* ``ring7``  - concentric annular barriers with one gap each (the reference's
  ``data/7_ring_*_2d.png`` family, drawn procedurally);
* ``value_noise`` - fractal value noise mapped to speed = clamp(exp(2 n), lo, hi);
* ``ca_maze`` - cellular-automaton walls after majority smoothing;
* ``batched_mix`` - many instances of uneven sizes mixing the first two.

Every field is row-major float32 with x fastest (``field[y, x]``), the layout
of the reference's ``Field2D`` (src/util_field.h, src/util_dim.h:17-21).
Seeds are ``uint32`` arrays of shape (n, 2) holding (x, y).

All randomness comes from ``numpy.random.default_rng`` (PCG64), which gives
the same stream on every platform.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def _seeds_array(points) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(points, dtype=np.uint32).reshape(-1, 2))


def ring7(n: int, r_first: float, r_last: float, width: float, wall_speed: float, gap: float,
          seed: int, rings: int = 7, background: float = 1.0):
    """Square ``n`` x ``n`` field with ``rings`` concentric annular barriers.

    Ring ``i`` covers radii ``[R_i, R_i + width)`` around the grid centre, with
    ``R_i`` evenly spaced from ``r_first`` to ``r_last``. Each ring has one gap
    of arc length ``gap`` cells (measured at the ring's mid radius) centred on
    an angle drawn uniformly from ``[0, 2 pi)``. Barrier cells get
    ``wall_speed``; the rest ``background``. The single source is the centre
    cell ``(n // 2, n // 2)``.
    """
    rng = np.random.default_rng(seed)
    angles = rng.uniform(0.0, 2.0 * math.pi, size=rings)
    c = n // 2
    coords = np.arange(n, dtype=np.float64) - c
    dy, dx = np.meshgrid(coords, coords, indexing="ij")
    r = np.hypot(dx, dy)
    theta = np.arctan2(dy, dx)
    speed = np.full((n, n), background, dtype=np.float32)
    step = (r_last - r_first) / max(rings - 1, 1)
    for i in range(rings):
        r_in = r_first + i * step
        wall = (r >= r_in) & (r < r_in + width)
        d = np.abs(np.angle(np.exp(1j * (theta - angles[i]))))
        in_gap = d * (r_in + width / 2.0) < gap / 2.0
        speed[wall & ~in_gap] = wall_speed
    return speed, _seeds_array([(c, c)])


def ring7_small(seed: int = 1):
    """256 x 256 seven-ring field: radii 16..120, width 4, speed 0.01, 8-cell gaps."""
    return ring7(256, 16.0, 120.0, 4.0, 0.01, 8.0, seed)


def ring7_large(seed: int = 1):
    """4096 x 4096 seven-ring field: radii 256..1920, width 16, speed 0.01, 64-cell gaps."""
    return ring7(4096, 256.0, 1920.0, 16.0, 0.01, 64.0, seed)


def ring7_scaled(n: int, seed: int):
    """The 4096-cell construction scaled to side ``n`` (radii n/16..15n/32)."""
    return ring7(n, n / 16.0, n * 15.0 / 32.0, max(1.0, n / 256.0), 0.01, max(2.0, n / 64.0), seed)


def _random_cells(rng, w: int, h: int, count: int, allowed=None) -> np.ndarray:
    """``count`` distinct cells, no two 4-adjacent, optionally restricted to ``allowed``."""
    pts: list[tuple[int, int]] = []
    taken: set[tuple[int, int]] = set()
    tries = 0
    while len(pts) < count:
        tries += 1
        if tries > 1000 * count + 1000:
            raise ValueError("could not place seed cells")
        x = int(rng.integers(0, w))
        y = int(rng.integers(0, h))
        if allowed is not None and not allowed[y, x]:
            continue
        if any((x + ox, y + oy) in taken for ox, oy in ((0, 0), (1, 0), (-1, 0), (0, 1), (0, -1))):
            continue
        taken.add((x, y))
        pts.append((x, y))
    return _seeds_array(pts)


def value_noise(n: int, seed: int, octaves: int = 6, base_period: float = 512.0, persistence: float = 0.5,
                lo: float = 0.02, hi: float = 1.0, sources: int = 16, w: int | None = None):
    """Fractal value noise speed field, ``speed = clip(exp(2 * noise), lo, hi)``.

    Octave ``k`` has lattice period ``base_period / 2**k`` and amplitude
    ``persistence**k``; lattice values are uniform in [-1, 1] from a stream
    seeded by ``(seed, k)``; cells interpolate the lattice bilinearly with
    smoothstep weights ``f*f*(3-2f)``. ``sources`` seed cells are uniform over
    the grid (no two adjacent).
    """
    h = n
    w = n if w is None else w
    acc = np.zeros((h, w), dtype=np.float64)
    for k in range(octaves):
        period = base_period / (2 ** k)
        lx = int(math.ceil(w / period)) + 2
        ly = int(math.ceil(h / period)) + 2
        lat = np.random.default_rng([seed, k]).uniform(-1.0, 1.0, size=(ly, lx))

        def weights(m):
            u = np.arange(m, dtype=np.float64) / period
            i0 = np.floor(u).astype(np.int64)
            f = u - i0
            return i0, f * f * (3.0 - 2.0 * f)

        ix, sx = weights(w)
        iy, sy = weights(h)
        rows = lat[:, ix] * (1.0 - sx) + lat[:, ix + 1] * sx          # (ly, w)
        val = rows[iy, :] * (1.0 - sy)[:, None] + rows[iy + 1, :] * sy[:, None]
        acc += (persistence ** k) * val
    speed = np.clip(np.exp(2.0 * acc), lo, hi).astype(np.float32)
    rng = np.random.default_rng([seed, 1000])
    return speed, _random_cells(rng, w, h, sources)


def ca_maze(n: int, seed: int, fill: float = 0.45, passes: int = 5, wall_speed: float = 0.001,
            open_speed: float = 1.0, sources: int = 64):
    """Cellular-automaton maze: random walls (probability ``fill``), then
    ``passes`` rounds of 3x3 majority smoothing (a cell becomes wall when at
    least 5 of the 9 cells of its neighbourhood are walls; outside counts as
    open). Walls get ``wall_speed``, open cells ``open_speed``; ``sources``
    seeds are placed in open cells."""
    rng = np.random.default_rng(seed)
    wall = (rng.random((n, n), dtype=np.float32) < fill).astype(np.uint8)
    for _ in range(passes):
        p = np.pad(wall, 1)
        cnt = np.zeros((n, n), dtype=np.uint8)
        for oy in range(3):
            for ox in range(3):
                cnt += p[oy:oy + n, ox:ox + n]
        wall = (cnt >= 5).astype(np.uint8)
    speed = np.where(wall == 1, np.float32(wall_speed), np.float32(open_speed)).astype(np.float32)
    return speed, _random_cells(np.random.default_rng([seed, 1000]), n, n, sources, allowed=(wall == 0))


@dataclass
class Instance:
    speed: np.ndarray
    seeds: np.ndarray
    kind: str


def batched_mix(count: int, seed: int, side_min: int = 64, side_max: int = 1024):
    """``count`` instances with side log-uniform in [side_min, side_max], rounded
    to a multiple of 16; each is a scaled seven-ring or a value-noise field with
    probability 1/2, with 1-8 random sources."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        side = int(round(math.exp(rng.uniform(math.log(side_min), math.log(side_max))) / 16.0)) * 16
        side = min(max(side, side_min), side_max)
        k = int(rng.integers(1, 9))
        if rng.random() < 0.5:
            speed, _ = ring7_scaled(side, seed=int(rng.integers(0, 2 ** 31)))
            kind = "ring7"
        else:
            speed, _ = value_noise(side, seed=int(rng.integers(0, 2 ** 31)), base_period=side / 8.0, sources=1)
            kind = "noise"
        seeds = _random_cells(np.random.default_rng([seed, i]), side, side, k, allowed=speed > 0.05)
        out.append(Instance(speed, seeds, kind))
    return out


def cost_from_speed(speed: np.ndarray, h: float = 1.0) -> np.ndarray:
    """cost = h / speed in float32, +inf where speed is 0 (src/test_runner.cpp:38-42)."""
    with np.errstate(divide="ignore"):
        return (np.float32(h) / speed.astype(np.float32)).astype(np.float32)
