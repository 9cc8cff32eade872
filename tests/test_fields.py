"""Synthetic workload generators: deterministic, in range, seeds valid."""
from __future__ import annotations

import numpy as np

from ghcm_gb300 import fields


def _check_seeds(seeds, w, h):
    assert seeds.dtype == np.uint32 and seeds.shape[1] == 2
    assert np.all(seeds[:, 0] < w) and np.all(seeds[:, 1] < h)
    pts = {tuple(p) for p in seeds.tolist()}
    assert len(pts) == len(seeds)
    for x, y in pts:
        assert not ({(x + 1, y), (x - 1, y), (x, y + 1), (x, y - 1)} & pts)


def test_ring7_small_shape_and_values():
    speed, seeds = fields.ring7_small(1)
    assert speed.shape == (256, 256) and speed.dtype == np.float32
    assert set(np.unique(speed).tolist()) == {np.float32(0.01), np.float32(1.0)}
    assert seeds.tolist() == [[128, 128]]
    a, _ = fields.ring7_small(1)
    b, _ = fields.ring7_small(2)
    assert np.array_equal(a, speed) and not np.array_equal(a, b)


def test_ring7_has_seven_gapped_rings():
    speed, _ = fields.ring7(512, 32.0, 240.0, 8.0, 0.01, 16.0, seed=4)
    row = speed[256, 256:]
    # walk outward along +x: count wall segments (a gap on this ray removes one)
    walls = np.flatnonzero(np.diff((row < 1).astype(np.int8)) == 1)
    assert 5 <= len(walls) <= 7
    # every ring has a gap: the wall fraction on each annulus is below 1
    yy, xx = np.mgrid[0:512, 0:512] - 256
    r = np.hypot(xx, yy)
    for i in range(7):
        r0 = 32.0 + i * (240.0 - 32.0) / 6
        ring = (r >= r0 + 1) & (r < r0 + 7)
        frac = np.mean(speed[ring] < 1)
        assert 0.9 < frac < 1.0


def test_value_noise_range_and_determinism():
    s1, d1 = fields.value_noise(128, seed=5, base_period=64.0, sources=16)
    s2, d2 = fields.value_noise(128, seed=5, base_period=64.0, sources=16)
    assert np.array_equal(s1, s2) and np.array_equal(d1, d2)
    assert s1.min() >= np.float32(0.02) and s1.max() <= np.float32(1.0)
    assert s1.std() > 0.05
    _check_seeds(d1, 128, 128)


def test_ca_maze_walls_and_sources():
    speed, seeds = fields.ca_maze(256, seed=9, sources=64)
    assert set(np.unique(speed).tolist()) == {np.float32(0.001), np.float32(1.0)}
    assert 0.2 < np.mean(speed < 1) < 0.8
    _check_seeds(seeds, 256, 256)
    assert np.all(speed[seeds[:, 1], seeds[:, 0]] == 1.0)


def test_batched_mix_sizes():
    inst = fields.batched_mix(24, seed=3)
    assert len(inst) == 24
    for it in inst:
        h, w = it.speed.shape
        assert h == w and 64 <= h <= 1024 and h % 16 == 0
        assert 1 <= len(it.seeds) <= 8
        _check_seeds(it.seeds, w, h)
    assert {it.kind for it in inst} == {"ring7", "noise"}


def test_cost_from_speed():
    c = fields.cost_from_speed(np.array([[0.0, 0.5, 1.0]], dtype=np.float32), h=2.0)
    assert np.isinf(c[0, 0]) and c[0, 1] == 4.0 and c[0, 2] == 2.0
