"""Host-side helpers of bench.py (no GPU): the DRAM traffic it reads from the
committed profiler summaries, the algorithmic bytes per block-solve, and the
reference-schedule figures it reports from the oracle."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import bench
from conftest import load_golden

PROFILES = Path(bench.__file__).resolve().parent / "profiles"


def test_bytes_per_solve_matches_the_formula():
    # 4 B^2 speed + 4 ((B+2)^2 - 4) time tile and edge halo + 4 B^2 time write
    assert [bench.bytes_per_solve(b) for b in (8, 16, 32)] == [896, 3328, 12800]


def test_ring_traffic_comes_from_the_committed_capture():
    d = json.loads((PROFILES / "k_solve_ring7_4096.json").read_text())
    t = bench.load_traffic()
    assert t == d["dram_bytes_per_launch"] > 0
    if d.get("dram_bytes_read") is not None:
        assert t == pytest.approx(d["dram_bytes_read"] + d["dram_bytes_write"], rel=1e-9)
    # a capture of another tile size or n is not used
    assert bench.load_traffic("k_solve_ring7_4096.json", block=32) is None
    assert bench.load_traffic("k_solve_ring7_4096.json", block=16, n=1024) is None
    assert bench.load_traffic("no_such_capture.json") is None


def test_batch_traffic_scales_bytes_per_block_solve():
    d = json.loads((PROFILES / "k_solve_batch512.json").read_text())
    assert d["dram_bytes_per_launch"] == pytest.approx(d["dram_bytes_read"] + d["dram_bytes_write"], rel=1e-6)
    per = d["dram_bytes_per_launch"] / d["block_solves"]
    assert bench.batch_traffic(d["block"], d["block_solves"]) == pytest.approx(d["dram_bytes_per_launch"])
    assert bench.batch_traffic(d["block"], 2 * d["block_solves"]) == pytest.approx(2 * per * d["block_solves"])
    # bytes per solve are at least the algorithmic bytes (the staged box is wider than the tile)
    assert per >= bench.bytes_per_solve(d["block"])
    assert bench.batch_traffic(8, 1000) is None


def test_reference_schedule_reports_counts_and_accuracy(oracle_lib):
    g = load_golden("constant_33x17")
    fim = g["fim_1e5"]
    r = bench.reference_schedule(oracle_lib, g["cost"], g["seeds"], 8, 4, 64, fim)
    assert r["block_solves"] >= 15 and r["waves"] >= 4  # 5 x 3 tiles, each solved at least once
    # nothing can be lost on a constant field: the reference schedule reaches the fixed point
    assert r["max_rel_vs_fim"] < 1e-5 and r["residual"] <= 1e-5
    assert {"block", "n", "work_group", "note"} <= set(r)


def test_fmm64_errors_conventions():
    ref = np.array([[0.0, 1.0], [2.0, np.inf]])
    got = np.array([[0.0, 1.5], [2.0, np.inf]], dtype=np.float32)
    e = bench.fmm64_errors(got, ref)
    assert e["linf"] == pytest.approx(0.5) and e["reachability_matches"]
    assert e["l1"] == pytest.approx(0.5 / 3)  # mean over the finite cells


def test_headline_traffic_comes_from_the_committed_capture():
    d = json.loads((PROFILES / "k_solve_noise4096_learned.json").read_text())
    t = bench.load_traffic("k_solve_noise4096_learned.json")
    assert t == pytest.approx(d["dram_bytes_read"] + d["dram_bytes_write"]) and t > 0
    assert d["block_solves"] > 0


def test_maze_traffic_scales_by_block_solves():
    d = json.loads((PROFILES / "k_solve_maze16384.json").read_text())
    assert bench.load_traffic("k_solve_maze16384.json", block=32, n=9728) == pytest.approx(d["dram_bytes_per_launch"])
    assert bench.load_traffic("k_solve_maze16384.json", block=16) is None
    assert bench.load_block_solves("k_solve_maze16384.json") == d["block_solves"] > 0
    assert bench.load_block_solves("no_such_capture.json") is None
    # bytes per block-solve at least the algorithmic 12,800 B of a 32 x 32 tile
    assert d["dram_bytes_per_launch"] / d["block_solves"] >= bench.bytes_per_solve(32)
