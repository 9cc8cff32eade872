"""Trial-harness formats (the reference's test_runner): .blob, .csv, names."""
from __future__ import annotations

import struct
from types import SimpleNamespace

import numpy as np
import pytest

import ghcm_gb300 as g
from ghcm_gb300 import harness


def test_blob_round_trip_and_layout(tmp_path):
    f = np.arange(12, dtype=np.float32).reshape(3, 4)
    f[1, 2] = np.inf
    p = tmp_path / "x.blob"
    harness.write_blob(p, f)
    raw = p.read_bytes()
    assert struct.unpack_from("<QQ", raw) == (4, 3)  # size_t W, size_t H
    assert len(raw) == 16 + 12 * 4
    np.testing.assert_array_equal(harness.read_blob(p), f)


def test_blob_rejects_truncated(tmp_path):
    p = tmp_path / "bad.blob"
    p.write_bytes(struct.pack("<QQ", 5, 5) + b"\0" * 8)
    with pytest.raises(ValueError):
        harness.read_blob(p)


def test_field_diff_infinity_rules():
    a = np.array([1.0, np.inf, np.inf, 2.0], np.float32)
    b = np.array([0.5, np.inf, 1.0, 2.0], np.float32)
    d = harness.field_diff(a, b)
    assert d[0] == 0.5 and np.isinf(d[1]) and np.isinf(d[2]) and d[3] == 0.0


def test_config_name_matches_reference_scheme():
    cfg = g.HcmConfig(block_size=16, compute_unit_overload=8, kernel=g.Kernel.FIM)
    assert harness.hcm_config_name(cfg) == "ghcm_fim_cache_both_cu_over_8_wg_over_1_block_sz_16"


def test_test_run_writes_csv_and_blob(tmp_path):
    calls = []

    def fake_solver(field, seeds):
        calls.append(1)
        return SimpleNamespace(field=field * 2, duration_device=10.4, duration_total=20.6)

    jobs = [("a", np.ones((2, 3), np.float32))]
    written = harness.test_run("solver", jobs, [[0, 0]], fake_solver, tmp_path, trials=3)
    assert written == [tmp_path / "solver_a.csv"] and len(calls) == 3
    rows = (tmp_path / "solver_a.csv").read_text().splitlines()
    assert rows == ["solver,a, device,10,10,10", "solver,a, total,21,21,21"]
    np.testing.assert_array_equal(harness.read_blob(tmp_path / "solver_a.blob"), np.full((2, 3), 2, np.float32))
    # an existing non-empty csv is skipped, as the reference does
    assert harness.test_run("solver", jobs, [[0, 0]], fake_solver, tmp_path, trials=3) == []
