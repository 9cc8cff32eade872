"""The trial harness on the GPU: the reference's configuration sweep
(src/test_runner.cpp:226-291: tile kernel x compute-unit overload x block
size over the jobs, k_num_trials trials each, eps 1e-3) run through
ghcm_gb300.harness at a small size, checking its files and every result.

Bars: each .csv has the reference's two rows (device, total) with one
duration per trial; each .blob has the field's shape, the reference FIM's
reachability, is a fixed point of the update to within the harness eps, and
lies within 2e-2 (absolute) of the reference FIM run to the same eps.
"""
from __future__ import annotations

import numpy as np
import pytest

from ghcm_gb300 import fields, harness

pytestmark = pytest.mark.gpu

SIZE = 128
TRIALS = 2
BLOCKS = (8, 16)
OVERLOADS = (1, 8)
EPS = harness.K_FIM_MINIMUM_CHANGE
TOL = 2e-2  # as the golden harness-eps test: both solvers stop within eps per update


def _jobs():
    """The harness's jobs at SIZE (the same construction as harness.main)."""
    ring, seeds = fields.ring7_scaled(SIZE, 1)
    return seeds, {"7 rings": fields.cost_from_speed(ring),
                   "constant": np.ones((SIZE, SIZE), np.float32),
                   "noise": fields.cost_from_speed(fields.value_noise(SIZE, seed=1, base_period=SIZE / 8)[0])}


def test_harness_sweep_on_gpu(cuda_ok, oracle_lib, tmp_path):
    argv = ["--out", str(tmp_path), "--size", str(SIZE), "--trials", str(TRIALS),
            "--blocks", ",".join(map(str, BLOCKS)), "--overloads", ",".join(map(str, OVERLOADS))]
    assert harness.main(argv) == 0
    seeds, jobs = _jobs()
    ref = {name: oracle_lib.fim(cost, seeds, EPS)[0] for name, cost in jobs.items()}
    csvs = sorted(tmp_path.glob("*.csv"))
    assert len(csvs) == 2 * len(OVERLOADS) * len(BLOCKS) * len(jobs)  # both tile kernels
    for csv in csvs:
        rows = [r.split(",") for r in csv.read_text().splitlines()]
        assert [r[2].strip() for r in rows] == ["device", "total"]
        for r in rows:
            assert len(r) == 3 + TRIALS and all(int(v) >= 0 for v in r[3:])
        solver, job = rows[0][0], rows[0][1]
        assert csv.name == f"{solver}_{job}.csv"
        out = harness.read_blob(csv.with_suffix(".blob"))
        assert out.shape == (SIZE, SIZE)
        assert np.array_equal(np.isfinite(out), np.isfinite(ref[job])), (solver, job)
        assert oracle_lib.residual(jobs[job], out) <= EPS, (solver, job)
        diff = np.abs(out.astype(np.float64) - ref[job])
        diff[~np.isfinite(ref[job])] = 0
        assert float(diff.max()) <= TOL, (solver, job)
    # a second run finds every CSV written and skips it, as the reference does
    assert harness.main(argv) == 0
    assert sorted(tmp_path.glob("*.csv")) == csvs
