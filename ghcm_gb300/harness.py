"""Trial harness and on-disk formats, after the reference's test_runner.

* ``.blob``: ``size_t W, size_t H, float[W*H]`` little-endian, row-major
  (src/test_runner.cpp:199-206, read back at :338-347).
* ``.csv``: two rows per (solver, job), ``solver,job, device,t1,...`` and
  ``solver,job, total,t1,...`` with one duration in microseconds per trial
  (src/test_runner.cpp:209-219), ``k_num_trials = 5`` trials (:18).
* ``hcm_config_name`` names a configuration the way the reference's sweep does
  (src/test_runner.cpp:119-145) so result files line up with its layout.
* ``field_diff``: a - b with inf - inf = inf (src/test_runner.cpp:143-153).

``python -m ghcm_gb300.harness --out trials`` runs the reference's
configuration sweep (block 8/16/32 x compute-unit overload 1..32,
src/test_runner.cpp:232-234) of the GPU solver over synthetic jobs.
"""
from __future__ import annotations

import argparse
import struct
from pathlib import Path
from typing import Callable, Iterable

import numpy as np

K_NUM_TRIALS = 5
K_FIM_MINIMUM_CHANGE = 1e-3  # the harness's eps (src/test_runner.cpp:17)


def write_blob(path: str | Path, field: np.ndarray) -> None:
    f = np.ascontiguousarray(field, dtype=np.float32)
    h, w = f.shape
    with open(path, "wb") as fh:
        fh.write(struct.pack("<QQ", w, h))
        fh.write(f.astype("<f4").tobytes())


def read_blob(path: str | Path) -> np.ndarray:
    data = Path(path).read_bytes()
    w, h = struct.unpack_from("<QQ", data, 0)
    body = np.frombuffer(data, dtype="<f4", offset=16)
    if body.size != w * h:
        raise ValueError(f"{path}: expected {w * h} floats, found {body.size}")
    return body.reshape(h, w).astype(np.float32)


def field_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a = np.asarray(a, dtype=np.float32)
    b = np.asarray(b, dtype=np.float32)
    if a.shape != b.shape:
        raise ValueError("fields differ in size")
    both_inf = np.isinf(a) & np.isinf(b)
    with np.errstate(invalid="ignore"):
        d = np.where(a == b, np.float32(0), a - b).astype(np.float32)
    d[both_inf] = np.inf
    return d


def hcm_config_name(config) -> str:
    kernel = "fim" if int(config.kernel) == 1 else "systolic"
    cache = {0: "cache_none", 1: "cache_time", 2: "cache_cost", 3: "cache_both"}[int(config.cache_mode)]
    return (f"ghcm_{kernel}_{cache}_cu_over_{int(config.compute_unit_overload)}"
            f"_wg_over_{int(config.workers_overload)}_block_sz_{int(config.block_size)}")


def test_run(solver_name: str, jobs: Iterable[tuple[str, np.ndarray]], seeds,
             fn: Callable[[np.ndarray, np.ndarray], object], out_dir: str | Path,
             trials: int = K_NUM_TRIALS) -> list[Path]:
    """Runs ``fn(field, seeds)`` ``trials`` times per job (the reference's
    test_run, src/test_runner.cpp:169-223); writes <solver>_<job>.csv and the
    last result's .blob. ``fn`` returns an object with ``field``,
    ``duration_device`` and ``duration_total`` (microseconds). Existing
    non-empty CSVs are skipped, as the reference does."""
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    written = []
    for job_name, field in jobs:
        base = out / f"{solver_name}_{job_name}"
        csv = base.with_suffix(".csv")
        if csv.exists() and csv.stat().st_size > 0:
            continue
        dev, tot, result = [], [], None
        for _ in range(trials):
            result = fn(field, seeds)
            dev.append(int(round(result.duration_device)))
            tot.append(int(round(result.duration_total)))
        write_blob(base.with_suffix(".blob"), result.field)
        csv.write_text(f"{solver_name},{job_name}, device," + ",".join(map(str, dev)) + "\n"
                       + f"{solver_name},{job_name}, total," + ",".join(map(str, tot)) + "\n")
        written.append(csv)
    return written


def main(argv=None) -> int:
    from . import fields
    from .eikonal import HcmConfig, HcmSetup, Kernel, eikonal_hcm_cuda_ex

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default="trials")
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--trials", type=int, default=K_NUM_TRIALS)
    ap.add_argument("--blocks", default="8,16,32")
    ap.add_argument("--overloads", default="1,2,4,8,16,32")
    args = ap.parse_args(argv)
    n = args.size
    ring, ring_seeds = fields.ring7_scaled(n, 1)
    jobs = [("7 rings", fields.cost_from_speed(ring)),
            ("constant", np.ones((n, n), np.float32)),
            ("noise", fields.cost_from_speed(fields.value_noise(n, seed=1, base_period=n / 8)[0]))]
    seeds = ring_seeds  # one source at the centre for every job
    for kernel in (Kernel.Systolic, Kernel.FIM):
        for ov in (float(x) for x in args.overloads.split(",")):
            for b in (int(x) for x in args.blocks.split(",")):
                cfg = HcmConfig(block_size=b, compute_unit_overload=ov, kernel=kernel,
                                fim_minimum_change=K_FIM_MINIMUM_CHANGE)
                with HcmSetup(cfg) as setup:
                    test_run(hcm_config_name(cfg), jobs, seeds,
                             lambda f, s: eikonal_hcm_cuda_ex(setup, f, s), args.out, args.trials)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
