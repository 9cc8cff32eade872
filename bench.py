"""Benchmark of the gHCM block eikonal solve on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ghcm|reference]

Workload (one "step" = one solve to convergence): the 4096 x 4096 seven-ring
speed field (radii 256..1920, barrier width 16, speed 0.01, 64-cell gaps at
seeded angles, one centre source, h = 1), tiles of 16 x 16, device top-n
selection with n = 256 (the fastest of the configuration's n in {256, 1024,
4096}; the other two are timed and reported beside it), eps = 1e-5. Synthetic, seeded input: the reference's
ring images are replaced by the same construction drawn procedurally.

Metric: Mcell/s to convergence = W*H / (time from device-resident speed and
seeds to the device-resident converged time field). `value` is that, summed
over all ranks; `e2e` is the same metric through the public host-pointer call
(ghcm_solve: pinned host speed in, host time field out, copies inside the
timed region). Multi-GPU runs are independent replicas (the single-grid solve
does not shard), so scaling is weak.

--impl reference times the reference's CPU solver (the FMM of
src/eikonal_fmm.cpp as restated in oracle/, bit-exact to the reference build)
on the same workload, one solve per host thread.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mcell/s to convergence (plain device top-n schedule), 1 GB300, max rel err <=1e-5 vs reference FIM"
UNIT = "Mcell/s"
WORKLOAD = "ring7_4096x4096"
BLOCK = 16
N_JOBS = 256
N_SWEEP = (256, 1024, 4096)
EPS = 1e-5
L2_FLUSH_BYTES = 256 << 20  # > 129 MB of L2


def bytes_per_solve(b: int) -> int:
    # speed read + time tile with its edge halo read + time write, FP32
    return 4 * b * b + 4 * ((b + 2) * (b + 2) - 4) + 4 * b * b


def make_workload():
    from ghcm_gb300 import fields

    return fields.ring7_large(seed=1)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(speed, seeds, threads: int = 1) -> dict:
    """The reference's CPU FMM and FIM (oracle restatement, bit-exact to the
    reference build) on the full workload, one core each."""
    from ghcm_gb300 import fields
    from oracle.oracle import Oracle, build

    build(with_reference=False)
    o = Oracle()
    cost = fields.cost_from_speed(speed)
    cells = speed.size
    fmm, us_fmm = o.fmm(cost, seeds)
    fim, us_fim = o.fim(cost, seeds, EPS)
    return fim, fmm, {"value": cells / us_fmm, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"one full {speed.shape[1]}x{speed.shape[0]} solve each by the FMM (value) and FIM of the "
                      "reference, 1 host thread",
            "fmm_ms": us_fmm / 1e3, "fim_ms": us_fim / 1e3, "fim_mcells": cells / us_fim,
            "cpu": _cpu_name(), "nproc": os.cpu_count()}


def _cpu_name() -> str:
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return os.uname().machine


def load_traffic():
    p = ROOT / "profiles" / "k_solve_ring7_4096.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("dram_bytes_per_launch")
        except (ValueError, OSError):
            return None
    return None


def run_reference(args, world, rank) -> int:
    if rank != 0:
        return 0
    from ghcm_gb300 import fields
    from oracle.oracle import Oracle, build

    build(with_reference=False)
    o = Oracle()
    speed, seeds = make_workload()
    cost = fields.cost_from_speed(speed)
    threads = max(1, min(os.cpu_count() or 1, args.steps))
    # warm-up: one solve per thread that will run (page in, warm caches)
    o.throughput("fmm", cost, seeds, count=min(args.warmup, threads) or 1, threads=threads)
    _, us = o.throughput("fmm", cost, seeds, count=args.steps, threads=threads)
    value = speed.size * args.steps / us
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": us / 1e3 / args.steps * threads, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "solver": "reference FMM (src/eikonal_fmm.cpp), CPU",
                   "threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full solves of the workload, one per host thread"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ghcm", choices=["ghcm", "reference"])
    ap.add_argument("--block", type=int, default=BLOCK)
    ap.add_argument("--n", type=int, default=N_JOBS)
    ap.add_argument("--kernel", default="systolic", choices=["systolic", "fim"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-n-sweep", action="store_true", help="time only the headline n")
    args = ap.parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch

    import ghcm_gb300 as g

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    speed, seeds = make_workload()
    h, w = speed.shape
    cells = h * w
    cfg = g.HcmConfig(block_size=args.block, max_jobs=args.n, fim_minimum_change=EPS,
                      kernel=g.Kernel.FIM if args.kernel == "fim" else g.Kernel.Systolic)
    setup = g.HcmSetup(cfg)
    d_speed = torch.from_numpy(speed).to(dev)
    d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    d_time = torch.empty_like(d_speed)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    for _ in range(args.warmup):
        g.solve_device(setup, d_speed, d_seeds, d_time, stream=stream)
    barrier()

    step_ms, kernel_ms, stats = [], [], []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with Clocks(local) as clk:
        barrier()
        t_wall = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))  # evict the field from L2 between steps (outside the events)
            ev[i][0].record(stream)
            st = g.solve_device(setup, d_speed, d_seeds, d_time, stream=stream)
            ev[i][1].record(stream)
            stats.append(st)
        barrier()
        t_wall = time.perf_counter() - t_wall
    clocks = clk.summary()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    kernel_ms = [st["kernel_ms"] for st in stats]
    ms = sum(step_ms) / len(step_ms)
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * cells / (ms * 1e3)

    # the configuration's other n values, timed the same way (device-resident)
    n_sweep = {}
    if not args.no_n_sweep:
        for n in N_SWEEP:
            if n == args.n:
                n_sweep[str(n)] = {"mcells": cells / (ms * 1e3), "ms": ms,
                                   "block_solves": statistics.mean(st["block_solves"] for st in stats),
                                   "waves": statistics.mean(st["waves"] for st in stats)}
                continue
            other = g.HcmSetup(g.HcmConfig(block_size=args.block, max_jobs=n, fim_minimum_change=EPS,
                                           kernel=cfg.kernel))
            for _ in range(args.warmup):
                g.solve_device(other, d_speed, d_seeds, d_time, stream=stream)
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(args.steps)]
            sts = []
            for i in range(args.steps):
                flush.fill_(float(i))
                evs[i][0].record(stream)
                sts.append(g.solve_device(other, d_speed, d_seeds, d_time, stream=stream))
                evs[i][1].record(stream)
            torch.cuda.synchronize(dev)
            n_ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
            n_sweep[str(n)] = {"mcells": cells / (n_ms * 1e3), "ms": n_ms,
                               "block_solves": statistics.mean(x["block_solves"] for x in sts),
                               "waves": statistics.mean(x["waves"] for x in sts)}
            other.close()
        g.solve_device(setup, d_speed, d_seeds, d_time, stream=stream)  # leave the headline field in d_time

    # end to end through the host-pointer call: pinned speed in, time field out
    h_speed = torch.from_numpy(speed).pin_memory()
    h_time = torch.empty((h, w), dtype=torch.float32).pin_memory()
    e2e_ms = []
    for i in range(max(1, min(args.steps, 5))):
        t0 = time.perf_counter()
        g.eikonal_hcm_cuda_ex(setup, h_speed.numpy(), seeds, input_is_speed=True, out=h_time.numpy())
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_mean = sum(e2e_ms) / len(e2e_ms)

    from oracle.oracle import Oracle, rel_diff  # checker: parity of the benchmarked field

    bps = bytes_per_solve(args.block)
    solves = statistics.mean(st["block_solves"] for st in stats)
    k_ms = statistics.mean(kernel_ms)
    achieved = solves * bps / (k_ms * 1e-3) / 1e9
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "block": args.block, "n": args.n, "kernel": args.kernel, "eps": EPS,
                   "sources": int(len(seeds)), "l2": "flushed between steps (256 MiB write outside the events)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * cells / (e2e_mean * 1e3), "unit": UNIT, "ms_per_step": e2e_mean,
                "h2d_bytes_per_step": cells * 4 + int(seeds.nbytes), "d2h_bytes_per_step": cells * 4},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": load_traffic(), "kernel": f"k_solve<{args.block},{args.kernel}>",
                     "bytes_per_block_solve": bps, "block_solves": solves, "kernel_ms": k_ms,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in peaks else "fallback"},
        "n_sweep": n_sweep,
        "gpu_launches": 5 * args.steps,
        "clocks": clocks,
        "solver": {"waves": statistics.mean(st["waves"] for st in stats),
                   "residual_passes": statistics.mean(st["residual_passes"] for st in stats),
                   "max_active": max(st["max_active"] for st in stats),
                   "wall_s_timed": t_wall},
    }
    if rank == 0:
        from ghcm_gb300 import fields

        field = d_time.cpu().numpy()
        cost = fields.cost_from_speed(speed)
        line["check"] = {"residual": Oracle().residual(cost, field),
                         "seeds_zero": bool(np.all(field[seeds[:, 1], seeds[:, 0]] == 0)),
                         "finite": bool(np.isfinite(field).all())}
        if not args.no_cpu_baseline:
            fim, fmm, base = cpu_baseline(speed, seeds)
            line["cpu_baseline"] = base
            line["check"]["max_rel_vs_fim"] = rel_diff(field, fim)
            line["check"]["max_rel_vs_fmm"] = rel_diff(field, fmm)
            line["check"]["fim_vs_fmm"] = rel_diff(fim, fmm)
        print(json.dumps(line), flush=True)
    setup.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
