"""Benchmark of the gHCM block eikonal solve on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ghcm|reference]
                    [--workload noise|ring|batched|maze]

Default workload (one "step" = one solve to convergence): the 4096 x 4096
fractal value-noise speed field (6 octaves, base period 512, persistence 0.5,
speed = clamp(exp(2 noise), 0.02, 1)) with 16 sources, seed 1, h = 1, tiles of
16, eps = 1e-5, solved by the LEARNED block schedule (the 12-64-64-1 MLP of
ghcm_gb300/models/, trained on traces of the plain solver on 32 other seeds;
score policy, at most 4096 jobs a wave, filled to 4 x SMs in key order).
`value` is its Mcell/s; the PLAIN device schedule is timed the same way in
the same run at n = 4 x SMs, 1024, 2048 and 4096, and the fastest is reported
beside it (`plain`, `learned_vs_plain`), the others and the veto policy under
`others`. Both fields are checked
against the reference's CPU FIM and FMM (oracle restatements, bit-exact to the
reference build) and an FP64 FMM. Sub-objects: `ring_4096` - the 4096 x 4096
seven-ring field (radii 256..1920, barrier width 16, speed 0.01, 64-cell gaps,
one centre source) with the plain schedule at n = 256, 1024, 4096 - and
`small_ring_256` (the 256 x 256 ring, B = 8, n = 64). Synthetic, seeded input.

--workload ring: the seven-ring field as the headline (plain schedule, --n).
--workload batched: 512 independent instances (side log-uniform in
[64, 1024], multiples of 16, seven-ring or noise, 1-8 sources) in one
persistent launch replayed from a CUDA graph, tile size / n / sweep cap from
the autotuner; with N ranks the instances are split by cells (weak scaling).
--workload maze: the 16384 x 16384 cellular-automaton maze, 64 sources.

Metric: Mcell/s to convergence = cells / (time from device-resident speed and
seeds to the device-resident converged time field). `value` is that, summed
over all ranks; `e2e` is the same metric through the public host-pointer call
with the host<->device copies of inputs and results inside the timed region.

--impl reference times the reference's CPU solver (the FMM of
src/eikonal_fmm.cpp as restated in oracle/, bit-exact to the reference build)
on the same workload, one full solve per host thread per step.
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


METRIC = "Mcell/s to convergence, learned vs plain schedule, 1 GB300, max rel err \u22641e-5"
UNIT = "Mcell/s"
WORKLOAD = "noise_4096x4096_16src"
RING_WORKLOAD = "ring7_4096x4096"
BATCH_WORKLOAD = "batched_512_ring7_or_noise_64_to_1024"
MAZE_WORKLOAD = "ca_maze_16384x16384_64src"
MAZE_SEED = 5
MAZE_CROP = 2048
BATCH_COUNT = 512
BATCH_SEED = 1234
NOISE_EVAL_SEED = 1
MODEL = ROOT / "ghcm_gb300" / "models" / "schedule_noise4096_b16.npz"
LAUNCHES_PER_SOLVE = 3  # k_init_inst, k_init_seeds, the persistent k_solve
LAUNCHES_PER_LEARNED_SOLVE = 4  # the same and k_tile_stats (the learned features' per-tile speed statistics)
BLOCK = 16
N_JOBS = 256  # the seven-ring workload's headline n
N_SWEEP = (256, 1024, 4096)
LEARNED_CAP = 4096  # the learned schedule's most jobs a wave; waves are filled to 4 x SMs in key order
PLAIN_SWEEP = (0, 1024, 2048, 4096)  # plain n timed beside it (0: 4 x SMs, one job per CTA of the 4-CTA grid);
                                     # the fastest is the comparison
EPS = 1e-5
L2_FLUSH_BYTES = 256 << 20  # > 129 MB of L2


def bytes_per_solve(b: int) -> int:
    # speed read + time tile with its edge halo read + time write, FP32
    return 4 * b * b + 4 * ((b + 2) * (b + 2) - 4) + 4 * b * b


def make_workload(kind: str = "noise"):
    """The headline field: 4096^2 fractal value noise (6 octaves, base period
    512, persistence 0.5, speed = clamp(exp(2 noise), 0.02, 1)), 16 sources,
    seed NOISE_EVAL_SEED (not among the schedule model's training seeds); or
    the 4096^2 seven-ring field."""
    from ghcm_gb300 import fields

    if kind == "ring":
        return fields.ring7_large(seed=1)
    return fields.value_noise(4096, seed=NOISE_EVAL_SEED, base_period=512.0, sources=16)


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
            # let the sampler finish starting up (NVML initialisation) before the
            # timed region: a step overlapping it once measured 150 ms longer
            time.sleep(0.5)
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


def load_traffic(name: str = "k_solve_ring7_4096.json", block: int | None = None, n: int | None = None):
    """DRAM bytes per launch from a committed ncu summary (profiles/), or None;
    with block / n given, only when the capture used that tile size and n."""
    p = ROOT / "profiles" / name
    if p.exists():
        try:
            d = json.loads(p.read_text())
        except (ValueError, OSError):
            return None
        if block is not None and d.get("block") not in (None, block):
            return None
        if n is not None and d.get("n") not in (None, n):
            return None
        return d.get("dram_bytes_per_launch")
    return None


def load_block_solves(name: str):
    """Block-solves of the launch a committed capture summary covers, or None."""
    try:
        return json.loads((ROOT / "profiles" / name).read_text()).get("block_solves")
    except (ValueError, OSError):
        return None


def batch_traffic(block: int, block_solves: float):
    """DRAM bytes of one batch launch: the captured bytes per block-solve
    (profiles/k_solve_batch512.json, same tile size) scaled to this run's
    block-solves - the staging reads scale with them; the residual passes,
    ~20% of the captured bytes, scale with the waves instead."""
    p = ROOT / "profiles" / "k_solve_batch512.json"
    try:
        d = json.loads(p.read_text())
    except (ValueError, OSError):
        return None
    if d.get("block") != block or not d.get("block_solves"):
        return None
    return d["dram_bytes_per_launch"] / d["block_solves"] * block_solves


def batch_instances():
    from ghcm_gb300 import fields

    return fields.batched_mix(BATCH_COUNT, seed=BATCH_SEED)


def cpu_fmm_pool(o, insts, threads: int) -> float:
    """Solves every instance once with the reference FMM over `threads` host
    threads; returns wall microseconds."""
    from concurrent.futures import ThreadPoolExecutor

    from ghcm_gb300 import fields

    costs = [(fields.cost_from_speed(i.speed), i.seeds) for i in insts]
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda cs: o.fmm(cs[0], cs[1]), costs))
    return (time.perf_counter() - t0) * 1e6


def run_reference(args, world, rank) -> int:
    if rank != 0:
        return 0
    from ghcm_gb300 import fields
    from oracle.oracle import Oracle, build

    build(with_reference=False)
    o = Oracle()
    if args.workload == "batched":
        insts = batch_instances()[::8]  # a fixed 1-in-8 sample of the batch per step
        cells = sum(i.speed.size for i in insts)
        threads = max(1, os.cpu_count() or 1)
        for _ in range(args.warmup):
            cpu_fmm_pool(o, insts[: threads], threads)
        us = sum(cpu_fmm_pool(o, insts, threads) for _ in range(args.steps))
        value = cells * args.steps / us
        line = {
            "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": us / 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": BATCH_WORKLOAD, "solver": "reference FMM (src/eikonal_fmm.cpp), CPU",
                       "threads": threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"every 8th instance of the batch ({len(insts)} instances, {cells} cells) "
                                       "per step, one instance per host thread at a time"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return 0
    speed, seeds = make_workload(args.workload)
    cost = fields.cost_from_speed(speed)
    # a step: one full solve of the workload on every host thread at once
    threads = max(1, os.cpu_count() or 1)
    if args.warmup:  # one untimed round (page in, warm caches)
        o.throughput("fmm", cost, seeds, count=threads, threads=threads)
    _, us = o.throughput("fmm", cost, seeds, count=args.steps * threads, threads=threads)
    value = speed.size * args.steps * threads / us
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": us / 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": RING_WORKLOAD if args.workload == "ring" else WORKLOAD,
                   "solver": "reference FMM (src/eikonal_fmm.cpp), CPU", "threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} step(s) of {threads} concurrent full solves of the workload, "
                                   "one per host thread"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def fmm64_errors(field: np.ndarray, ref64: np.ndarray) -> dict:
    """L-inf and L1 (mean) absolute error of `field` against the FP64 FMM over
    cells finite in both, with the largest relative error."""
    f = field.astype(np.float64)
    m = np.isfinite(f) & np.isfinite(ref64)
    d = np.abs(f[m] - ref64[m])
    pos = m & (ref64 > 0)
    rel = np.abs(f[pos] - ref64[pos]) / ref64[pos]
    return {"linf": float(d.max()) if d.size else 0.0, "l1": float(d.mean()) if d.size else 0.0,
            "max_rel": float(rel.max()) if rel.size else 0.0,
            "reachability_matches": bool(np.array_equal(np.isfinite(f), np.isfinite(ref64)))}


def timed_device_solves(g, setup, d_speed, d_seeds, d_time, stream, flush, steps: int, warmup: int):
    """`steps` device-resident solves timed with CUDA events on `stream`, the
    L2 flushed before each (outside the events). Returns (mean ms, stats)."""
    import torch

    for _ in range(warmup):
        g.solve_device(setup, d_speed, d_seeds, d_time, stream=stream)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    sts = []
    for i in range(steps):
        flush.fill_(float(i))
        evs[i][0].record(stream)
        sts.append(g.solve_device(setup, d_speed, d_seeds, d_time, stream=stream))
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / steps, sts


def small_ring_check(g) -> dict:
    """The configuration the reference runs on the CPU: the 256 x 256 seven-ring
    field (radii 16..120, width 4, speed 0.01, 8-cell gaps, centre source),
    solved by gHCM with tiles of 8 and n = 64, against the reference FIM and
    FMM and the FP64 FMM."""
    from ghcm_gb300 import fields
    from oracle.oracle import Oracle, build, rel_diff

    build(with_reference=False)
    o = Oracle()
    speed, seeds = fields.ring7_small(seed=1)
    cost = fields.cost_from_speed(speed)
    with g.HcmSetup(g.HcmConfig(block_size=8, max_jobs=64, fim_minimum_change=EPS)) as s:
        res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
    fim, us_fim = o.fim(cost, seeds, EPS)
    fmm, us_fmm = o.fmm(cost, seeds)
    ref64, _ = o.fmm64(cost, seeds)
    return {"workload": "ring7_256x256", "block": 8, "n": 64, "block_solves": res.stats["block_solves"],
            "waves": res.stats["waves"], "device_ms": res.stats["device_ms"], "cpu_fim_ms": us_fim / 1e3,
            "cpu_fmm_ms": us_fmm / 1e3, "max_rel_vs_fim": rel_diff(res.field, fim),
            "max_rel_vs_fmm": rel_diff(res.field, fmm), "vs_fmm64": fmm64_errors(res.field, ref64),
            "fim_vs_fmm64": fmm64_errors(fim, ref64),
            "reference_schedule": reference_schedule(o, cost, seeds, 8, 64, 64, fim)}


def reference_schedule(o, cost, seeds, block: int, n: int, wg: int, fim) -> dict:
    """The reference's own gHCM schedule on the same field, restated on the CPU
    by the oracle (stale priority keys, the dirty set cleared after the wave so
    a block dirtied in flight is lost, check_border writing into neighbours,
    no residual check; one work-group of wg lanes per tile): its block-solves
    and waves, and how far its field ends from the fixed point."""
    from oracle.oracle import rel_diff

    out, solves, waves = o.hcm(cost, seeds, block=block, max_jobs=n, eps=EPS, wg=wg)
    return {"block": block, "n": n, "work_group": wg, "block_solves": int(solves), "waves": int(waves),
            "max_rel_vs_fim": rel_diff(out, fim), "residual": o.residual(cost, out),
            "note": "CPU restatement; the wave's jobs run one after another"}


def _learned_setup(g, learned, params, threshold, policy, block: int = BLOCK, **kw):
    cfg = g.HcmConfig(block_size=block, fim_minimum_change=EPS, schedule=g.Schedule.Learned, **kw)
    s = g.HcmSetup(cfg)
    learned.set_model(s, params, threshold)
    learned.set_policy(s, policy)
    return s


def ring_4096(g, dev, stream, flush, steps: int, warmup: int, checks: bool) -> dict:
    """The plain device schedule at scale: the 4096^2 seven-ring field (radii
    256..1920, width 16, speed 0.01, 64-cell gaps, one centre source), tiles of
    16, n in {256, 1024, 4096}, device-resident and timed like the headline,
    with its parity against the reference FIM and FMM and its error against
    the FP64 FMM."""
    import torch

    from ghcm_gb300 import fields
    from oracle.oracle import Oracle, build, rel_diff

    speed, seeds = fields.ring7_large(seed=1)
    cells = speed.size
    d_speed = torch.from_numpy(speed).to(dev)
    d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    out, fields_out = {"workload": RING_WORKLOAD, "block": BLOCK}, {}
    for n in N_SWEEP:
        d_time = torch.empty_like(d_speed)
        with g.HcmSetup(g.HcmConfig(block_size=BLOCK, max_jobs=n, fim_minimum_change=EPS)) as s:
            ms, sts = timed_device_solves(g, s, d_speed, d_seeds, d_time, stream, flush, steps, warmup)
        fields_out[n] = d_time.cpu().numpy()
        out[f"n{n}"] = {"mcells": cells / (ms * 1e3), "ms": ms,
                        "kernel_ms": statistics.mean(x["kernel_ms"] for x in sts),
                        "block_solves": statistics.mean(x["block_solves"] for x in sts),
                        "waves": statistics.mean(x["waves"] for x in sts)}
    if checks:
        build(with_reference=False)
        o = Oracle()
        cost = fields.cost_from_speed(speed)
        fim, us_fim = o.fim(cost, seeds, EPS)
        fmm, us_fmm = o.fmm(cost, seeds)
        ref64, _ = o.fmm64(cost, seeds)
        out["cpu_fim_ms"], out["cpu_fmm_ms"] = us_fim / 1e3, us_fmm / 1e3
        out["fim_vs_fmm"] = rel_diff(fmm, fim)
        out["fim_vs_fmm64"] = fmm64_errors(fim, ref64)
        for n, f in fields_out.items():
            out[f"n{n}"]["check"] = {"max_rel_vs_fim": rel_diff(f, fim), "max_rel_vs_fmm": rel_diff(f, fmm),
                                     "vs_fmm64": fmm64_errors(f, ref64), "residual": o.residual(cost, f)}
    return out


def kernel_compare(g, dev, stream, flush, steps: int) -> dict:
    """The two tile kernels of the reference (systolic, data/eikonal_ghcm_systolic.cl,
    and block-FIM, data/eikonal_ghcm_fim.cl:214-392) timed on the same fields:
    the 256^2 ring (B = 8, n = 64), the 4096^2 rings (B = 16, n = 256) and the
    4096^2 noise field (B = 16, n = 1024), plain schedule, device-resident."""
    import torch

    from ghcm_gb300 import fields

    cases = {"ring7_256x256_b8_n64": (fields.ring7_small(seed=1), 8, 64),
             "ring7_4096x4096_b16_n256": (fields.ring7_large(seed=1), 16, 256),
             "noise_4096x4096_b16_n1024": (make_workload("noise"), 16, 1024)}
    out = {}
    for name, ((speed, seeds), block, n) in cases.items():
        d_speed = torch.from_numpy(speed).to(dev)
        d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
        d_time = torch.empty_like(d_speed)
        row = {}
        for kname, kern in (("systolic", g.Kernel.Systolic), ("fim", g.Kernel.FIM)):
            with g.HcmSetup(g.HcmConfig(block_size=block, max_jobs=n, fim_minimum_change=EPS, kernel=kern)) as s:
                ms, sts = timed_device_solves(g, s, d_speed, d_seeds, d_time, stream, flush, steps, 1)
            row[kname] = {"ms": ms, "mcells": speed.size / (ms * 1e3),
                          "block_solves": statistics.mean(x["block_solves"] for x in sts),
                          "waves": statistics.mean(x["waves"] for x in sts),
                          "sweeps_note": "block-FIM counts one open-set iteration as a sweep"}
        row["faster"] = min(("systolic", "fim"), key=lambda k: row[k]["ms"])
        out[name] = row
    return out


def run_batched(args, world, rank, local) -> int:
    """C4: the batch of independent instances in one persistent launch from a
    CUDA graph, configured by the autotuner; ranks split the instances."""
    import torch

    import ghcm_gb300 as g
    from ghcm_gb300 import fields
    from oracle.oracle import Oracle, build, rel_diff

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    all_insts = batch_instances()
    mine = g.shard_instances([i.speed.size for i in all_insts], world)[rank]
    insts = [all_insts[i] for i in mine]
    cells = sum(i.speed.size for i in insts)
    total_cells = sum(i.speed.size for i in all_insts)
    # every instance's speed and time field packed in one buffer each (host
    # pinned and device), at 256-byte aligned offsets, so the end-to-end step
    # moves the batch with one copy each way
    offs, at = [], 0
    for i in insts:
        offs.append(at)
        at += (i.speed.size + 63) // 64 * 64
    h_speed_all = torch.empty(at, dtype=torch.float32).pin_memory()
    h_time_all = torch.empty(at, dtype=torch.float32).pin_memory()
    d_speed_all = torch.empty(at, dtype=torch.float32, device=dev)
    d_time_all = torch.empty(at, dtype=torch.float32, device=dev)
    view = lambda buf, k: buf[offs[k]:offs[k] + insts[k].speed.size].view(insts[k].speed.shape)
    for k, i in enumerate(insts):
        view(h_speed_all, k).copy_(torch.from_numpy(i.speed))
    d_speed_all.copy_(h_speed_all)
    dinst = [g.DeviceInstance(view(d_speed_all, k), torch.from_numpy(i.seeds.astype(np.int32)).to(dev),
                              view(d_time_all, k)) for k, i in enumerate(insts)]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    t0 = time.perf_counter()
    if args.no_autotune:  # a fixed tile size and n (e.g. for a profiler capture of the timed launch)
        best, trials = g.HcmConfig(block_size=args.block, max_jobs=args.n, fim_minimum_change=EPS), []
    else:
        best, trials = g.autotune_batch(g.HcmConfig(block_size=16, fim_minimum_change=EPS), dinst, reps=1)
    tune_s = time.perf_counter() - t0
    setup = g.HcmSetup(best)
    batch = g.Batch(setup, dinst)
    info = batch.info()
    for _ in range(args.warmup):
        batch.run(stream)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    with Clocks(local) as clk:
        barrier()
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            stats.append(batch.run(stream))
            ev[i][1].record(stream)
        barrier()
    clocks = clk.summary()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = total_cells / (ms * 1e3)

    # end to end: pinned host fields in, every time field out, inside the timed region
    e2e = []
    for it in range(1 + max(3, min(args.steps, 5))):  # the first pass is an untimed warm-up
        barrier()
        t0 = time.perf_counter()
        d_speed_all.copy_(h_speed_all, non_blocking=True)
        batch.run(stream)
        h_time_all.copy_(d_time_all, non_blocking=True)
        torch.cuda.synchronize(dev)
        if it:
            e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = statistics.median(e2e)
    if dist is not None:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())

    B = info["block_size"]
    solves = statistics.mean(st["block_solves"] for st in stats)
    achieved = solves * bytes_per_solve(B) / (ms * 1e-3) / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD, "instances": len(all_insts), "cells": total_cells,
                   "instances_this_rank": len(insts), "block": B, "n": info["max_jobs"],
                   "max_sweeps": info["max_sweeps"], "cuda_graph": bool(info["graph"]), "eps": EPS,
                   "tma_instances": info["tma_instances"], "autotune_s": tune_s,
                   "l2": "flushed between steps (256 MiB write outside the events)",
                   "parallelism": f"instances split over {world} rank(s)"},
        "e2e": {"value": total_cells / (e2e_ms * 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 4 * at, "d2h_bytes_per_step": 4 * at,
                "layout": "all instances in one pinned buffer each way (256-byte aligned offsets), one copy each",
                "samples_ms": e2e},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": batch_traffic(B, solves),
                     "traffic_basis": "DRAM bytes per block-solve of an ncu capture of this batch at the same tile "
                                      "size (profiles/k_solve_batch512.json) x this run's block-solves",
                     "kernel": f"k_solve<{B},systolic> (batch)",
                     "bytes_per_block_solve": bytes_per_solve(B), "block_solves": solves,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in peaks else "fallback"},
        "autotune": trials,
        "gpu_launches": LAUNCHES_PER_SOLVE * args.steps,
        "clocks": clocks,
        "solver": {"waves": statistics.mean(st["waves"] for st in stats),
                   "residual_passes": statistics.mean(st["residual_passes"] for st in stats),
                   "max_active": max(st["max_active"] for st in stats)},
    }
    if rank == 0:
        build(with_reference=False)
        o = Oracle()
        # parity on a fixed sample of this rank's instances against the reference FIM
        worst = 0.0
        for k in range(0, len(insts), max(1, len(insts) // 8)):
            inst = insts[k]
            ref = o.fim(fields.cost_from_speed(inst.speed), inst.seeds, EPS)[0]
            worst = max(worst, rel_diff(dinst[k].d_time.cpu().numpy(), ref))
        line["check"] = {"max_rel_vs_fim_sample": worst, "sample": "every len/8-th instance of rank 0"}
        # FP64 accuracy on a few instances of each kind
        errs = []
        for k in range(0, len(insts), max(1, len(insts) // 6)):
            inst = insts[k]
            ref64, _ = o.fmm64(fields.cost_from_speed(inst.speed), inst.seeds)
            e = fmm64_errors(dinst[k].d_time.cpu().numpy(), ref64)
            errs.append({"kind": inst.kind, "side": int(inst.speed.shape[0]), **e})
        line["check"]["vs_fmm64_sample"] = errs
        if not args.no_cpu_baseline:
            sample = all_insts[::8]
            threads = max(1, os.cpu_count() or 1)
            us = cpu_fmm_pool(o, sample, threads)
            sc = sum(i.speed.size for i in sample)
            line["cpu_baseline"] = {"value": sc / us, "unit": UNIT, "cores": threads, "kind": "port",
                                    "sample": f"every 8th instance ({len(sample)} instances, {sc} cells), reference "
                                              "FMM, one instance per host thread at a time",
                                    "cpu": _cpu_name()}
        print(json.dumps(line), flush=True)
    batch.close()
    setup.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def maze_model(block: int):
    """The schedule model trained on maze traces for tiles of `block`, if present."""
    p = ROOT / "ghcm_gb300" / "models" / f"schedule_maze4096_b{block}.npz"
    return p if p.exists() else None


def run_maze(args, world, rank, local) -> int:
    """C5: the 16384^2 cellular-automaton maze (wall speed 0.001, open 1.0, 64
    sources in open cells, ~2 GB of device state). The library's autotuner
    (ghcm_autotune_batch, on the field as a batch of one) picks tile size, n,
    sweep cap and tile kernel; the learned schedule (a model trained on maze
    traces for that tile size) is timed against the plain schedule at that
    config. `value` is the learned schedule's Mcell/s; both fields are
    checked against the reference FIM, and against an FP64 FMM of the whole
    field (errors on the whole field and on the central 2048^2 crop)."""
    import torch

    import ghcm_gb300 as g
    from ghcm_gb300 import fields, learned
    from oracle.oracle import Oracle, build, rel_diff

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    t0 = time.perf_counter()
    speed, seeds = fields.ca_maze(16384, seed=MAZE_SEED)
    gen_s = time.perf_counter() - t0
    cells = speed.size
    d_speed = torch.from_numpy(speed).to(dev)
    d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    d_time = torch.empty_like(d_speed)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    t0 = time.perf_counter()
    if args.no_autotune:  # a fixed config (e.g. for a profiler capture of the timed launches)
        tuned, trials = g.HcmConfig(block_size=args.block, max_jobs=args.n, max_sweeps=args.sweeps,
                                    fim_minimum_change=EPS), []
    else:
        tuned, trials = g.autotune_batch(g.HcmConfig(block_size=16, fim_minimum_change=EPS),
                                         [g.DeviceInstance(d_speed, d_seeds, d_time)], reps=1)
    tune_s = time.perf_counter() - t0
    block, n = tuned.block_size, tuned.max_jobs
    plain_cfg = g.HcmConfig(block_size=block, max_jobs=n, max_sweeps=tuned.max_sweeps, kernel=tuned.kernel,
                            fim_minimum_change=EPS)
    s_plain = g.HcmSetup(plain_cfg)
    mpath = maze_model(block)
    s_learned = None
    if mpath is not None and tuned.kernel == g.Kernel.Systolic:
        params, threshold, meta = learned.load_model(mpath)
        # the tuned n caps the wave and waves with fewer qualifying tiles are
        # filled to n in key order (the best of a cap / fill / threshold sweep
        # on this field: 141 waves against the plain schedule's 172)
        s_learned = _learned_setup(g, learned, params, threshold, learned.POLICY_SCORE, block=block, max_jobs=n,
                                   fallback_jobs=n, max_sweeps=tuned.max_sweeps)
    head = s_learned if s_learned is not None else s_plain
    d_time_p = torch.empty_like(d_speed)
    with Clocks(local) as clk:
        ms, stats = timed_device_solves(g, head, d_speed, d_seeds, d_time, stream, flush, args.steps, args.warmup)
        pms, pstats = timed_device_solves(g, s_plain, d_speed, d_seeds, d_time_p, stream, flush, args.steps,
                                          args.warmup)
    clocks = clk.summary()
    value = cells / (ms * 1e3)
    h_speed = torch.from_numpy(speed).pin_memory()
    h_time = torch.empty_like(h_speed).pin_memory()
    g.eikonal_hcm_cuda_ex(head, h_speed.numpy(), seeds, input_is_speed=True, out=h_time.numpy())  # warm-up
    e2e = []
    for _ in range(2):
        t0 = time.perf_counter()
        g.eikonal_hcm_cuda_ex(head, h_speed.numpy(), seeds, input_is_speed=True, out=h_time.numpy())
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = min(e2e)
    g.solve_device(head, d_speed, d_seeds, d_time, stream=stream)
    g.solve_device(s_plain, d_speed, d_seeds, d_time_p, stream=stream)
    field = d_time.cpu().numpy()
    field_p = d_time_p.cpu().numpy()
    del d_time, d_time_p
    solves = statistics.mean(st["block_solves"] for st in stats)
    k_ms = statistics.mean(st["kernel_ms"] for st in stats)
    achieved = solves * bytes_per_solve(block) / (k_ms * 1e-3) / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    capture = load_traffic("k_solve_maze16384.json", block=block, n=n)
    cap_solves = load_block_solves("k_solve_maze16384.json")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": MAZE_WORKLOAD, "seed": MAZE_SEED, "block": block, "n": n,
                   "max_sweeps": tuned.max_sweeps, "kernel": "fim" if tuned.kernel == g.Kernel.FIM else "systolic",
                   "schedule": "learned (score policy)" if s_learned is not None else "plain",
                   "model": mpath.name if mpath is not None else None, "eps": EPS, "sources": int(len(seeds)),
                   "generate_s": gen_s, "autotune_s": tune_s, "device_state_gb": 2 * 4 * cells / 1e9,
                   "l2": "flushed between steps"},
        "plain": {"value": cells / (pms * 1e3), "unit": UNIT, "ms_per_step": pms,
                  "block_solves": statistics.mean(st["block_solves"] for st in pstats),
                  "waves": statistics.mean(st["waves"] for st in pstats)},
        "learned_vs_plain": {"mcells_ratio": pms / ms,
                             "block_solves_ratio": solves / statistics.mean(st["block_solves"] for st in pstats)},
        "e2e": {"value": cells / (e2e_ms * 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 4 * cells + int(seeds.nbytes), "d2h_bytes_per_step": 4 * cells},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (capture / cap_solves * solves) if capture and cap_solves else None,
                     "traffic_basis": "DRAM bytes per block-solve of an ncu capture of the plain maze launch at the "
                                      "same tile size and n (profiles/k_solve_maze16384.json) x this run's "
                                      "block-solves",
                     "kernel": f"k_solve<{block},{'fim' if tuned.kernel == g.Kernel.FIM else 'systolic'}>",
                     "bytes_per_block_solve": bytes_per_solve(block), "block_solves": solves, "kernel_ms": k_ms},
        "autotune": trials,
        "gpu_launches": (LAUNCHES_PER_LEARNED_SOLVE if s_learned is not None else LAUNCHES_PER_SOLVE) * args.steps,
        "clocks": clocks,
        "solver": {"waves": statistics.mean(st["waves"] for st in stats),
                   "residual_passes": statistics.mean(st["residual_passes"] for st in stats),
                   "max_active": max(st["max_active"] for st in stats)},
    }
    if rank == 0:
        build(with_reference=False)
        o = Oracle()
        cost = fields.cost_from_speed(speed)
        line["check"] = {"residual": o.residual(cost, field), "finite": bool(np.isfinite(field).all()),
                         "seeds_zero": bool(np.all(field[seeds[:, 1], seeds[:, 0]] == 0)),
                         "learned_vs_plain_max_rel": rel_diff(field, field_p)}
        if not args.no_cpu_baseline:
            fim, us_fim = o.fim(cost, seeds, EPS)
            line["check"]["max_rel_vs_fim"] = rel_diff(field, fim)
            line["check"]["plain_max_rel_vs_fim"] = rel_diff(field_p, fim)
            del fim
            ref64, us64 = o.fmm64(cost, seeds)
            c0 = (16384 - MAZE_CROP) // 2
            crop = (slice(c0, c0 + MAZE_CROP), slice(c0, c0 + MAZE_CROP))
            line["check"]["vs_fmm64_crop"] = {**fmm64_errors(field[crop], ref64[crop]),
                                              "crop": f"[{c0}:{c0 + MAZE_CROP}]^2"}
            line["check"]["vs_fmm64_full"] = fmm64_errors(field, ref64)
            line["check"]["plain_vs_fmm64_full"] = fmm64_errors(field_p, ref64)
            line["cpu_baseline"] = {"value": cells / us_fim, "unit": UNIT, "cores": 1, "kind": "port",
                                    "sample": "one reference FIM of the whole field (eps 1e-5), 1 host thread",
                                    "fmm64_ms": us64 / 1e3, "cpu": _cpu_name()}
        print(json.dumps(line), flush=True)
    if s_learned is not None:
        s_learned.close()
    s_plain.close()
    return 0


def run_ring(args, world, rank, local) -> int:
    """C2 as its own line: the 4096^2 seven-ring field with the plain device
    schedule at --n (the configuration's other n beside it)."""
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

    speed, seeds = make_workload("ring")
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
    step_spread = {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)}
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
    # untimed warm-up: the first host-pointer call sizes the context's staging buffers
    g.eikonal_hcm_cuda_ex(setup, h_speed.numpy(), seeds, input_is_speed=True, out=h_time.numpy())
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
        "warmup": args.warmup, "ms_per_step": ms, "step_ms": step_spread, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": RING_WORKLOAD, "block": args.block, "n": args.n, "kernel": args.kernel, "eps": EPS,
                   "sources": int(len(seeds)), "l2": "flushed between steps (256 MiB write outside the events)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * cells / (e2e_mean * 1e3), "unit": UNIT, "ms_per_step": e2e_mean,
                "h2d_bytes_per_step": cells * 4 + int(seeds.nbytes), "d2h_bytes_per_step": cells * 4},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": load_traffic(), "kernel": f"k_solve<{args.block},{args.kernel}>",
                     "bytes_per_block_solve": bps, "block_solves": solves, "kernel_ms": k_ms,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in peaks else "fallback"},
        "n_sweep": n_sweep,
        "gpu_launches": LAUNCHES_PER_SOLVE * args.steps,
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
            ref64, _ = Oracle().fmm64(cost, seeds)
            line["check"]["vs_fmm64"] = fmm64_errors(field, ref64)
            line["check"]["fim_vs_fmm64"] = fmm64_errors(fim, ref64)
        if not args.no_cpu_baseline:
            line["small_ring_256"] = small_ring_check(g)
        print(json.dumps(line), flush=True)
    setup.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_noise(args, world, rank, local) -> int:
    """The headline: the learned block schedule against the plain one on the
    4096^2 noise field. `value` is the learned schedule's Mcell/s (at most
    LEARNED_CAP jobs a wave, filled to 4 x SMs in key order); the plain
    schedule is timed the same way in the same run at each n of PLAIN_SWEEP
    and the fastest is the comparison (`plain`), the others and the veto
    policy under `others`; both fields are checked against the reference FIM
    and FMM and the FP64 FMM. The seven-ring field (C2) and the 256^2 ring
    (C1) ride along as sub-objects."""
    import torch

    import ghcm_gb300 as g
    from ghcm_gb300 import fields, learned

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

    params, threshold, meta = learned.load_model(MODEL)
    speed, seeds = make_workload("noise")
    h, w = speed.shape
    cells = h * w
    d_speed = torch.from_numpy(speed).to(dev)
    d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    d_time_l = torch.empty_like(d_speed)
    d_time_p = torch.empty_like(d_speed)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    with g.HcmSetup(g.HcmConfig(block_size=BLOCK)) as probe:
        sms = probe.sm_count
    fill = 4 * sms
    caps = {"max_jobs": LEARNED_CAP, "fallback_jobs": fill}
    s_learned = _learned_setup(g, learned, params, threshold, learned.POLICY_SCORE, **caps)
    plain_ns = [n or fill for n in (PLAIN_SWEEP if not args.quick else (0,))]
    s_plains = {n: g.HcmSetup(g.HcmConfig(block_size=BLOCK, max_jobs=n, fim_minimum_change=EPS)) for n in plain_ns}

    for _ in range(args.warmup):
        g.solve_device(s_learned, d_speed, d_seeds, d_time_l, stream=stream)
        for sp in s_plains.values():
            g.solve_device(sp, d_speed, d_seeds, d_time_p, stream=stream)
    barrier()

    def timed(setup, d_time):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        sts = []
        barrier()
        for i in range(args.steps):
            flush.fill_(float(i))  # evict the fields from L2 between steps (outside the events)
            ev[i][0].record(stream)
            sts.append(g.solve_device(setup, d_speed, d_seeds, d_time, stream=stream))
            ev[i][1].record(stream)
        barrier()
        return [a.elapsed_time(b) for a, b in ev], sts

    with Clocks(local) as clk:
        t_wall = time.perf_counter()
        step_ms, stats = timed(s_learned, d_time_l)
        t_wall = time.perf_counter() - t_wall
        plain_runs = {n: timed(sp, d_time_p) for n, sp in s_plains.items()}
    clocks = clk.summary()
    plain_n = min(plain_runs, key=lambda n: sum(plain_runs[n][0]))  # the fastest plain n is the comparison
    plain_ms, plain_stats = plain_runs[plain_n]
    s_plain = s_plains[plain_n]
    ms = sum(step_ms) / len(step_ms)
    pms = sum(plain_ms) / len(plain_ms)
    if dist is not None:
        t = torch.tensor([ms, pms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, pms = float(t[0].item()), float(t[1].item())
    value = world * cells / (ms * 1e3)
    plain_value = world * cells / (pms * 1e3)
    counters = learned.counters(s_learned)

    # end to end through the public host-pointer call (pinned speed in, time field out), both schedules
    h_speed = torch.from_numpy(speed).pin_memory()
    h_time = torch.empty((h, w), dtype=torch.float32).pin_memory()

    def e2e_of(setup):
        g.eikonal_hcm_cuda_ex(setup, h_speed.numpy(), seeds, input_is_speed=True, out=h_time.numpy())  # warm-up
        out = []
        for _ in range(max(3, min(args.steps, 5))):
            t0 = time.perf_counter()
            g.eikonal_hcm_cuda_ex(setup, h_speed.numpy(), seeds, input_is_speed=True, out=h_time.numpy())
            out.append((time.perf_counter() - t0) * 1e3)
        return statistics.median(out), out

    e2e_ms, e2e_samples = e2e_of(s_learned)
    e2e_plain_ms = e2e_of(s_plain)[0] if not args.quick else float("nan")
    if dist is not None:
        t = torch.tensor([e2e_ms, e2e_plain_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms, e2e_plain_ms = float(t[0].item()), float(t[1].item())
    # leave each schedule's device-resident field for the checks
    g.solve_device(s_learned, d_speed, d_seeds, d_time_l, stream=stream)
    g.solve_device(s_plain, d_speed, d_seeds, d_time_p, stream=stream)
    field_l = d_time_l.cpu().numpy()
    field_p = d_time_p.cpu().numpy()

    # the plain schedule's other n (timed above) and the veto policy, device-timed (fewer steps)
    k = max(1, min(args.steps, 3))
    others, other_fields = {}, {}
    for n, (n_ms, n_st) in plain_runs.items():
        if n == plain_n:
            continue
        others[f"plain_n{n}"] = {"mcells": cells / (statistics.mean(n_ms) * 1e3), "ms": statistics.mean(n_ms),
                                 "block_solves": statistics.mean(x["block_solves"] for x in n_st),
                                 "waves": statistics.mean(x["waves"] for x in n_st)}
    if not args.quick:
        s_veto = _learned_setup(g, learned, params, threshold, learned.POLICY_VETO, max_jobs=plain_n)
        d_t = torch.empty_like(d_speed)
        o_ms, o_st = timed_device_solves(g, s_veto, d_speed, d_seeds, d_t, stream, flush, k, 1)
        other_fields["learned_veto"] = d_t.cpu().numpy()
        others["learned_veto"] = {"n": plain_n, "mcells": cells / (o_ms * 1e3), "ms": o_ms,
                                        "block_solves": statistics.mean(x["block_solves"] for x in o_st),
                                        "waves": statistics.mean(x["waves"] for x in o_st)}
        s_veto.close()

    solves = statistics.mean(st["block_solves"] for st in stats)
    plain_solves = statistics.mean(st["block_solves"] for st in plain_stats)
    k_ms = statistics.mean(st["kernel_ms"] for st in stats)
    bps = bytes_per_solve(BLOCK)
    achieved = solves * bps / (k_ms * 1e-3) / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms,
        "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)},
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "schedule": "learned (score policy)", "block": BLOCK, **caps,
                   "model": MODEL.name, "model_train_seeds": int(len(meta.get("train_seeds", []))),
                   "threshold": threshold, "field_seed": NOISE_EVAL_SEED, "sources": int(len(seeds)), "eps": EPS,
                   "l2": "flushed between steps (256 MiB write outside the events)",
                   "parallelism": f"replicas x{world}"},
        "plain": {"value": plain_value, "unit": UNIT, "ms_per_step": pms, "n": plain_n,
                  "chosen_as": f"fastest of plain n in {sorted(plain_runs)}",
                  "block_solves": plain_solves, "waves": statistics.mean(st["waves"] for st in plain_stats),
                  "kernel_ms": statistics.mean(st["kernel_ms"] for st in plain_stats),
                  "e2e": None if args.quick else {"value": world * cells / (e2e_plain_ms * 1e3), "unit": UNIT,
                                                  "ms_per_step": e2e_plain_ms}},
        "learned_vs_plain": {"mcells_ratio": value / plain_value, "block_solves_ratio": solves / plain_solves,
                             "waves_ratio": statistics.mean(st["waves"] for st in stats) /
                                            statistics.mean(st["waves"] for st in plain_stats)},
        "e2e": {"value": world * cells / (e2e_ms * 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": cells * 4 + int(seeds.nbytes), "d2h_bytes_per_step": cells * 4,
                "samples_ms": e2e_samples, "api": "ghcm_solve (host pointers, pinned)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": load_traffic("k_solve_noise4096_learned.json"),
                     "kernel": f"k_solve<{BLOCK},systolic> (learned schedule)",
                     "bytes_per_block_solve": bps, "block_solves": solves, "kernel_ms": k_ms,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in peaks else "fallback"},
        "others": others,
        "gpu_launches": LAUNCHES_PER_LEARNED_SOLVE * args.steps,
        "clocks": clocks,
        "solver": {"waves": statistics.mean(st["waves"] for st in stats),
                   "residual_passes": statistics.mean(st["residual_passes"] for st in stats),
                   "max_active": max(st["max_active"] for st in stats), "counters": counters,
                   "wall_s_timed": t_wall},
    }
    if rank == 0:
        from oracle.oracle import Oracle, rel_diff  # checker: parity of the benchmarked fields

        cost = fields.cost_from_speed(speed)
        o = Oracle()
        line["check"] = {"residual": o.residual(cost, field_l), "residual_plain": o.residual(cost, field_p),
                         "seeds_zero": bool(np.all(field_l[seeds[:, 1], seeds[:, 0]] == 0)),
                         "learned_vs_plain_max_rel": rel_diff(field_l, field_p)}
        if not args.no_cpu_baseline:
            fim, fmm, base = cpu_baseline(speed, seeds)
            line["cpu_baseline"] = base
            ref64, _ = o.fmm64(cost, seeds)
            line["check"].update({
                "max_rel_vs_fim": rel_diff(field_l, fim), "max_rel_vs_fmm": rel_diff(field_l, fmm),
                "plain_max_rel_vs_fim": rel_diff(field_p, fim), "plain_max_rel_vs_fmm": rel_diff(field_p, fmm),
                "fim_vs_fmm": rel_diff(fim, fmm), "vs_fmm64": fmm64_errors(field_l, ref64),
                "plain_vs_fmm64": fmm64_errors(field_p, ref64), "fim_vs_fmm64": fmm64_errors(fim, ref64)})
            for name, f in other_fields.items():
                others[name]["max_rel_vs_fim"] = rel_diff(f, fim)
            if not args.quick:
                line["reference_schedule_n1024"] = reference_schedule(o, cost, seeds, BLOCK, 1024, 256, fim)
        if not args.quick:
            line["ring_4096"] = ring_4096(g, dev, stream, flush, k, 1, checks=not args.no_cpu_baseline)
        if not args.no_cpu_baseline and not args.quick:
            line["small_ring_256"] = small_ring_check(g)
        if not args.quick:
            line["kernels"] = kernel_compare(g, dev, stream, flush, k)
        print(json.dumps(line), flush=True)
    s_learned.close()
    for sp in s_plains.values():
        sp.close()
    if dist is not None:
        dist.destroy_process_group()
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
    ap.add_argument("--quick", action="store_true",
                    help="default workload: the headline pair only (no other n, veto policy or ring sub-objects)")
    ap.add_argument("--workload", default="noise", choices=["noise", "ring", "batched", "maze"])
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched and maze workloads: use --block, --n (and --sweeps) instead of the autotuner's choice")
    ap.add_argument("--sweeps", type=int, default=0, help="maze workload with --no-autotune: the inner-sweep cap")
    args = ap.parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.workload == "batched":
        return run_batched(args, world, rank, local)
    if args.workload == "maze":
        return run_maze(args, world, rank, local)
    if args.workload == "ring":
        return run_ring(args, world, rank, local)
    return run_noise(args, world, rank, local)



if __name__ == "__main__":
    sys.exit(main())
