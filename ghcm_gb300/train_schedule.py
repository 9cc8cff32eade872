"""Trains the learned block schedule on traces of the plain solver.

    python -m ghcm_gb300.train_schedule [--field noise|maze] [--size 4096] [--seeds 32]
                                         [--first-seed 1001] [--block 16] [--n 1024]
                                         [--epochs 12] [--out FILE]

For each training seed: a fractal value-noise speed field (6 octaves, base
period size/8, persistence 0.5, speed = clamp(exp(2 noise), 0.02, 1)) with 16
random sources, or (--field maze) a cellular-automaton maze (walls at speed
0.001, open cells 1.0, 5 smoothing passes) with 64 sources in open cells, is
solved by the plain device schedule (tiles of --block, n = --n) with the trace
recorder on. Each block-solve's features are labelled with the
hindsight target of learned.final_labels (the solve moved some cell by more
than eps and no later solve of its tile did); the 12 -> 64 -> 64 -> 1 MLP is
trained by the library's CUDA kernels and written with its metadata to --out.

The fields are generated in a process pool started before any CUDA call.
"""
from __future__ import annotations

import argparse
import json
import time
from concurrent.futures import ProcessPoolExecutor
from multiprocessing import get_context
from pathlib import Path

import numpy as np

DEFAULT_OUT = Path(__file__).resolve().parent / "models" / "schedule_noise4096_b16.npz"


def _field(args):
    from ghcm_gb300 import fields

    kind, size, seed = args
    if kind == "maze":
        return seed, fields.ca_maze(size, seed=seed, sources=64)
    return seed, fields.value_noise(size, seed=seed, base_period=size / 8.0, sources=16)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--field", default="noise", choices=["noise", "maze"])
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--seeds", type=int, default=32)
    ap.add_argument("--first-seed", type=int, default=1001)
    ap.add_argument("--block", type=int, default=16)
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--threshold", type=float, default=0.5)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--out", type=Path, default=DEFAULT_OUT)
    args = ap.parse_args(argv)

    seeds = list(range(args.first_seed, args.first_seed + args.seeds))
    t0 = time.perf_counter()
    with ProcessPoolExecutor(max_workers=max(1, args.workers), mp_context=get_context("spawn")) as ex:
        made = dict(ex.map(_field, [(args.field, args.size, s) for s in seeds]))
    t_gen = time.perf_counter() - t0

    import ghcm_gb300 as g
    from ghcm_gb300 import learned

    traces, labels = [], []
    t0 = time.perf_counter()
    with g.HcmSetup(g.HcmConfig(block_size=args.block, max_jobs=args.n)) as setup:
        learned.enable_trace(setup, 1 << 23)
        for s in seeds:
            speed, src = made[s]
            g.eikonal_hcm_cuda_ex(setup, speed, src, input_is_speed=True)
            tr = learned.read_trace(setup)
            if tr.total > len(tr):
                raise RuntimeError(f"trace of seed {s} overflowed ({tr.total} solves)")
            traces.append(tr)
            labels.append(learned.final_labels(tr))
    t_trace = time.perf_counter() - t0
    tr = learned.Trace.concat(traces)
    y = np.concatenate(labels)
    t0 = time.perf_counter()
    params, losses = learned.train(tr.features, y, epochs=args.epochs, batch=4096, lr=args.lr, seed=0)
    t_train = time.perf_counter() - t0
    p = learned.predict(params, tr.features)
    yb = y.astype(bool)
    summary = {
        "records": int(len(tr)), "useful_rate": float(tr.useful.mean()), "final_rate": float(y.mean()),
        "train_accuracy": float(np.mean((p >= args.threshold) == yb)), "mean_p_final": float(p[yb].mean()),
        "mean_p_not_final": float(p[~yb].mean()), "epoch_loss": [float(v) for v in losses],
        "seconds": {"generate": t_gen, "trace": t_trace, "train": t_train},
    }
    args.out.parent.mkdir(parents=True, exist_ok=True)
    learned.save_model(args.out, params, args.threshold, train_seeds=np.array(seeds), size=args.size,
                       field=args.field, block=args.block, trace_n=args.n, label="final", epoch_loss=np.array(losses),
                       summary=json.dumps(summary))
    print(json.dumps({"model": str(args.out), **summary}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
