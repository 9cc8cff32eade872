"""ctypes front end of the CPU checkers.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of bench.py. The product package ``ghcm_gb300`` never
imports this module.

* ``Oracle``     - the restatement in ghcm_oracle.cpp (builds on any host).
* ``Reference``  - the reference's own solvers compiled from its sources into
  ``_ref/libghcm_ref.so`` (only where the reference sources are present).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "libghcm_oracle.so"
REF_SO = HERE / "_ref" / "libghcm_ref.so"
# the reference checkout beside this repository, or GHCM_REF_SRC
REF_SRC = Path(os.environ.get("GHCM_REF_SRC", HERE.parent.parent / "reference" / "src"))

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_i64p = ctypes.POINTER(ctypes.c_int64)


def build(with_reference: bool = True) -> None:
    """Compile the restatement, and the reference build when its sources exist."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if with_reference and (REF_SRC / "eikonal_fim.cpp").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_SRC={REF_SRC}"], check=True)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def _prep(cost: np.ndarray, seeds: np.ndarray):
    cost = np.ascontiguousarray(cost, dtype=np.float32)
    seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint32).reshape(-1, 2))
    h, w = cost.shape
    return cost, seeds, w, h


class _Lib:
    prefix = ""

    def __init__(self, path: Path):
        self.lib = ctypes.CDLL(str(path))
        p = self.prefix
        fim = getattr(self.lib, f"{p}_fim")
        fim.argtypes = [ctypes.c_float, _f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, ctypes.c_uint32, _f32p, _i64p]
        fim.restype = ctypes.c_int
        fmm = getattr(self.lib, f"{p}_fmm")
        fmm.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, ctypes.c_uint32, _f32p, _i64p]
        fmm.restype = ctypes.c_int
        self._fim, self._fmm = fim, fmm

    def fim(self, cost, seeds, eps: float = 1e-5):
        """Sequential FIM on a COST field; returns (time field, microseconds)."""
        cost, seeds, w, h = _prep(cost, seeds)
        out = np.empty((h, w), dtype=np.float32)
        us = ctypes.c_int64(0)
        rc = self._fim(eps, _ptr(cost, _f32p), w, h, _ptr(seeds, _u32p), len(seeds), _ptr(out, _f32p), ctypes.byref(us))
        if rc != 0:
            raise ValueError(f"fim failed ({rc})")
        return out, us.value

    def fmm(self, cost, seeds):
        """Sequential FP32 FMM on a COST field; returns (time field, microseconds)."""
        cost, seeds, w, h = _prep(cost, seeds)
        out = np.empty((h, w), dtype=np.float32)
        us = ctypes.c_int64(0)
        rc = self._fmm(_ptr(cost, _f32p), w, h, _ptr(seeds, _u32p), len(seeds), _ptr(out, _f32p), ctypes.byref(us))
        if rc != 0:
            raise ValueError(f"fmm failed ({rc})")
        return out, us.value


class Oracle(_Lib):
    prefix = "ghcm_oracle"

    def __init__(self, path: Path = ORACLE_SO):
        if not path.exists():
            build(with_reference=False)
        super().__init__(path)
        f = self.lib.ghcm_oracle_fmm64
        f.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, ctypes.c_uint32, _f64p, _i64p]
        f.restype = ctypes.c_int
        r = self.lib.ghcm_oracle_residual
        r.argtypes = [_f32p, _f32p, ctypes.c_uint32, ctypes.c_uint32]
        r.restype = ctypes.c_double
        t = self.lib.ghcm_oracle_throughput
        t.argtypes = [ctypes.c_int, ctypes.c_float, _f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, ctypes.c_uint32,
                      ctypes.c_uint32, ctypes.c_uint32, _f32p]
        t.restype = ctypes.c_int64
        hc = self.lib.ghcm_oracle_hcm
        hc.argtypes = [ctypes.c_float, _f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                       ctypes.c_uint32, ctypes.c_uint32, _f32p, ctypes.POINTER(ctypes.c_uint64)]
        hc.restype = ctypes.c_int

    def hcm(self, cost, seeds, block: int = 8, max_jobs: int = 64, eps: float = 1e-5, wg: int = 64):
        """The reference gHCM schedule with its systolic kernel, on the CPU:
        returns (field, block_solves, waves)."""
        cost, seeds, w, h = _prep(cost, seeds)
        out = np.empty((h, w), dtype=np.float32)
        counts = (ctypes.c_uint64 * 2)()
        rc = self.lib.ghcm_oracle_hcm(eps, _ptr(cost, _f32p), w, h, _ptr(seeds, _u32p), len(seeds), block, max_jobs,
                                      wg, _ptr(out, _f32p), counts)
        if rc != 0:
            raise ValueError("hcm failed")
        return out, int(counts[0]), int(counts[1])

    def fmm64(self, cost, seeds):
        """FMM carried out in FP64: the accuracy oracle."""
        cost, seeds, w, h = _prep(cost, seeds)
        out = np.empty((h, w), dtype=np.float64)
        us = ctypes.c_int64(0)
        rc = self.lib.ghcm_oracle_fmm64(_ptr(cost, _f32p), w, h, _ptr(seeds, _u32p), len(seeds), _ptr(out, _f64p),
                                        ctypes.byref(us))
        if rc != 0:
            raise ValueError(f"fmm64 failed ({rc})")
        return out, us.value

    def residual(self, cost, time) -> float:
        """Largest fixed-point residual T - G(T) over cells of finite cost."""
        cost = np.ascontiguousarray(cost, dtype=np.float32)
        time = np.ascontiguousarray(time, dtype=np.float32)
        h, w = cost.shape
        return float(self.lib.ghcm_oracle_residual(_ptr(cost, _f32p), _ptr(time, _f32p), w, h))

    def throughput(self, kind: str, cost, seeds, count: int, threads: int, eps: float = 1e-5):
        """``count`` solves on ``threads`` host threads; returns (field, wall microseconds)."""
        cost, seeds, w, h = _prep(cost, seeds)
        out = np.empty((h, w), dtype=np.float32)
        us = self.lib.ghcm_oracle_throughput(0 if kind == "fmm" else 1, eps, _ptr(cost, _f32p), w, h,
                                             _ptr(seeds, _u32p), len(seeds), count, threads, _ptr(out, _f32p))
        if us < 0:
            raise ValueError("throughput run failed")
        return out, us


class Reference(_Lib):
    prefix = "ghcm_ref"

    def __init__(self, path: Path = REF_SO):
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (needs the reference sources)")
        super().__init__(path)


def reference_available() -> bool:
    return REF_SO.exists() or (REF_SRC / "eikonal_fim.cpp").exists()


def rel_diff(a: np.ndarray, b: np.ndarray) -> float:
    """Largest |a-b|/|b| over cells where b is finite and > 0, with the
    reference's conventions (src/eikonal.h:142-143, src/test_runner.cpp:154-165):
    inf == inf counts as 0 and a finite-vs-inf mismatch is an infinite error."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    if np.any(fa != fb):
        return float("inf")
    m = fb & (b > 0)
    if not np.any(m):
        return 0.0
    return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m])))
