"""Python mirror of the reference's solver interface (src/eikonal.h:12-67) over
the C ABI of libghcm.so.

    HcmConfig               <- HcmConfig                  (src/eikonal.h:12-27)
    EikonalResult           <- EikonalResult              (src/eikonal.h:31-36)
    eikonal_hcm_cuda_setup  <- eikonal_hcm_opencl_setup   (src/eikonal_hcm.cpp:137-175)
    eikonal_hcm_cuda_ex     <- eikonal_hcm_opencl_ex      (src/eikonal_hcm.cpp:186-529)
    eikonal_hcm_cuda        <- eikonal_hcm_opencl         (src/eikonal_hcm.cpp:177-184)

Fields are 2-D arrays indexed ``[y, x]`` (row-major, x fastest, as Field2D);
the field passed in is a COST field (h / speed) as in the reference, unless
``input_is_speed`` is set. Seeds are (x, y) pairs. Errors raise GhcmError
instead of exiting the process (src/eikonal_hcm.cpp:181-182).
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field as dc_field
from enum import IntEnum

import numpy as np

from . import _lib
from ._lib import GhcmConfig, GhcmError, GhcmStats


class Kernel(IntEnum):
    Systolic = _lib.GHCM_KERNEL_SYSTOLIC
    FIM = _lib.GHCM_KERNEL_FIM


class CacheMode(IntEnum):
    """Accepted for interface parity. Tiles and their halo are always staged in
    shared memory, so every mode behaves as ``Both``."""
    None_ = 0
    Time = 1
    Cost = 2
    Both = 3


class Schedule(IntEnum):
    Plain = _lib.GHCM_SCHEDULE_PLAIN
    Learned = _lib.GHCM_SCHEDULE_LEARNED


class KeyMode(IntEnum):
    BoundaryMin = _lib.GHCM_KEY_BOUNDARY_MIN
    BlockMin = _lib.GHCM_KEY_BLOCK_MIN


@dataclass
class HcmConfig:
    """Solver knobs; the first six fields are the reference's, with its defaults."""
    block_size: int = 8
    workers_overload: float = 1.0          # CTA size follows the tile size; kept for parity
    compute_unit_overload: float = 1.0     # n = max(1, compute_unit_overload * SM count)
    fim_minimum_change: float = 1e-5
    cache_mode: CacheMode = CacheMode.Both
    kernel: Kernel = Kernel.Systolic
    # GB300 additions
    max_jobs: int = 0                      # explicit n; overrides compute_unit_overload when > 0
    schedule: Schedule = Schedule.Plain
    key_mode: KeyMode = KeyMode.BoundaryMin
    max_sweeps: int = 0
    max_waves: int = 0
    wait_timeout_ms: int = 2000
    use_tma: bool = True
    device: int = -1
    fallback_jobs: int = 0                 # learned schedule: n of a wave in which no tile qualifies
    cost_cap: float = 0.0                  # > 0: cost = min(cost, cost_cap) (field_cost_as_permeable)
    refresh_solves: int = 0                # quiet solves per tile that may raise cells (0 = 1; _lib.GHCM_REFRESH_*)

    def to_c(self, sm_count: int | None = None) -> GhcmConfig:
        c = GhcmConfig()
        _lib.load().ghcm_config_default(ctypes.byref(c))
        c.block_size = int(self.block_size)
        if self.max_jobs > 0:
            c.max_jobs = int(self.max_jobs)
        elif sm_count is not None:
            c.max_jobs = max(1, int(self.compute_unit_overload * sm_count))
        c.eps = float(self.fim_minimum_change)
        c.kernel = int(self.kernel)
        c.schedule = int(self.schedule)
        c.key_mode = int(self.key_mode)
        c.max_sweeps = int(self.max_sweeps)
        c.max_waves = int(self.max_waves)
        c.wait_timeout_ms = int(self.wait_timeout_ms)
        c.device = int(self.device)
        c.use_tma = 1 if self.use_tma else 0
        c.fallback_jobs = int(self.fallback_jobs)
        c.cost_cap = float(self.cost_cap)
        c.refresh_solves = int(self.refresh_solves)
        return c


@dataclass
class EikonalResult:
    field: np.ndarray
    duration_total: float   # microseconds, host wall time of the call
    duration_device: float  # microseconds, device time of the solve
    stats: dict = dc_field(default_factory=dict)


class HcmSetup:
    """An open solver context (the reference's HcmSetup). Close it, or use it
    as a context manager, to release its device memory."""

    def __init__(self, config: HcmConfig):
        self.config = config
        lib = _lib.load()
        probe = config.to_c()
        handle = ctypes.c_void_p()
        rc = lib.ghcm_create(ctypes.byref(probe), ctypes.byref(handle))
        if rc != 0:
            raise GhcmError(rc, "ghcm_create")
        sms = ctypes.c_uint32(0)
        lib.ghcm_device_sm_count(handle, ctypes.byref(sms))
        self.sm_count = int(sms.value)
        final = config.to_c(self.sm_count)
        if final.max_jobs != probe.max_jobs:
            lib.ghcm_destroy(handle)
            handle = ctypes.c_void_p()
            rc = lib.ghcm_create(ctypes.byref(final), ctypes.byref(handle))
            if rc != 0:
                raise GhcmError(rc, "ghcm_create")
        self.c_config = final
        self.handle = handle

    def close(self) -> None:
        if self.handle:
            _lib.load().ghcm_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def eikonal_hcm_cuda_setup(config: HcmConfig) -> HcmSetup | None:
    """Opens a context; returns None when the device or config is unusable
    (the reference returns an empty optional, src/eikonal_hcm.cpp:161-174)."""
    try:
        return HcmSetup(config)
    except (GhcmError, FileNotFoundError, OSError):
        return None


def _seeds(seed_points) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(seed_points, dtype=np.uint32).reshape(-1, 2))


def eikonal_hcm_cuda_ex(info: HcmSetup, field_cost: np.ndarray, seed_points, *, input_is_speed: bool = False,
                        h: float = 1.0, out: np.ndarray | None = None) -> EikonalResult:
    """Solves with host arrays (copies in and out are part of the call).
    `out`, when given, is a C-contiguous float32 array of the field's shape
    (pinned memory makes the copies faster) that receives the times."""
    f = np.ascontiguousarray(field_cost, dtype=np.float32)
    if f.ndim != 2:
        raise ValueError("field must be 2-D [y, x]")
    height, width = f.shape
    seeds = _seeds(seed_points)
    if out is None:
        out = np.empty_like(f)
    elif out.shape != f.shape or out.dtype != np.float32 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float32 array of the field's shape")
    st = GhcmStats()
    t0 = time.perf_counter()
    rc = _lib.load().ghcm_solve(info.handle, f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), int(input_is_speed),
                                width, height, float(h), seeds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                len(seeds), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(st))
    t1 = time.perf_counter()
    if rc != 0:
        raise GhcmError(rc, "ghcm_solve")
    return EikonalResult(out, (t1 - t0) * 1e6, st.device_ms * 1e3, st.as_dict())


def eikonal_hcm_cuda(config: HcmConfig, field_cost: np.ndarray, seed_points, **kw) -> EikonalResult:
    """One-shot setup + solve (the reference's eikonal_hcm_opencl)."""
    with HcmSetup(config) as info:
        return eikonal_hcm_cuda_ex(info, field_cost, seed_points, **kw)


def solve_device(info: HcmSetup, d_field, d_seeds, d_time, *, input_is_speed: bool = True, h: float = 1.0,
                 stream=None) -> dict:
    """Solves with device-resident torch tensors (float32 [H, W] field and
    time, uint32/int32 [n, 2] seeds) on ``stream`` (a torch.cuda.Stream or
    None for the current stream). Returns the solver statistics."""
    import torch

    if d_field.dtype != torch.float32 or d_time.dtype != torch.float32:
        raise TypeError("field and time must be float32")
    if not (d_field.is_cuda and d_time.is_cuda and d_seeds.is_cuda):
        raise TypeError("tensors must be on the GPU")
    if not (d_field.is_contiguous() and d_time.is_contiguous() and d_seeds.is_contiguous()):
        raise ValueError("tensors must be contiguous")
    if d_seeds.element_size() != 4:
        raise TypeError("seeds must be 32-bit")
    height, width = d_field.shape
    if tuple(d_time.shape) != (height, width):
        raise ValueError("time must match the field's shape")
    s = stream if stream is not None else torch.cuda.current_stream(d_field.device)
    st = GhcmStats()
    rc = _lib.load().ghcm_solve_device(info.handle, ctypes.c_void_p(d_field.data_ptr()), int(input_is_speed), width,
                                       height, float(h), ctypes.c_void_p(d_seeds.data_ptr()), d_seeds.shape[0],
                                       ctypes.c_void_p(d_time.data_ptr()), ctypes.c_void_p(s.cuda_stream),
                                       ctypes.byref(st))
    if rc != 0:
        raise GhcmError(rc, "ghcm_solve_device")
    return st.as_dict()
