"""Batches of independent eikonal instances over the C ABI (ghcm_batch_* in
include/ghcm.h), the batch autotuner, and the split of a batch over ranks.

The reference solves one field per call (eikonal_hcm_opencl_ex,
src/eikonal_hcm.cpp:186-529) and its harness loops over trials
(src/test_runner.cpp:226-291). A batch puts the tiles of many instances
under one device scheduler and one persistent launch, replayed from a CUDA
graph:

    insts = [DeviceInstance(d_speed, d_seeds, d_time), ...]   # torch CUDA tensors
    with Batch(setup, insts) as b:
        stats = b.run()            # every d_time now holds its arrival times

Several GPUs: instances are independent, so a batch splits by instance with no
collective on the data path (``shard_instances``: greedy longest-processing-
time on cell counts); ``solve_sharded`` runs one rank's share and gathers the
per-instance results on rank 0 over torch.distributed (host objects).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Callable, Sequence

from . import _lib
from ._lib import GhcmError, GhcmStats
from .eikonal import HcmConfig, HcmSetup, Kernel


@dataclass
class DeviceInstance:
    """One instance of a batch: float32 [H, W] field and time tensors and an
    int32/uint32 [n, 2] (x, y) seed tensor, all contiguous on one GPU."""
    d_field: object
    d_seeds: object
    d_time: object
    h: float = 1.0
    input_is_speed: bool = True

    def to_c(self) -> _lib.GhcmInstance:
        import torch

        f, s, t = self.d_field, self.d_seeds, self.d_time
        if f.dtype != torch.float32 or t.dtype != torch.float32:
            raise TypeError("field and time must be float32")
        if not (f.is_cuda and s.is_cuda and t.is_cuda):
            raise TypeError("tensors must be on the GPU")
        if not (f.is_contiguous() and s.is_contiguous() and t.is_contiguous()):
            raise ValueError("tensors must be contiguous")
        if s.element_size() != 4 or (s.numel() and s.shape[-1] != 2):
            raise TypeError("seeds must be 32-bit (x, y) pairs")
        height, width = f.shape
        if tuple(t.shape) != (height, width):
            raise ValueError("time must match the field's shape")
        c = _lib.GhcmInstance()
        c.field = f.data_ptr()
        c.time_out = t.data_ptr()
        c.seeds_xy = s.data_ptr() if s.numel() else None
        c.n_seeds = s.shape[0] if s.numel() else 0
        c.width = width
        c.height = height
        c.h = float(self.h)
        c.input_is_speed = 1 if self.input_is_speed else 0
        c.reserved = 0
        return c


def _c_array(instances: Sequence[DeviceInstance]):
    arr = (_lib.GhcmInstance * len(instances))()
    for i, inst in enumerate(instances):
        arr[i] = inst.to_c()
    return arr


def _stream_handle(stream, device):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream(device)
    return ctypes.c_void_p(s.cuda_stream)


class Batch:
    """A batch bound to a context: workspace and CUDA graph made once, then
    ``run`` replays it. Keeps references to the instances' tensors."""

    def __init__(self, setup: HcmSetup, instances: Sequence[DeviceInstance]):
        if not instances:
            raise ValueError("a batch needs at least one instance")
        self.instances = list(instances)
        self._arr = _c_array(self.instances)
        self.device = self.instances[0].d_field.device
        handle = ctypes.c_void_p()
        rc = _lib.load().ghcm_batch_create(setup.handle, self._arr, len(self.instances), ctypes.byref(handle))
        if rc != 0:
            raise GhcmError(rc, "ghcm_batch_create")
        self.handle = handle

    def run(self, stream=None) -> dict:
        st = GhcmStats()
        rc = _lib.load().ghcm_batch_run(self.handle, _stream_handle(stream, self.device), ctypes.byref(st))
        if rc != 0:
            raise GhcmError(rc, "ghcm_batch_run")
        return st.as_dict()

    def info(self) -> dict:
        inf = _lib.GhcmBatchInfo()
        rc = _lib.load().ghcm_batch_query(self.handle, ctypes.byref(inf))
        if rc != 0:
            raise GhcmError(rc, "ghcm_batch_query")
        return inf.as_dict()

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.load().ghcm_batch_destroy(self.handle)
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


def solve_batched(setup: HcmSetup, instances: Sequence[DeviceInstance], stream=None) -> dict:
    """One solve of every instance (create + run + destroy)."""
    arr = _c_array(instances)
    st = GhcmStats()
    rc = _lib.load().ghcm_solve_batched(setup.handle, arr, len(instances),
                                        _stream_handle(stream, instances[0].d_field.device), ctypes.byref(st))
    if rc != 0:
        raise GhcmError(rc, "ghcm_solve_batched")
    return st.as_dict()


def autotune_batch(config: HcmConfig, instances: Sequence[DeviceInstance], stream=None, reps: int = 2):
    """Times the batch under tile sizes 8/16/32, n, inner-sweep caps and both
    tile kernels (ghcm_autotune_batch) and returns (best HcmConfig, list of
    trial dicts).
    The instances' time tensors hold a converged solve afterwards."""
    base = config.to_c()
    best = _lib.GhcmConfig()
    trials = (_lib.GhcmTuneTrial * 64)()
    n = ctypes.c_uint32()
    arr = _c_array(instances)
    rc = _lib.load().ghcm_autotune_batch(ctypes.byref(base), arr, len(instances),
                                         _stream_handle(stream, instances[0].d_field.device), int(reps),
                                         ctypes.byref(best), trials, 64, ctypes.byref(n))
    if rc != 0:
        raise GhcmError(rc, "ghcm_autotune_batch")
    tuned = HcmConfig(**{**config.__dict__})
    tuned.block_size = int(best.block_size)
    tuned.max_jobs = int(best.max_jobs)
    tuned.max_sweeps = int(best.max_sweeps)
    tuned.kernel = Kernel(int(best.kernel))
    return tuned, [trials[i].as_dict() for i in range(min(n.value, 64))]


def shard_instances(cells: Sequence[int], world_size: int) -> list[list[int]]:
    """Splits instance indices over ranks, balancing total cells: largest
    first, each to the rank with the fewest cells so far (ties to the lower
    rank). Deterministic, so every rank computes the same split."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(cells)), key=lambda i: (-int(cells[i]), i))
    load = [0] * world_size
    shards: list[list[int]] = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += int(cells[i])
    for s in shards:
        s.sort()
    return shards


def solve_sharded(cells: Sequence[int], solve: Callable[[list[int]], dict], rank: int, world_size: int,
                  group=None) -> dict | None:
    """Runs this rank's share of a batch and gathers the results on rank 0.

    ``solve(indices)`` solves the given instances on this rank's GPU and
    returns {index: result}; the gather is host-side (torch.distributed
    gather_object), so no collective touches the data path. Returns the
    merged {index: result} on rank 0 and None elsewhere."""
    import torch.distributed as dist

    mine = shard_instances(cells, world_size)[rank]
    local = solve(mine)
    if world_size == 1:
        return dict(local)
    gathered = [None] * world_size if rank == 0 else None
    dist.gather_object(local, gathered, dst=0, group=group)
    if rank != 0:
        return None
    merged: dict = {}
    for part in gathered:
        merged.update(part)
    return merged
