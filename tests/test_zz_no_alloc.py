"""ghcm_solve_device_noalloc: the solve for callers that cannot allocate GPU
memory (a host whose pool owns every device allocation, a path that must not
synchronise the device as cudaMalloc/cudaFree can, a service whose footprint
must not grow). It keeps its scheduler scratch in a static device array and
creates no context, so this test calls it straight through the C ABI and
checks its field against the context-based ghcm_solve_device on the same
inputs, on two calls in a row (the second reuses the scratch the first left
behind), within the parity tolerance of the other GPU tests. The buffers are
the caller's: the test allocates them with torch, the entry point allocates
nothing.

This file is named to be collected last, so a failure here cannot hide other
failures in a run that stops at the first one; it also passes on its own in
a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from ghcm_gb300 import _lib, fields
from oracle.oracle import rel_diff

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the parity tolerance of the other GPU tests (max relative difference)


def _config(block=16, max_jobs=256):
    c = _lib.GhcmConfig()
    _lib.load().ghcm_config_default(ctypes.byref(c))
    c.block_size = block
    c.max_jobs = max_jobs
    return c


def _noalloc(lib, cfg, d_speed, d_seeds, d_time, stream):
    h, w = d_speed.shape
    return lib.ghcm_solve_device_noalloc(ctypes.byref(cfg), ctypes.c_void_p(d_speed.data_ptr()), 1, w, h, 1.0,
                                         ctypes.c_void_p(d_seeds.data_ptr()), d_seeds.shape[0],
                                         ctypes.c_void_p(d_time.data_ptr()), ctypes.c_void_p(stream.cuda_stream))


def _with_context(lib, cfg, d_speed, d_seeds, d_time, stream):
    h, w = d_speed.shape
    ctx = ctypes.c_void_p()
    assert lib.ghcm_create(ctypes.byref(cfg), ctypes.byref(ctx)) == 0
    try:
        return lib.ghcm_solve_device(ctx, ctypes.c_void_p(d_speed.data_ptr()), 1, w, h, 1.0,
                                     ctypes.c_void_p(d_seeds.data_ptr()), d_seeds.shape[0],
                                     ctypes.c_void_p(d_time.data_ptr()), ctypes.c_void_p(stream.cuda_stream), None)
    finally:
        lib.ghcm_destroy(ctx)


@pytest.mark.parametrize("block", [16, 8])
def test_noalloc_matches_context_entry_twice(cuda_ok, ghcm_lib, block):
    import torch

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    cfg = _config(block)
    cases = [fields.value_noise(384, seed=12, base_period=48.0, sources=4),
             fields.ring7_scaled(512, 3)]
    for speed, seeds in cases:
        d_speed = torch.from_numpy(speed).to(dev)
        d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
        ref = torch.empty_like(d_speed)
        assert _with_context(ghcm_lib, cfg, d_speed, d_seeds, ref, stream) == 0
        expected = ref.cpu().numpy()
        for _ in range(2):  # the second call starts from the scratch the first left
            out = torch.full_like(d_speed, -1.0)
            assert _noalloc(ghcm_lib, cfg, d_speed, d_seeds, out, stream) == 0
            stream.synchronize()
            got = out.cpu().numpy()
            assert np.array_equal(np.isfinite(got), np.isfinite(expected))
            assert rel_diff(got, expected) <= TOL
            assert np.all(got[seeds[:, 1], seeds[:, 0]] == 0.0)


def test_noalloc_rejects_oversized_tiling(cuda_ok, ghcm_lib):
    import torch

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    cfg = _config(8)
    # 4104 x 4096 cells at block 8 is 513 x 512 tiles, one row of tiles over the limit
    w, h = 4104, 4096
    assert ((w + 7) // 8) * ((h + 7) // 8) > _lib.GHCM_NOALLOC_MAX_TILES
    d_speed = torch.ones((h, w), device=dev)
    d_time = torch.empty_like(d_speed)
    d_seeds = torch.zeros((1, 2), dtype=torch.int32, device=dev)
    assert _noalloc(ghcm_lib, cfg, d_speed, d_seeds, d_time, stream) == _lib.GHCM_ERR_TOO_LARGE
    # and the next call in bounds still works
    small = torch.ones((64, 64), device=dev)
    out = torch.empty_like(small)
    assert _noalloc(ghcm_lib, cfg, small, d_seeds, out, stream) == 0
    stream.synchronize()
    assert out[0, 5].item() == 5.0 and out[5, 0].item() == 5.0
