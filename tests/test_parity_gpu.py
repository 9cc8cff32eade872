"""Parity of the CUDA solver (through the C ABI) with the reference's CPU FIM.

The bar (tolerance in every assert below): max relative difference <= 1e-5
against the reference FIM run to the same eps, with the reference's
comparison rules (inf == inf, finite vs inf fails, seeds exactly 0).
Golden fixtures were produced by the reference build itself; larger cases run
the CPU oracle (bit-exact to the reference) on the same inputs here.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import ghcm_gb300 as g
from conftest import golden_cases, load_golden
from ghcm_gb300 import _lib, fields
from oracle.oracle import rel_diff

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the parity bar: max relative difference vs the reference FIM


@pytest.fixture(scope="module")
def setups(cuda_ok, ghcm_lib):
    cache = {}

    def get(block=16, kernel=g.Kernel.Systolic, use_tma=True, max_jobs=64, **kw):
        key = (block, kernel, use_tma, max_jobs, tuple(sorted(kw.items())))
        if key not in cache:
            cache[key] = g.HcmSetup(g.HcmConfig(block_size=block, kernel=kernel, use_tma=use_tma, max_jobs=max_jobs,
                                                **kw))
        return cache[key]

    yield get
    for s in cache.values():
        s.close()


def check_field(out, ref, seeds, cost=None, tol=TOL):
    assert out.shape == ref.shape and out.dtype == np.float32
    assert np.array_equal(np.isfinite(out), np.isfinite(ref)), "reachability differs"
    err = rel_diff(out, ref)
    assert err <= tol, f"max relative difference {err:.3g} > {tol}"
    for x, y in np.asarray(seeds).reshape(-1, 2):
        assert out[y, x] == 0.0


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("block", [8, 16, 32])
@pytest.mark.parametrize("kernel", [g.Kernel.Systolic, g.Kernel.FIM])
@pytest.mark.parametrize("use_tma", [True, False])
def test_golden_fixtures(setups, name, block, kernel, use_tma):
    gd = load_golden(name)
    res = g.eikonal_hcm_cuda_ex(setups(block, kernel, use_tma), gd["cost"], gd["seeds"])
    check_field(res.field, gd["fim_1e5"], gd["seeds"])
    assert res.stats["block_solves"] >= (1 if np.isfinite(res.field).sum() > len(gd["seeds"]) else 0)


@pytest.mark.parametrize("name", golden_cases())
def test_golden_fixed_point(setups, oracle_lib, name):
    gd = load_golden(name)
    res = g.eikonal_hcm_cuda_ex(setups(), gd["cost"], gd["seeds"])
    # the device field is a fixed point of the update to within eps
    assert oracle_lib.residual(gd["cost"], res.field) <= 1e-5


@pytest.mark.parametrize("name", ["ring7_64", "noise_48x40", "ref_7_ring_256_2d"])
def test_golden_harness_eps(setups, name):
    """eps = 1e-3, the reference harness value (src/test_runner.cpp:17): both
    solvers stop within eps per update, so they agree to a few eps."""
    gd = load_golden(name)
    s = setups(16, fim_minimum_change=1e-3)
    res = g.eikonal_hcm_cuda_ex(s, gd["cost"], gd["seeds"])
    diff = np.abs(res.field.astype(np.float64) - gd["fim_1e3"])
    diff[~np.isfinite(gd["fim_1e3"])] = 0
    assert np.array_equal(np.isfinite(res.field), np.isfinite(gd["fim_1e3"]))
    assert float(diff.max()) <= 2e-2


CASES = {
    "ring7_1024": lambda: fields.ring7_scaled(1024, 1),
    "noise_1024": lambda: fields.value_noise(1024, seed=5, base_period=128.0, sources=16),
    "maze_768": lambda: fields.ca_maze(768, seed=3, sources=8),
    "noise_ragged_997x613": lambda: fields.value_noise(613, seed=9, base_period=64.0, sources=5, w=997),
}


@pytest.fixture(scope="module")
def medium(oracle_lib):
    out = {}
    for k, make in CASES.items():
        speed, seeds = make()
        cost = fields.cost_from_speed(speed)
        out[k] = (speed, cost, seeds, oracle_lib.fim(cost, seeds, 1e-5)[0])
    return out


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("block,kernel", [(8, g.Kernel.Systolic), (16, g.Kernel.Systolic), (32, g.Kernel.Systolic),
                                          (16, g.Kernel.FIM)])
def test_medium_vs_oracle(setups, medium, case, block, kernel):
    speed, cost, seeds, ref = medium[case]
    s = setups(block, kernel, max_jobs=1024)
    res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
    check_field(res.field, ref, seeds)


@pytest.mark.parametrize("max_jobs", [1, 3, 256, 100000])
@pytest.mark.parametrize("key_mode", [g.KeyMode.BoundaryMin, g.KeyMode.BlockMin])
def test_top_n_and_key_modes(setups, medium, max_jobs, key_mode):
    speed, cost, seeds, ref = medium["noise_1024"]
    res = g.eikonal_hcm_cuda_ex(setups(16, max_jobs=max_jobs, key_mode=key_mode), speed, seeds, input_is_speed=True)
    check_field(res.field, ref, seeds)
    if max_jobs < 4096:
        assert res.stats["waves"] * max_jobs >= res.stats["block_solves"]


def test_speed_and_cost_inputs_agree_with_spacing(setups):
    speed, seeds = fields.value_noise(200, seed=2, base_period=32.0, sources=3)
    h = 0.25
    cost = fields.cost_from_speed(speed, h=h)
    s = setups(16)
    a = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True, h=h).field
    b = g.eikonal_hcm_cuda_ex(s, cost, seeds).field
    check_field(a, b, seeds, tol=1e-6)


def test_eps_zero_reaches_exact_fixed_point(setups, oracle_lib):
    speed, seeds = fields.value_noise(300, seed=4, base_period=40.0, sources=4)
    cost = fields.cost_from_speed(speed)
    res = g.eikonal_hcm_cuda_ex(setups(16, fim_minimum_change=0.0), cost, seeds)
    assert oracle_lib.residual(cost, res.field) == 0.0
    check_field(res.field, oracle_lib.fim(cost, seeds, 0.0)[0], seeds)


@pytest.mark.parametrize("block", [16, 32])
def test_costs_outside_the_short_root_range(setups, oracle_lib, block):
    """Tiles whose costs leave [2^-49, 2^63) (here 0, 1e-18 times the noise
    costs and 1e19, where 2c^2 is still finite) sweep with the general square
    root, the others with its short form: at eps = 0 every cell is an exact
    fixed point of the reference update, and the field is within the bar of
    the reference FIM."""
    speed, seeds = fields.value_noise(300, seed=5, base_period=40.0, sources=4)
    cost = fields.cost_from_speed(speed)
    cost[0:64, 0:64] *= np.float32(1e-18)
    cost[100:164, 100:164] = 0.0
    cost[200:264, 16:80] = np.float32(1e19)
    res = g.eikonal_hcm_cuda_ex(setups(block, fim_minimum_change=0.0), cost, seeds)
    assert oracle_lib.residual(cost, res.field) == 0.0
    check_field(res.field, oracle_lib.fim(cost, seeds, 0.0)[0], seeds)


def test_workspace_reuse_across_sizes(setups, oracle_lib):
    s = setups(16)
    for n, w in ((300, 301), (40, 41), (520, 260), (17, 9)):
        speed, seeds = fields.value_noise(n, seed=n, base_period=16.0, sources=2, w=w)
        cost = fields.cost_from_speed(speed)
        res = g.eikonal_hcm_cuda_ex(s, cost, seeds)
        check_field(res.field, oracle_lib.fim(cost, seeds, 1e-5)[0], seeds)


def test_no_seeds_all_infinite(setups):
    res = g.eikonal_hcm_cuda_ex(setups(16), np.ones((33, 47), np.float32), np.zeros((0, 2), np.uint32))
    assert np.all(np.isinf(res.field)) and res.stats["block_solves"] == 0


def test_single_cell_field(setups):
    res = g.eikonal_hcm_cuda_ex(setups(8), np.ones((1, 1), np.float32), [[0, 0]])
    assert res.field.tolist() == [[0.0]]


def test_seed_on_impassable_cell(setups, oracle_lib):
    cost = np.ones((40, 40), np.float32)
    cost[10, 10] = np.inf
    seeds = np.array([[10, 10]], np.uint32)
    res = g.eikonal_hcm_cuda_ex(setups(16), cost, seeds)
    check_field(res.field, oracle_lib.fim(cost, seeds, 1e-5)[0], seeds)


def test_bad_inputs_are_rejected(setups):
    s = setups(16)
    speed = np.ones((20, 20), np.float32)
    for bad in (np.nan, -1.0):
        f = speed.copy()
        f[3, 4] = bad
        with pytest.raises(g.GhcmError) as e:
            g.eikonal_hcm_cuda_ex(s, f, [[0, 0]], input_is_speed=True)
        assert e.value.status == _lib.GHCM_ERR_BAD_INPUT
    with pytest.raises(g.GhcmError) as e:
        g.eikonal_hcm_cuda_ex(s, speed, [[20, 0]])
    assert e.value.status == _lib.GHCM_ERR_BAD_ARG
    with pytest.raises(g.GhcmError) as e:
        g.eikonal_hcm_cuda_ex(s, speed, [[0, 0]], h=0.0)
    assert e.value.status == _lib.GHCM_ERR_BAD_ARG
    # the context stays usable after rejected calls
    ok = g.eikonal_hcm_cuda_ex(s, speed, [[0, 0]])
    assert ok.field[0, 0] == 0.0 and ok.field[19, 19] > 0


def test_wave_cap_reports_not_converged(setups):
    speed, seeds = fields.ring7_scaled(512, 2)
    with pytest.raises(g.GhcmError) as e:
        g.eikonal_hcm_cuda_ex(setups(16, max_waves=3), speed, seeds, input_is_speed=True)
    assert e.value.status == _lib.GHCM_ERR_NOT_CONVERGED


def test_bounded_wait_times_out_cleanly(setups):
    s = setups(16)
    assert _lib.load().ghcm_selftest_wait_timeout(s.handle, 100) == _lib.GHCM_ERR_TIMEOUT
    res = g.eikonal_hcm_cuda_ex(s, np.ones((32, 32), np.float32), [[1, 1]])  # GPU still healthy
    assert res.field[1, 1] == 0.0 and np.isfinite(res.field).all()


def test_update_sqrt_is_ieee_for_every_float(setups):
    """The device update's square root (an FMA-corrected hardware estimate)
    gives the bits of CUDA's IEEE __fsqrt_rn for all 2^32 inputs, and so does
    its short form on [2^-100, +inf), which tiles of costs in [2^-49, 2^63)
    use."""
    import ctypes

    s = setups(16)
    bad = ctypes.c_ulonglong(123)
    assert _lib.load().ghcm_selftest_sqrt(s.handle, ctypes.byref(bad)) == _lib.GHCM_OK
    assert bad.value == 0


def test_device_entry_with_torch_tensors(setups, medium):
    import torch

    speed, cost, seeds, ref = medium["ring7_1024"]
    dev = torch.device("cuda", 0)
    d_speed = torch.from_numpy(speed).to(dev)
    d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    d_time = torch.empty_like(d_speed)
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        st = g.solve_device(setups(16, max_jobs=1024), d_speed, d_seeds, d_time, stream=stream)
    stream.synchronize()
    check_field(d_time.cpu().numpy(), ref, seeds)
    assert st["block_solves"] > 0 and st["device_ms"] > 0


def test_device_seed_out_of_range(setups):
    import torch

    dev = torch.device("cuda", 0)
    d_speed = torch.ones((16, 16), device=dev)
    d_time = torch.empty_like(d_speed)
    d_seeds = torch.tensor([[3, 99]], dtype=torch.int32, device=dev)
    with pytest.raises(g.GhcmError) as e:
        g.solve_device(setups(16), d_speed, d_seeds, d_time)
    assert e.value.status == _lib.GHCM_ERR_BAD_ARG


def test_misaligned_device_pointer_uses_plain_loads(setups, oracle_lib):
    import torch

    speed, seeds = fields.value_noise(64, seed=8, base_period=16.0, sources=2)
    dev = torch.device("cuda", 0)
    buf = torch.empty(64 * 64 + 1, device=dev)
    buf[1:] = torch.from_numpy(speed).to(dev).reshape(-1)
    d_speed = buf[1:].view(64, 64)  # 4-byte offset: not 16-byte aligned
    d_time = torch.empty((64, 64), device=dev)
    d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    g.solve_device(setups(16), d_speed, d_seeds, d_time)
    check_field(d_time.cpu().numpy(), oracle_lib.fim(fields.cost_from_speed(speed), seeds, 1e-5)[0], seeds)


def test_stats_are_consistent(setups, medium):
    speed, cost, seeds, ref = medium["ring7_1024"]
    res = g.eikonal_hcm_cuda_ex(setups(16, max_jobs=256), speed, seeds, input_is_speed=True)
    st = res.stats
    assert st["cells"] == 1024 * 1024 and st["tiles"] == 64 * 64
    assert st["bytes_alg"] == st["block_solves"] * (4 * 256 + 4 * (18 * 18 - 4) + 4 * 256)
    assert 0 < st["max_active"] <= st["tiles"] and st["waves"] > 0
    assert 0 < st["device_ms"] <= st["total_ms"]


def test_abi_call_directly(ghcm_lib, cuda_ok):
    """ghcm_solve through raw ctypes, as a C caller would use it."""
    c = _lib.GhcmConfig()
    ghcm_lib.ghcm_config_default(ctypes.byref(c))
    h = ctypes.c_void_p()
    assert ghcm_lib.ghcm_create(ctypes.byref(c), ctypes.byref(h)) == 0
    try:
        cost = np.ones((24, 24), np.float32)
        seeds = np.array([[0, 0]], np.uint32)
        out = np.empty_like(cost)
        st = _lib.GhcmStats()
        rc = ghcm_lib.ghcm_solve(h, cost.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 0, 24, 24, 1.0,
                                 seeds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), 1,
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(st))
        assert rc == 0
        assert out[0, 5] == 5.0 and out[5, 0] == 5.0 and st.block_solves > 0
    finally:
        ghcm_lib.ghcm_destroy(h)


@pytest.mark.parametrize("block", [8, 16, 32])
def test_permeable_cost_cap(setups, oracle_lib, block):
    """cost = min(cost, cap), the reference's field_cost_as_permeable
    (src/test_runner.cpp:70-75): speed-0 walls become passable at cost 1e3."""
    rng = np.random.default_rng(40 + block)
    speed = rng.uniform(0.3, 1.0, size=(150, 170)).astype(np.float32)
    speed[40:44, :150] = 0.0  # a wall with no gap on the left side
    speed[100:130, 60:64] = 0.0
    seeds = np.array([[20, 10], [160, 140]], dtype=np.uint32)
    capped = np.minimum(fields.cost_from_speed(speed), np.float32(1e3))
    ref = oracle_lib.fim(capped, seeds, 1e-5)[0]
    assert np.isfinite(ref).all()
    res = g.eikonal_hcm_cuda_ex(setups(block, cost_cap=1e3), speed, seeds, input_is_speed=True)
    check_field(res.field, ref, seeds)
    # the cost form of the input gives the same field
    res2 = g.eikonal_hcm_cuda_ex(setups(block, cost_cap=1e3), fields.cost_from_speed(speed), seeds)
    check_field(res2.field, ref, seeds)


@pytest.mark.parametrize("refresh", [_lib.GHCM_REFRESH_OFF, _lib.GHCM_REFRESH_IN_SOLVE, 1, 4, 15])
@pytest.mark.parametrize("block,kernel", [(8, g.Kernel.Systolic), (16, g.Kernel.Systolic), (16, g.Kernel.FIM),
                                          (32, g.Kernel.Systolic)])
def test_update_bounds_keep_parity(setups, medium, refresh, block, kernel):
    """Every way a sweep may bound the update (the reference's min(T_old, .),
    recompute up to the staged value, and 1-15 quiet solves that may raise
    cells) converges to the oracle's field within the bar on the medium cases."""
    for case in ("ring7_1024", "noise_1024"):
        speed, cost, seeds, ref = medium[case]
        res = g.eikonal_hcm_cuda_ex(setups(block, kernel, max_jobs=1024, refresh_solves=refresh), speed, seeds,
                                    input_is_speed=True)
        check_field(res.field, ref, seeds)


@pytest.mark.parametrize("mult", [1, 2])
@pytest.mark.parametrize("kernel", [g.Kernel.Systolic, g.Kernel.FIM])
@pytest.mark.parametrize("block", [8, 16])
def test_sweep_caps_terminate_with_parity(setups, medium, mult, kernel, block):
    """Inner-sweep caps at which most block-solves finish (twice and four
    times the tile side) re-queue the capped tiles; the solve still ends, within a wave bound that turns a
    non-terminating schedule into GHCM_ERR_NOT_CONVERGED instead of a hang,
    and keeps parity. Tighter caps leave most solves capped, each ending on a
    lower-only sweep, and drift further from the FIM (8 sweeps on 8 x 8 tiles
    measured 1.56e-5, 16 on 16 x 16 tiles 1.04e-5, on the 1024^2 rings);
    test_small_sweep_caps_terminate covers them."""
    cap = mult * 2 * block
    for case in ("ring7_1024", "noise_1024"):
        speed, cost, seeds, ref = medium[case]
        s = setups(block, kernel, max_jobs=1024, max_sweeps=cap, max_waves=200000)
        res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
        check_field(res.field, ref, seeds)


@pytest.mark.parametrize("cap", [1, 4])
@pytest.mark.parametrize("kernel", [g.Kernel.Systolic, g.Kernel.FIM])
@pytest.mark.parametrize("block", [8, 16])
def test_small_sweep_caps_terminate(setups, oracle_lib, medium, cap, kernel, block):
    """Caps of one sweep (every solve lower-only and re-queued until nothing
    moves) and of four still end at a fixed point, within the wave bound."""
    speed, cost, seeds, ref = medium["noise_1024"]
    s = setups(block, kernel, max_jobs=1024, max_sweeps=cap, max_waves=200000)
    res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
    assert np.array_equal(np.isfinite(res.field), np.isfinite(ref))
    assert oracle_lib.residual(cost, res.field) <= 1e-5
    assert rel_diff(res.field, ref) <= 1e-4
