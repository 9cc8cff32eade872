"""Batches (ghcm_batch_* / ghcm_solve_batched / ghcm_autotune_batch) on the GPU.

Each instance of a batch is one reference solve; the bar is the single-field
one (max relative difference <= 1e-5, same reachability, seeds exactly 0)
against (a) the reference FIM restatement (oracle) for instances small enough
to solve on the CPU in the test, and (b) a plain single-instance run of the
same field through ghcm_solve_device.
"""
from __future__ import annotations

import numpy as np
import pytest

import ghcm_gb300 as g
from ghcm_gb300 import _lib, fields
from oracle.oracle import rel_diff

pytestmark = pytest.mark.gpu

TOL = 1e-5  # max relative difference


def _to_device(insts, dev):
    import torch

    out = []
    for inst in insts:
        d_speed = torch.from_numpy(np.ascontiguousarray(inst.speed, dtype=np.float32)).to(dev)
        d_seeds = torch.from_numpy(np.ascontiguousarray(inst.seeds, dtype=np.int32).reshape(-1, 2)).to(dev)
        d_time = torch.full_like(d_speed, -1.0)
        out.append(g.DeviceInstance(d_speed, d_seeds, d_time))
    return out


def _mix(count, seed, side_max=256):
    insts = fields.batched_mix(count, seed, side_min=48, side_max=side_max)
    # two odd widths (rows not 16-byte aligned: staged with plain loads, no TMA)
    rng = np.random.default_rng(seed)
    for w, h in ((67, 45), (33, 90)):
        speed = rng.uniform(0.2, 1.0, size=(h, w)).astype(np.float32)
        insts.append(fields.Instance(speed, np.array([[w // 2, h // 3], [1, h - 2]], dtype=np.uint32), "odd"))
    return insts


def _check(got, ref, seeds):
    assert np.array_equal(np.isfinite(got), np.isfinite(ref)), "reachability differs"
    assert rel_diff(got, ref) <= TOL
    s = np.asarray(seeds).reshape(-1, 2)
    assert np.all(got[s[:, 1], s[:, 0]] == 0.0)


@pytest.fixture(scope="module")
def dev(cuda_ok, ghcm_lib):
    import torch

    return torch.device("cuda", 0)


@pytest.mark.parametrize("block", [8, 16, 32])
def test_batch_matches_oracle_and_single_runs(dev, oracle_lib, block):
    insts = _mix(20, seed=5)
    dinst = _to_device(insts, dev)
    with g.HcmSetup(g.HcmConfig(block_size=block, max_jobs=512)) as setup:
        with g.Batch(setup, dinst) as b:
            info = b.info()
            assert info["instances"] == len(insts) and info["graph"] == 1
            assert info["tma_instances"] == len(insts) - 2  # the two odd widths use plain loads
            st = b.run()
        assert st["cells"] == sum(i.speed.size for i in insts)
        assert st["block_solves"] >= st["tiles"]
        for k, (inst, di) in enumerate(zip(insts, dinst)):
            got = di.d_time.cpu().numpy()
            ref_single = di.d_time.clone()
            single = g.solve_device(setup, di.d_field, di.d_seeds, ref_single)
            _check(got, ref_single.cpu().numpy(), inst.seeds)
            assert single["cells"] == inst.speed.size
            if inst.speed.size <= 160 * 160 or k < 4:
                cost = fields.cost_from_speed(inst.speed)
                ref = oracle_lib.fim(cost, inst.seeds, 1e-5)[0]
                _check(got, ref, inst.seeds)


def test_batch_fim_kernel_and_block_min_key(dev, oracle_lib):
    insts = _mix(8, seed=9, side_max=160)
    dinst = _to_device(insts, dev)
    cfg = g.HcmConfig(block_size=16, kernel=g.Kernel.FIM, key_mode=g.KeyMode.BlockMin, max_jobs=64)
    with g.HcmSetup(cfg) as setup:
        g.solve_batched(setup, dinst)
    for inst, di in zip(insts, dinst):
        ref = oracle_lib.fim(fields.cost_from_speed(inst.speed), inst.seeds, 1e-5)[0]
        _check(di.d_time.cpu().numpy(), ref, inst.seeds)


def test_batch_replays_are_consistent_and_independent_of_order(dev):
    import torch

    insts = _mix(12, seed=3)
    dinst = _to_device(insts, dev)
    with g.HcmSetup(g.HcmConfig(block_size=16, max_jobs=256)) as setup:
        with g.Batch(setup, dinst) as b:
            b.run()
            first = [d.d_time.clone() for d in dinst]
            for d in dinst:
                d.d_time.fill_(-1.0)
            b.run()
            second = [d.d_time.clone() for d in dinst]
        # the same instances in reverse order, as another batch
        rev = list(reversed(dinst))
        for d in rev:
            d.d_time.fill_(-1.0)
        g.solve_batched(setup, rev)
    for a, b2, d in zip(first, second, dinst):
        a, b2, c = a.cpu().numpy(), b2.cpu().numpy(), d.d_time.cpu().numpy()
        assert rel_diff(b2, a) <= TOL and rel_diff(c, a) <= TOL
    torch.cuda.synchronize()


def test_batch_reports_bad_instances(dev):
    import torch

    insts = _to_device(_mix(4, seed=11, side_max=96), dev)
    with g.HcmSetup(g.HcmConfig(block_size=16)) as setup:
        # a seed outside its field
        bad = list(insts)
        w = bad[1].d_field.shape[1]
        bad[1] = g.DeviceInstance(bad[1].d_field, torch.tensor([[w + 3, 0]], dtype=torch.int32, device=dev),
                                  bad[1].d_time)
        with pytest.raises(g.GhcmError) as e:
            g.solve_batched(setup, bad)
        assert e.value.status == _lib.GHCM_ERR_BAD_ARG
        # a NaN speed
        nan_field = insts[2].d_field.clone()
        nan_field[3, 3] = float("nan")
        bad = list(insts)
        bad[2] = g.DeviceInstance(nan_field, insts[2].d_seeds, insts[2].d_time)
        with pytest.raises(g.GhcmError) as e:
            g.solve_batched(setup, bad)
        assert e.value.status == _lib.GHCM_ERR_BAD_INPUT
        # the context still works afterwards
        st = g.solve_batched(setup, insts)
        assert st["block_solves"] > 0


def test_autotuner_picks_a_working_config(dev, oracle_lib):
    insts = _mix(10, seed=21, side_max=192)
    dinst = _to_device(insts, dev)
    best, trials = g.autotune_batch(g.HcmConfig(block_size=16), dinst, reps=1)
    assert best.block_size in (8, 16, 32)
    assert len(trials) == 15
    assert all(t["status"] == 0 for t in trials)
    assert {t["kernel"] for t in trials} == {int(g.Kernel.Systolic), int(g.Kernel.FIM)}
    ok = [t for t in trials if t["block_size"] == best.block_size and t["max_jobs"] == best.max_jobs
          and t["max_sweeps"] == best.max_sweeps and t["kernel"] == int(best.kernel)]
    assert ok and ok[0]["ms"] == min(t["ms"] for t in trials)
    for inst, di in zip(insts, dinst):
        ref = oracle_lib.fim(fields.cost_from_speed(inst.speed), inst.seeds, 1e-5)[0]
        _check(di.d_time.cpu().numpy(), ref, inst.seeds)
