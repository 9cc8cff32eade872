"""The learned schedule on the GPU: the trace recorder, the hand-written MLP
kernels against a plain PyTorch fp32 reference, and learned-schedule solves.

Tolerances (in each assert): MLP probabilities within 1e-5 absolute of torch
fp32; summed gradients within 1e-4 of the largest gradient component; one
Adam step within 1e-6 where the gradient is not negligible; solved fields
within 1e-5 max relative difference of the reference FIM (the parity bar of
every solve).
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import ghcm_gb300 as g
from ghcm_gb300 import _lib, fields, learned
from oracle.oracle import rel_diff

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def dev(cuda_ok, ghcm_lib):
    import torch

    return torch.device("cuda", 0)


def _noise(n, seed, sources=4):
    return fields.value_noise(n, seed=seed, base_period=n / 4.0, sources=sources)


def _torch_mlp(p, x):
    import torch

    u = {k: torch.from_numpy(v.copy()).to(x.device).requires_grad_(True) for k, v in learned.unpack(p).items()}
    h1 = torch.relu(x @ u["W1"] + u["b1"])
    h2 = torch.relu(h1 @ u["W2"] + u["b2"])
    return h2 @ u["W3"] + u["b3"][0], u


def _flat_grad(u):
    import torch

    return torch.cat([u[k].grad.reshape(-1) for k in ("W1", "b1", "W2", "b2", "W3", "b3")]).cpu().numpy()


def test_trace_records_every_block_solve(dev, oracle_lib):
    speed, seeds = _noise(256, 4)
    cost = fields.cost_from_speed(speed)
    ref = oracle_lib.fim(cost, seeds, 1e-5)[0]
    for block, kernel in ((16, g.Kernel.Systolic), (8, g.Kernel.Systolic), (16, g.Kernel.FIM)):
        with g.HcmSetup(g.HcmConfig(block_size=block, kernel=kernel, max_jobs=64)) as s:
            learned.enable_trace(s, 1 << 16)
            res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
            tr = learned.read_trace(s)
            assert rel_diff(res.field, ref) <= TOL
            assert tr.total == res.stats["block_solves"] == len(tr)
            tiles = res.stats["tiles"]
            assert tr.tile.max() < tiles and len(np.unique(tr.tile)) == tiles  # every tile solved
            assert np.all(np.isfinite(tr.features)) and np.all(np.abs(tr.features) <= 2.0)
            assert tr.wave.min() >= 1 and tr.wave.max() <= res.stats["waves"]
            assert np.all(tr.sweeps >= 1)
            # a tile's first solve: never solved before, and it always moves cells (from +inf)
            first = np.unique(tr.tile, return_index=True)[1]
            assert np.all(tr.features[first, 2] == 1.0) and np.all(tr.useful[first] == 1)
            assert np.all(tr.features[first, 9] == 0.0)  # no solves so far
            later = np.setdiff1d(np.arange(len(tr)), first)
            assert np.all(tr.features[later, 2] == 0.0)
            # overflow: capacity 10 keeps the first 10, counts them all
            learned.enable_trace(s, 10)
            g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
            small = learned.read_trace(s)
            assert len(small) == 10 and small.total > 10


def test_forward_kernel_matches_torch(dev):
    import torch

    rng = np.random.default_rng(0)
    p = learned.init_params(5, prior=0.3)
    x = rng.uniform(-1.5, 1.5, size=(1000, 12)).astype(np.float32)
    got = learned.predict(p, x)
    z, _ = _torch_mlp(p, torch.from_numpy(x).to(dev))
    want = torch.sigmoid(z).detach().cpu().numpy()
    assert np.max(np.abs(got - want)) <= 1e-5
    assert np.max(np.abs(got - learned.forward_numpy(p, x))) <= 1e-5


def test_grad_kernel_matches_torch_autograd(dev):
    import torch
    import torch.nn.functional as F

    rng = np.random.default_rng(1)
    p = learned.init_params(2)
    n = 300  # not a multiple of the 64-sample CTA
    x = rng.uniform(-1, 1, size=(n, 12)).astype(np.float32)
    y = (rng.random(n) < 0.6).astype(np.float32)
    dp, dx, dy = (torch.from_numpy(a).to(dev) for a in (p, x, y))
    grad = torch.zeros(learned.N_PARAMS, dtype=torch.float32, device=dev)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    rc = _lib.load().ghcm_mlp_grad(ctypes.c_void_p(dp.data_ptr()), ctypes.c_void_p(dx.data_ptr()),
                                   ctypes.c_void_p(dy.data_ptr()), n, 2.0, ctypes.c_void_p(grad.data_ptr()),
                                   ctypes.c_void_p(loss.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    z, u = _torch_mlp(p, dx)
    ref_loss = F.binary_cross_entropy_with_logits(z, dy, pos_weight=torch.tensor(2.0, device=dev), reduction="sum")
    ref_loss.backward()
    want = _flat_grad(u)
    got = grad.cpu().numpy()
    assert abs(loss.item() - ref_loss.item()) <= 1e-4 * abs(ref_loss.item())
    assert np.max(np.abs(got - want)) <= 1e-4 * np.max(np.abs(want))


def test_adam_step_matches_torch(dev):
    import torch
    import torch.nn.functional as F

    rng = np.random.default_rng(3)
    p = learned.init_params(4)
    n = 256
    x = rng.uniform(-1, 1, size=(n, 12)).astype(np.float32)
    y = (rng.random(n) < 0.5).astype(np.float32)
    dp, dx, dy = (torch.from_numpy(a).to(dev) for a in (p.copy(), x, y))
    cfg = _lib.GhcmTrainConfig()
    lib = _lib.load()
    lib.ghcm_train_config_default(ctypes.byref(cfg))
    cfg.epochs, cfg.batch, cfg.lr = 1, n, 1e-3
    losses = (ctypes.c_float * 1)()
    assert lib.ghcm_mlp_train(ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dy.data_ptr()), n,
                              ctypes.c_void_p(dp.data_ptr()), ctypes.byref(cfg), None, losses) == 0
    z, u = _torch_mlp(p, dx)
    loss = F.binary_cross_entropy_with_logits(z, dy, reduction="mean")
    opt = torch.optim.Adam([u[k] for k in ("W1", "b1", "W2", "b2", "W3", "b3")], lr=1e-3, eps=1e-8)
    loss.backward()
    g0 = _flat_grad(u)
    opt.step()
    want = torch.cat([u[k].detach().reshape(-1) for k in ("W1", "b1", "W2", "b2", "W3", "b3")]).cpu().numpy()
    got = dp.cpu().numpy()
    clear = np.abs(g0) > 1e-5  # Adam's first step is lr * sign(g): compare where the sign is not noise
    assert clear.sum() > 1000
    assert np.max(np.abs(got - want)[clear]) <= 1e-6
    assert abs(losses[0] - loss.item()) <= 1e-5


def test_training_separates_a_simple_rule(dev):
    rng = np.random.default_rng(9)
    x = rng.uniform(-1, 1, size=(20000, 12)).astype(np.float32)
    y = ((x[:, 0] + 0.5 * x[:, 3] - 0.3 * x[:, 7]) > 0.1).astype(np.float32)
    params, losses = learned.train(x, y, epochs=15, batch=512, lr=3e-3)
    assert losses[-1] < 0.5 * losses[0]
    acc = np.mean((learned.predict(params, x) >= 0.5) == (y > 0.5))
    assert acc > 0.95


@pytest.fixture(scope="module")
def trained(dev):
    """A model trained on the traces of two small noise fields."""
    traces = []
    with g.HcmSetup(g.HcmConfig(block_size=16, max_jobs=64)) as s:
        learned.enable_trace(s, 1 << 18)
        for seed in (11, 12):
            speed, seeds = _noise(256, seed)
            g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
            traces.append(learned.read_trace(s))
    tr = learned.Trace.concat(traces)
    params, _ = learned.train(tr.features, tr.useful, epochs=5, batch=1024)
    return params


@pytest.mark.parametrize("policy", [learned.POLICY_VETO, learned.POLICY_SCORE])
@pytest.mark.parametrize("block", [16, 8, 32])
def test_learned_schedule_keeps_parity(dev, oracle_lib, trained, block, policy):
    speed, seeds = _noise(256, 13)
    ref = oracle_lib.fim(fields.cost_from_speed(speed), seeds, 1e-5)[0]
    with g.HcmSetup(g.HcmConfig(block_size=block, max_jobs=64, fallback_jobs=16, schedule=g.Schedule.Learned)) as s:
        with pytest.raises(g.GhcmError) as e:  # no model yet
            g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
        assert e.value.status == _lib.GHCM_ERR_BAD_ARG
        learned.set_model(s, trained, threshold=0.5)
        learned.set_policy(s, policy)
        res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
        c = learned.counters(s)
    assert rel_diff(res.field, ref) <= TOL and np.all(res.field[seeds[:, 1], seeds[:, 0]] == 0.0)
    if policy == learned.POLICY_SCORE:
        assert c["score_waves"] + c["fallback_waves"] == res.stats["waves"] and c["vetoes"] == 0
        if block != 8:  # one warp per tile at block 8 queues tiles unscored: those waves go by key
            assert c["score_waves"] > c["fallback_waves"]
    else:
        assert c["score_waves"] == 0 and c["fallback_waves"] == 0


@pytest.mark.parametrize("policy", [learned.POLICY_VETO, learned.POLICY_SCORE])
@pytest.mark.parametrize("bias", [-60.0, 60.0])
def test_extreme_models(dev, oracle_lib, bias, policy):
    """A constant score of ~0 or ~1: the schedule still converges to the same
    field; a score of ~0 defers every claim max_vetoes times (veto) or leaves
    every wave to the plain fill (score); ~1 defers nothing."""
    speed, seeds = _noise(192, 14)
    ref = oracle_lib.fim(fields.cost_from_speed(speed), seeds, 1e-5)[0]
    p = np.zeros(learned.N_PARAMS, dtype=np.float32)
    learned.unpack(p)["b3"][:] = bias
    with g.HcmSetup(g.HcmConfig(block_size=16, max_jobs=32, fallback_jobs=8, schedule=g.Schedule.Learned)) as s:
        learned.set_model(s, p, threshold=0.5)
        learned.set_policy(s, policy, max_vetoes=2)
        res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
        c = learned.counters(s)
    assert rel_diff(res.field, ref) <= TOL
    if policy == learned.POLICY_VETO:
        if bias < 0:  # every claim not re-queued in full is deferred twice before it is solved
            assert c["vetoes"] >= res.stats["block_solves"] // 2
        else:
            assert c["vetoes"] == 0
    elif bias < 0:  # nothing qualifies: every wave is filled in key order
        assert c["fallback_waves"] > 0
    else:  # every scored tile qualifies; only the first wave (the seeds', queued unscored) goes by key
        assert c["fallback_waves"] <= 2 and c["score_waves"] > c["fallback_waves"]


def test_learned_batch(dev, oracle_lib, trained):
    import torch

    insts = fields.batched_mix(6, seed=31, side_min=48, side_max=160)
    dinst = []
    for inst in insts:
        d = torch.from_numpy(inst.speed).to(dev)
        dinst.append(g.DeviceInstance(d, torch.from_numpy(inst.seeds.astype(np.int32)).to(dev), torch.empty_like(d)))
    for policy in (learned.POLICY_VETO, learned.POLICY_SCORE):
        with g.HcmSetup(g.HcmConfig(block_size=16, max_jobs=128, schedule=g.Schedule.Learned)) as s:
            learned.set_model(s, trained, threshold=0.5)
            learned.set_policy(s, policy)
            for di in dinst:
                di.d_time.fill_(-1.0)
            g.solve_batched(s, dinst)
        for inst, di in zip(insts, dinst):
            ref = oracle_lib.fim(fields.cost_from_speed(inst.speed), inst.seeds, 1e-5)[0]
            assert rel_diff(di.d_time.cpu().numpy(), ref) <= TOL
