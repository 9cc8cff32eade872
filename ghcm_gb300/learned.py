"""Learned block schedule: traces, the schedule MLP, training and use.

The reference orders block-solves by a min-time priority queue only
(src/eikonal_hcm.cpp:47-80, 344-358). Here the plain device solver records a
trace of its block-solves - the 12 features the scheduler saw for the tile and
whether the solve moved some cell by more than eps - and a 12 -> 64 -> 64 -> 1
FP32 MLP trained on those traces by the library's own CUDA kernels
(ghcm_mlp_train) scores the active tiles of a learned-schedule solve
(HcmConfig(schedule=Schedule.Learned)); see include/ghcm.h for the features
and the flat parameter layout this module mirrors.

    with HcmSetup(HcmConfig(block_size=16)) as plain:
        enable_trace(plain, 1 << 22)
        eikonal_hcm_cuda_ex(plain, speed, seeds, input_is_speed=True)
        tr = read_trace(plain)
    params, losses = train(tr.features, tr.useful)
    with HcmSetup(HcmConfig(block_size=16, schedule=Schedule.Learned)) as s:
        set_model(s, params, threshold=0.5)
        res = eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)

Device memory for training is held in torch tensors (plumbing); the
arithmetic runs in libghcm.so.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import GhcmError

FEATURES = 12
HIDDEN = 64
N_PARAMS = _lib.GHCM_MLP_PARAMS
FEATURE_NAMES = (
    "key_in_wave_range", "activation_key_spread", "never_solved", "tmin_above_key",
    "log2_min_speed", "log2_max_speed", "log2_mean_speed", "active_neighbours",
    "waves_since_useful", "log2_solves", "requeued_full", "new_edges",
)

# offsets of the flat parameter vector (W1 and W2 input-major)
OFF_W1 = 0
OFF_B1 = OFF_W1 + FEATURES * HIDDEN
OFF_W2 = OFF_B1 + HIDDEN
OFF_B2 = OFF_W2 + HIDDEN * HIDDEN
OFF_W3 = OFF_B2 + HIDDEN
OFF_B3 = OFF_W3 + HIDDEN
assert OFF_B3 + 1 == N_PARAMS


def unpack(params: np.ndarray) -> dict:
    """Views of the flat parameter vector: W1 [12, 64], b1, W2 [64, 64]
    (input-major: h2 = relu(h1 @ W2 + b2)), b2, W3 [64], b3."""
    p = np.asarray(params, dtype=np.float32).reshape(-1)
    if p.size != N_PARAMS:
        raise ValueError(f"expected {N_PARAMS} parameters, got {p.size}")
    return {
        "W1": p[OFF_W1:OFF_B1].reshape(FEATURES, HIDDEN),
        "b1": p[OFF_B1:OFF_W2],
        "W2": p[OFF_W2:OFF_B2].reshape(HIDDEN, HIDDEN),
        "b2": p[OFF_B2:OFF_W3],
        "W3": p[OFF_W3:OFF_B3],
        "b3": p[OFF_B3:],
    }


def init_params(seed: int = 0, prior: float = 0.5) -> np.ndarray:
    """He-uniform hidden weights, small output weights, zero biases and an
    output bias at the logit of `prior`."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, dtype=np.float32)
    u = unpack(p)
    u["W1"][:] = rng.uniform(-1, 1, size=(FEATURES, HIDDEN)) * np.sqrt(6.0 / FEATURES)
    u["W2"][:] = rng.uniform(-1, 1, size=(HIDDEN, HIDDEN)) * np.sqrt(6.0 / HIDDEN)
    u["W3"][:] = rng.uniform(-1, 1, size=HIDDEN) * np.sqrt(1.0 / HIDDEN)
    u["b3"][:] = np.log(prior / (1.0 - prior))
    return p


def forward_numpy(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Probabilities of the MLP in float64 numpy (a host reference)."""
    u = {k: v.astype(np.float64) for k, v in unpack(params).items()}
    h1 = np.maximum(np.asarray(x, dtype=np.float64) @ u["W1"] + u["b1"], 0.0)
    h2 = np.maximum(h1 @ u["W2"] + u["b2"], 0.0)
    z = h2 @ u["W3"] + u["b3"][0]
    return 1.0 / (1.0 + np.exp(-z))


@dataclass
class Trace:
    features: np.ndarray   # [n, 12] float32
    tile: np.ndarray       # [n] uint32
    wave: np.ndarray       # [n] uint32
    useful: np.ndarray     # [n] uint8
    sweeps: np.ndarray     # [n] uint32
    total: int = 0         # block-solves the trace saw (> n when it overflowed)

    def __len__(self) -> int:
        return len(self.tile)

    @staticmethod
    def concat(traces) -> "Trace":
        traces = list(traces)
        return Trace(np.concatenate([t.features for t in traces]), np.concatenate([t.tile for t in traces]),
                     np.concatenate([t.wave for t in traces]), np.concatenate([t.useful for t in traces]),
                     np.concatenate([t.sweeps for t in traces]), sum(t.total for t in traces))


def final_labels(trace: Trace) -> np.ndarray:
    """Hindsight training target from a trace: 1 for a block-solve that moved
    some cell by more than eps (the recorded label) and was the last such
    solve of its tile, i.e. whose result no later solve superseded; 0 for a
    solve that moved nothing (wasted) or whose tile moved again later
    (premature). Records must be in the order the solves committed, as the
    recorder writes them."""
    n = len(trace)
    useful = np.asarray(trace.useful).astype(bool)
    out = np.zeros(n, dtype=np.uint8)
    idx = np.nonzero(useful)[0]
    if idx.size:
        tiles = np.asarray(trace.tile)[idx]
        # last useful record of each tile: reverse, first occurrence
        _, first_rev = np.unique(tiles[::-1], return_index=True)
        out[idx[idx.size - 1 - first_rev]] = 1
    return out


_REC = np.dtype([("features", np.float32, (FEATURES,)), ("tile", np.uint32), ("wave", np.uint32),
                 ("useful", np.uint32), ("sweeps", np.uint32)])
assert _REC.itemsize == ctypes.sizeof(_lib.GhcmTraceRecord)


def enable_trace(setup, capacity: int) -> None:
    """Records up to `capacity` block-solves of each following solve."""
    rc = _lib.load().ghcm_trace_enable(setup.handle, int(capacity))
    if rc != 0:
        raise GhcmError(rc, "ghcm_trace_enable")


def read_trace(setup) -> Trace:
    """The trace of the last solve on `setup`."""
    lib = _lib.load()
    total = ctypes.c_uint32()
    n = ctypes.c_uint32()
    rc = lib.ghcm_trace_read(setup.handle, None, 0, ctypes.byref(n), ctypes.byref(total))
    if rc != 0:
        raise GhcmError(rc, "ghcm_trace_read")
    buf = np.empty(total.value, dtype=_REC)
    if total.value:
        rc = lib.ghcm_trace_read(setup.handle, buf.ctypes.data, total.value, ctypes.byref(n), None)
        if rc != 0:
            raise GhcmError(rc, "ghcm_trace_read")
        buf = buf[: n.value]
    return Trace(buf["features"].copy(), buf["tile"].copy(), buf["wave"].copy(), buf["useful"].astype(np.uint8),
                 buf["sweeps"].copy(), int(total.value))


def set_model(setup, params: np.ndarray | None, threshold: float = 0.5) -> None:
    """Installs (or with None removes) the model of the learned schedule."""
    lib = _lib.load()
    if params is None:
        rc = lib.ghcm_set_schedule_model(setup.handle, None, 0, 0.5)
    else:
        p = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
        rc = lib.ghcm_set_schedule_model(setup.handle, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.size,
                                         float(threshold))
    if rc != 0:
        raise GhcmError(rc, "ghcm_set_schedule_model")


POLICY_SCORE = _lib.GHCM_POLICY_SCORE
POLICY_VETO = _lib.GHCM_POLICY_VETO


def set_policy(setup, policy: int = POLICY_SCORE, max_vetoes: int = 2) -> None:
    """How the model is used: POLICY_SCORE (the default: each tile is scored by
    the solve that queues it; a wave takes those at or above the threshold
    and is filled up to fallback_jobs in key order) or POLICY_VETO (the plain
    top-n proposes, the model defers low-scoring claims)."""
    rc = _lib.load().ghcm_set_schedule_policy(setup.handle, int(policy), int(max_vetoes))
    if rc != 0:
        raise GhcmError(rc, "ghcm_set_schedule_policy")


def counters(setup) -> dict:
    """Learned-schedule counters of the last solve."""
    out = (ctypes.c_uint32 * 4)()
    rc = _lib.load().ghcm_schedule_counters(setup.handle, out)
    if rc != 0:
        raise GhcmError(rc, "ghcm_schedule_counters")
    return {"score_waves": out[0], "fallback_waves": out[1], "trace_records": out[2], "vetoes": out[3]}


def _device():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("the MLP kernels need a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


def predict(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Probabilities from the inference kernel (ghcm_mlp_forward)."""
    import torch

    dev = _device()
    dp = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).to(dev)
    dx = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32).reshape(-1, FEATURES)).to(dev)
    out = torch.empty(dx.shape[0], dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream(dev)
    rc = _lib.load().ghcm_mlp_forward(ctypes.c_void_p(dp.data_ptr()), ctypes.c_void_p(dx.data_ptr()), dx.shape[0],
                                      ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s.cuda_stream))
    if rc != 0:
        raise GhcmError(rc, "ghcm_mlp_forward")
    return out.cpu().numpy()


def train(x: np.ndarray, y: np.ndarray, params: np.ndarray | None = None, *, epochs: int = 20, batch: int = 4096,
          lr: float = 1e-3, pos_weight: float = 1.0, seed: int = 0) -> tuple[np.ndarray, list[float]]:
    """Trains the MLP with the library's kernels (ghcm_mlp_train, Adam on
    weighted BCE). Samples are shuffled once with `seed`. Returns the
    parameters and the mean loss of every epoch."""
    import torch

    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, FEATURES)
    y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1)
    if len(x) != len(y) or len(x) == 0:
        raise ValueError("x and y must be non-empty and of the same length")
    order = np.random.default_rng(seed).permutation(len(x))
    dev = _device()
    dx = torch.from_numpy(x[order]).to(dev)
    dy = torch.from_numpy(y[order]).to(dev)
    p0 = init_params(seed) if params is None else np.asarray(params, dtype=np.float32).copy()
    dp = torch.from_numpy(p0).to(dev)
    cfg = _lib.GhcmTrainConfig()
    lib = _lib.load()
    lib.ghcm_train_config_default(ctypes.byref(cfg))
    cfg.epochs, cfg.batch, cfg.lr, cfg.pos_weight = int(epochs), int(batch), float(lr), float(pos_weight)
    losses = (ctypes.c_float * int(epochs))()
    s = torch.cuda.current_stream(dev)
    rc = lib.ghcm_mlp_train(ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dy.data_ptr()), len(x),
                            ctypes.c_void_p(dp.data_ptr()), ctypes.byref(cfg), ctypes.c_void_p(s.cuda_stream), losses)
    if rc != 0:
        raise GhcmError(rc, "ghcm_mlp_train")
    return dp.cpu().numpy(), list(losses)


def save_model(path, params: np.ndarray, threshold: float, **meta) -> None:
    """Writes a model file (.npz): parameters, threshold, feature names and
    any metadata (training seeds, losses, ...)."""
    np.savez(path, params=np.asarray(params, dtype=np.float32), threshold=np.float32(threshold),
             feature_names=np.array(FEATURE_NAMES), **{k: np.asarray(v) for k, v in meta.items()})


def load_model(path) -> tuple[np.ndarray, float, dict]:
    with np.load(Path(path), allow_pickle=False) as z:
        params = z["params"].astype(np.float32)
        if params.size != N_PARAMS:
            raise ValueError(f"{path}: {params.size} parameters, expected {N_PARAMS}")
        meta = {k: z[k] for k in z.files if k not in ("params", "threshold")}
        return params, float(z["threshold"]), meta
