"""Host side of the learned schedule (ghcm_gb300.learned): the flat parameter
layout shared with the CUDA kernels, initialisation, the float64 numpy
reference of the MLP, trace containers and model files. No GPU."""
from __future__ import annotations

import numpy as np
import pytest

from ghcm_gb300 import _lib, learned


def test_parameter_layout_matches_the_c_abi():
    assert learned.N_PARAMS == _lib.GHCM_MLP_PARAMS == 12 * 64 + 64 + 64 * 64 + 64 + 64 + 1
    p = np.arange(learned.N_PARAMS, dtype=np.float32)
    u = learned.unpack(p)
    assert u["W1"].shape == (12, 64) and u["W1"][1, 0] == 64  # input-major
    assert u["b1"][0] == 768 and u["W2"].shape == (64, 64) and u["W2"][0, 1] == 833
    assert u["b2"][0] == 4928 and u["W3"][0] == 4992 and u["b3"][0] == 5056
    with pytest.raises(ValueError):
        learned.unpack(np.zeros(10, dtype=np.float32))


def test_numpy_forward_matches_a_plain_loop():
    p = learned.init_params(3)
    u = learned.unpack(p)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, size=(5, 12)).astype(np.float32)
    got = learned.forward_numpy(p, x)
    for r in range(5):
        h1 = [max(0.0, float(u["b1"][k]) + sum(float(u["W1"][i, k]) * float(x[r, i]) for i in range(12)))
              for k in range(64)]
        h2 = [max(0.0, float(u["b2"][j]) + sum(float(u["W2"][k, j]) * h1[k] for k in range(64))) for j in range(64)]
        z = float(u["b3"][0]) + sum(float(u["W3"][j]) * h2[j] for j in range(64))
        assert abs(got[r] - 1.0 / (1.0 + np.exp(-z))) < 1e-12


def test_init_is_seeded_and_sets_the_prior():
    a, b = learned.init_params(7, prior=0.8), learned.init_params(7, prior=0.8)
    assert np.array_equal(a, b) and not np.array_equal(a, learned.init_params(8))
    assert abs(float(learned.unpack(a)["b3"][0]) - np.log(4.0)) < 1e-6
    zero = np.zeros((1, 12), dtype=np.float32)  # zero input, zero hidden biases: output = prior
    assert abs(learned.forward_numpy(a, zero)[0] - 0.8) < 1e-6


def test_trace_concat_and_model_files(tmp_path):
    def tr(n, base):
        return learned.Trace(np.full((n, 12), base, dtype=np.float32), np.arange(n, dtype=np.uint32),
                             np.zeros(n, dtype=np.uint32), np.ones(n, dtype=np.uint8), np.full(n, 3, dtype=np.uint32),
                             total=n + 1)
    t = learned.Trace.concat([tr(3, 0.0), tr(2, 1.0)])
    assert len(t) == 5 and t.total == 7 and t.features[4, 0] == 1.0
    p = learned.init_params(0)
    path = tmp_path / "m.npz"
    learned.save_model(path, p, 0.6, train_seeds=np.arange(4), epoch_loss=[0.5, 0.4])
    q, thr, meta = learned.load_model(path)
    assert np.array_equal(p, q) and abs(thr - 0.6) < 1e-7
    assert list(meta["feature_names"]) == list(learned.FEATURE_NAMES) and meta["train_seeds"].tolist() == [0, 1, 2, 3]


def test_final_labels_keep_only_the_last_useful_solve_of_each_tile():
    tile = np.array([5, 7, 5, 9, 7, 5, 9], dtype=np.uint32)
    useful = np.array([1, 1, 1, 0, 0, 0, 1], dtype=np.uint8)
    n = len(tile)
    tr = learned.Trace(np.zeros((n, 12), np.float32), tile, np.zeros(n, np.uint32), useful, np.ones(n, np.uint32))
    # tile 5: solves 0, 2 useful, 5 not -> 2 is final; tile 7: 1 useful, 4 not -> 1; tile 9: 6
    assert learned.final_labels(tr).tolist() == [0, 1, 1, 0, 0, 0, 1]
    empty = learned.Trace(np.zeros((0, 12), np.float32), np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                          np.zeros(0, np.uint8), np.zeros(0, np.uint32))
    assert learned.final_labels(empty).size == 0
