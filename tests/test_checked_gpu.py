"""The GHCM_CHECKED build of the solver: every shared-memory and global index
the tile solvers, the residual pass and the top-n gather compute is checked
(a failed check sets an error bit and skips the access; the solve returns
GHCM_ERR_INTERNAL and names the site on stderr). Small and odd grid sizes,
every tile size, both tile kernels, TMA and plain staging, batches (the
8-CTA-per-SM builds), a single field with many jobs per wave and the no-alloc
entry point must pass every check and still match the oracle FIM.

The checked library is built in-tree and run in a child process, so that its
handles never mix with those of the library the other tests load.
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
CHECKED_SO = ROOT / "ghcm_gb300" / "_checked" / "libghcm_checked.so"
TOL = 1e-5  # max relative difference vs the reference FIM

CHILD = r"""
import json, sys
sys.path.insert(0, {root!r})
from pathlib import Path
import numpy as np
import torch
from ghcm_gb300 import _lib, fields
from ghcm_gb300.build import build
_lib._lib = _lib.load(build(extra_nvcc=["-DGHCM_CHECKED"], out=Path({so!r})))
import ghcm_gb300 as g
from oracle.oracle import Oracle, build as build_oracle, rel_diff
build_oracle(with_reference=False)
o = Oracle()
rng = np.random.default_rng(7)
worst, runs = 0.0, 0
cases = []
for w, h in ((32, 32), (64, 64), (37, 53), (67, 45), (129, 97)):
    speed = rng.uniform(0.1, 1.0, size=(h, w)).astype(np.float32)
    seeds = np.array([[w // 3, h // 2], [w - 1, 0]], dtype=np.uint32)
    cases.append((speed, seeds, o.fim(fields.cost_from_speed(speed), seeds, 1e-5)[0]))
for speed, seeds, ref in cases:
    for block in (8, 16, 32):
        for kernel in (g.Kernel.Systolic, g.Kernel.FIM):
            for tma in (True, False):
                with g.HcmSetup(g.HcmConfig(block_size=block, kernel=kernel, use_tma=tma, max_jobs=16)) as s:
                    res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
                worst = max(worst, rel_diff(res.field, ref))
                runs += 1
# one field with more jobs per wave than twice the 4-CTA grid (the wide build for B=16)
speed, seeds = fields.value_noise(1024, seed=5, base_period=128.0, sources=16)
ref = o.fim(fields.cost_from_speed(speed), seeds, 1e-5)[0]
with g.HcmSetup(g.HcmConfig(block_size=16, max_jobs=100000)) as s:
    res = g.eikonal_hcm_cuda_ex(s, speed, seeds, input_is_speed=True)
worst = max(worst, rel_diff(res.field, ref))
runs += 1
# batches of the small fields (the wide builds for B=16 and B=32)
dev = torch.device("cuda", 0)
for block in (16, 32):
    insts = [g.DeviceInstance(torch.from_numpy(sp).to(dev), torch.from_numpy(sd.astype(np.int32)).to(dev),
                              torch.empty(sp.shape, dtype=torch.float32, device=dev)) for sp, sd, _ in cases]
    with g.HcmSetup(g.HcmConfig(block_size=block, max_jobs=4096)) as s:
        g.solve_batched(s, insts)
    for di, (_, _, r) in zip(insts, cases):
        worst = max(worst, rel_diff(di.d_time.cpu().numpy(), r))
        runs += 1
# the no-alloc entry point on one small odd-size field
import ctypes
speed, seeds, ref = cases[3]
cfg = _lib.GhcmConfig()
_lib._lib.ghcm_config_default(ctypes.byref(cfg))
cfg.block_size = 16
cfg.max_jobs = 16
d_speed = torch.from_numpy(speed).to(dev)
d_seeds = torch.from_numpy(seeds.astype(np.int32)).to(dev)
d_time = torch.empty_like(d_speed)
rc = _lib._lib.ghcm_solve_device_noalloc(ctypes.byref(cfg), ctypes.c_void_p(d_speed.data_ptr()), 1, speed.shape[1],
                                          speed.shape[0], 1.0, ctypes.c_void_p(d_seeds.data_ptr()), seeds.shape[0],
                                          ctypes.c_void_p(d_time.data_ptr()),
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
assert rc == 0, rc
worst = max(worst, rel_diff(d_time.cpu().numpy(), ref))
runs += 1
print(json.dumps({{"worst": worst, "runs": runs}}))
"""


def test_checked_build_passes_every_index_check(cuda_ok):
    CHECKED_SO.parent.mkdir(parents=True, exist_ok=True)
    child = CHILD.format(root=str(ROOT), so=str(CHECKED_SO))
    r = subprocess.run([sys.executable, "-c", child], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "[ghcm-checked]" not in r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["runs"] == 5 * 3 * 2 * 2 + 1 + 2 * 5 + 1
    assert d["worst"] <= TOL
