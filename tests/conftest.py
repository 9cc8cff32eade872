"""Shared test setup: the `gpu` marker, import paths, library builds."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libghcm.so")


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.oracle import Oracle, build

    build(with_reference=False)
    return Oracle()


@pytest.fixture(scope="session")
def ghcm_lib():
    """libghcm.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from ghcm_gb300 import _lib, build as b

    if not _lib.LIB_PATH.exists():
        b.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda_ok():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
