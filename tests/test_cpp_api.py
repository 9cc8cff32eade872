"""The C++ interface in include/ghcm_eikonal.hpp compiles against the C ABI,
links to libghcm.so and, on a GPU, solves like the reference's interface."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

from ghcm_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def cpp_exe(ghcm_lib, tmp_path_factory):
    exe = tmp_path_factory.mktemp("cpp") / "eikonal_api_check"
    lib_dir = _lib.LIB_PATH.parent
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "eikonal_api_check.cpp"), "-L", str(lib_dir), "-lghcm",
                    f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    return exe


def test_cpp_interface_builds_and_handles_no_device(cpp_exe):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present (covered by the gpu test)")
    r = subprocess.run([str(cpp_exe)], capture_output=True, text=True)
    assert r.returncode == 2 and "no device" in r.stdout


@pytest.mark.gpu
def test_cpp_interface_solves(cpp_exe, cuda_ok):
    r = subprocess.run([str(cpp_exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
