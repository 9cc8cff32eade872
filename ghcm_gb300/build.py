"""Builds libghcm.so in-tree with nvcc for sm_103a (GB300).

    python -m ghcm_gb300.build            # or ghcm_gb300.build.build()

Translation units are compiled in parallel into ghcm_gb300/_build/ and linked
into ghcm_gb300/libghcm.so (the CUDA runtime is linked statically, so the
library carries no dependency on a particular libcudart next to it).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libghcm.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _nvcc() -> str:
    return str(_cuda_home() / "bin" / "nvcc")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _compile(src: Path, extra: list[str], build_dir: Path) -> Path:
    obj = build_dir / (src.name + ".o")
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *inc, *extra,
               "-c", str(src), "-o", str(obj)]
    else:
        cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-Wall", "-Wextra",
               "-I", str(_cuda_home() / "include"), *inc, *[d for d in extra if d.startswith("-D")],
               "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra_nvcc: list[str] | None = None, out: Path | None = None) -> Path:
    """Compiles every CUDA/C++ source of the package and links libghcm.so
    (or `out`). `-D` flags in extra_nvcc also reach the host compiler."""
    lib = Path(out) if out else LIB
    build_dir = BUILD if out is None else lib.parent / (lib.stem + "_build")
    build_dir.mkdir(parents=True, exist_ok=True)
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=max(2, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra_nvcc or []), build_dir), srcs))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl",
           "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(verbose=True, extra_nvcc=sys.argv[1:])
