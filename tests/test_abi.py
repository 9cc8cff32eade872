"""The C ABI without a GPU: libghcm.so loads, exports every entry point that
include/ghcm.h declares, its structs have the ctypes layout, and calls that
need no device behave (defaults, status strings, argument checks)."""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from ghcm_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "ghcm.h"


def declared_functions() -> set[str]:
    text = HEADER.read_text()
    return set(re.findall(r"^\s*(?:int|const char\*)\s+(ghcm_\w+)\s*\(", text, flags=re.M))


def test_header_declares_what_the_binding_lists():
    assert declared_functions() == set(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(ghcm_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\bT (ghcm_\w+)", out.stdout))
    missing = declared_functions() - exported
    assert not missing, missing
    for name in declared_functions():
        assert hasattr(ghcm_lib, name)


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "ghcm.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(ghcm_config), sizeof(ghcm_stats),"
        " offsetof(ghcm_stats, device_ms), offsetof(ghcm_config, use_tma), sizeof(ghcm_instance),"
        " offsetof(ghcm_instance, input_is_speed), sizeof(ghcm_batch_info), offsetof(ghcm_batch_info, tma_instances),"
        " sizeof(ghcm_tune_trial), offsetof(ghcm_tune_trial, ms), sizeof(ghcm_trace_record),"
        " sizeof(ghcm_train_config), (size_t)GHCM_MLP_PARAMS); return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ctypes.sizeof(_lib.GhcmConfig), ctypes.sizeof(_lib.GhcmStats),
                   _lib.GhcmStats.device_ms.offset, _lib.GhcmConfig.use_tma.offset,
                   ctypes.sizeof(_lib.GhcmInstance), _lib.GhcmInstance.input_is_speed.offset,
                   ctypes.sizeof(_lib.GhcmBatchInfo), _lib.GhcmBatchInfo.tma_instances.offset,
                   ctypes.sizeof(_lib.GhcmTuneTrial), _lib.GhcmTuneTrial.ms.offset,
                   ctypes.sizeof(_lib.GhcmTraceRecord), ctypes.sizeof(_lib.GhcmTrainConfig), _lib.GHCM_MLP_PARAMS]


def test_header_compiles_as_cpp(tmp_path):
    src = tmp_path / "h.cpp"
    src.write_text('#include "ghcm.h"\nint main(){ ghcm_config c; ghcm_config_default(&c); return (int)c.block_size - 16; }\n')
    subprocess.run(["g++", "-std=c++14", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                   check=True)


def test_defaults_mirror_the_reference_config(ghcm_lib):
    c = _lib.GhcmConfig()
    assert ghcm_lib.ghcm_config_default(ctypes.byref(c)) == 0
    assert c.block_size == 16 and c.max_jobs == 0
    assert abs(c.eps - 1e-5) < 1e-12  # HcmConfig::fim_minimum_change (src/eikonal.h:24)
    assert c.kernel == _lib.GHCM_KERNEL_SYSTOLIC  # HcmConfig::kernel (src/eikonal.h:26)
    assert c.use_tma == 1 and c.device == -1 and c.fallback_jobs == 0 and c.cost_cap == 0.0 and c.refresh_solves == 0 and list(c.reserved) == [0] * 2


def test_status_strings(ghcm_lib):
    for code in range(-9, 1):
        assert ghcm_lib.ghcm_status_string(code)
    assert ghcm_lib.ghcm_status_string(-99) == b"unknown status"
    assert ghcm_lib.ghcm_abi_version() == 1


def test_create_rejects_bad_config(ghcm_lib):
    c = _lib.GhcmConfig()
    ghcm_lib.ghcm_config_default(ctypes.byref(c))
    h = ctypes.c_void_p()
    for field, value in (("block_size", 12), ("kernel", 7), ("eps", -1.0), ("refresh_solves", 16)):
        bad = _lib.GhcmConfig.from_buffer_copy(c)
        setattr(bad, field, value)
        assert ghcm_lib.ghcm_create(ctypes.byref(bad), ctypes.byref(h)) == _lib.GHCM_ERR_BAD_ARG
    bad = _lib.GhcmConfig.from_buffer_copy(c)
    bad.reserved[1] = 1
    assert ghcm_lib.ghcm_create(ctypes.byref(bad), ctypes.byref(h)) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_create(None, ctypes.byref(h)) == _lib.GHCM_ERR_BAD_ARG


def test_null_context_calls(ghcm_lib):
    assert ghcm_lib.ghcm_destroy(None) == 0
    assert ghcm_lib.ghcm_solve(None, None, 1, 4, 4, 1.0, None, 0, None, None) == _lib.GHCM_ERR_BAD_ARG
    n = ctypes.c_uint32()
    assert ghcm_lib.ghcm_device_sm_count(None, ctypes.byref(n)) == _lib.GHCM_ERR_BAD_ARG


def test_create_without_gpu_fails_cleanly(ghcm_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c = _lib.GhcmConfig()
    ghcm_lib.ghcm_config_default(ctypes.byref(c))
    h = ctypes.c_void_p()
    assert ghcm_lib.ghcm_create(ctypes.byref(c), ctypes.byref(h)) == _lib.GHCM_ERR_UNSUPPORTED
    assert not h.value


def test_python_interface_reports_missing_gpu():
    import torch

    import ghcm_gb300 as g

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert g.eikonal_hcm_cuda_setup(g.HcmConfig()) is None
    with pytest.raises(g.GhcmError):
        g.HcmSetup(g.HcmConfig())


def test_batch_calls_check_arguments(ghcm_lib):
    b = ctypes.c_void_p()
    inst = (_lib.GhcmInstance * 1)()
    assert ghcm_lib.ghcm_batch_create(None, inst, 1, ctypes.byref(b)) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_batch_create(None, inst, 1, None) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_batch_run(None, None, None) == _lib.GHCM_ERR_BAD_ARG
    info = _lib.GhcmBatchInfo()
    assert ghcm_lib.ghcm_batch_query(None, ctypes.byref(info)) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_batch_destroy(None) == 0
    assert ghcm_lib.ghcm_solve_batched(None, inst, 1, None, None) == _lib.GHCM_ERR_BAD_ARG
    c = _lib.GhcmConfig()
    ghcm_lib.ghcm_config_default(ctypes.byref(c))
    best = _lib.GhcmConfig()
    n = ctypes.c_uint32()
    assert ghcm_lib.ghcm_autotune_batch(ctypes.byref(c), None, 0, None, 1, ctypes.byref(best), None, 0,
                                        ctypes.byref(n)) == _lib.GHCM_ERR_BAD_ARG
    bad = _lib.GhcmConfig.from_buffer_copy(c)
    bad.block_size = 24
    assert ghcm_lib.ghcm_autotune_batch(ctypes.byref(bad), inst, 1, None, 1, ctypes.byref(best), None, 0,
                                        ctypes.byref(n)) == _lib.GHCM_ERR_BAD_ARG


def test_learned_calls_check_arguments(ghcm_lib):
    n = ctypes.c_uint32()
    assert ghcm_lib.ghcm_trace_enable(None, 16) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_trace_read(None, None, 0, ctypes.byref(n), None) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_set_schedule_model(None, None, 0, 0.5) == _lib.GHCM_ERR_BAD_ARG
    out = (ctypes.c_uint32 * 4)()
    assert ghcm_lib.ghcm_schedule_counters(None, out) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_mlp_forward(None, None, 4, None, None) == _lib.GHCM_ERR_BAD_ARG
    assert ghcm_lib.ghcm_mlp_grad(None, None, None, 4, 1.0, None, None, None) == _lib.GHCM_ERR_BAD_ARG
    tc = _lib.GhcmTrainConfig()
    assert ghcm_lib.ghcm_train_config_default(ctypes.byref(tc)) == 0
    assert tc.epochs > 0 and tc.batch > 0 and tc.lr > 0 and tc.pos_weight == 1.0 and list(tc.reserved) == [0] * 5
    assert ghcm_lib.ghcm_mlp_train(None, None, 0, None, ctypes.byref(tc), None, None) == _lib.GHCM_ERR_BAD_ARG


def test_cost_cap_must_be_a_non_negative_number(ghcm_lib):
    c = _lib.GhcmConfig()
    ghcm_lib.ghcm_config_default(ctypes.byref(c))
    h = ctypes.c_void_p()
    for bad in (-1.0, float("nan")):
        x = _lib.GhcmConfig.from_buffer_copy(c)
        x.cost_cap = bad
        assert ghcm_lib.ghcm_create(ctypes.byref(x), ctypes.byref(h)) == _lib.GHCM_ERR_BAD_ARG


def test_noalloc_rejects_sizes_that_wrap_before_any_launch(ghcm_lib):
    """A width near 2^32 must not wrap the tile count to a small number: the
    call returns GHCM_ERR_TOO_LARGE before touching the device (so this runs
    without a GPU, with dummy pointers that are never dereferenced)."""
    c = _lib.GhcmConfig()
    ghcm_lib.ghcm_config_default(ctypes.byref(c))
    dummy = ctypes.c_void_p(16)
    for w, h in ((0xFFFFFFFF, 1), (1, 0xFFFFFFFF), (0xFFFFFFF1, 0xFFFFFFF1), (1 << 31, 2)):
        rc = ghcm_lib.ghcm_solve_device_noalloc(ctypes.byref(c), dummy, 1, w, h, 1.0, dummy, 1, dummy, None)
        assert rc == _lib.GHCM_ERR_TOO_LARGE, (w, h, rc)


def test_refresh_modes_pass_the_config_check(ghcm_lib):
    """The named update-bound modes and 1..15 pass the config check (without a
    GPU ghcm_create then stops at the device, never at the config); 16 and
    other values are bad arguments."""
    c = _lib.GhcmConfig()
    ghcm_lib.ghcm_config_default(ctypes.byref(c))
    h = ctypes.c_void_p()
    for ok in (0, 1, 15, _lib.GHCM_REFRESH_OFF, _lib.GHCM_REFRESH_IN_SOLVE):
        c.refresh_solves = ok
        rc = ghcm_lib.ghcm_create(ctypes.byref(c), ctypes.byref(h))
        assert rc != _lib.GHCM_ERR_BAD_ARG, ok
        if rc == 0:
            ghcm_lib.ghcm_destroy(h)
    for bad in (16, 1000, 0xFFFFFFFD):
        c.refresh_solves = bad
        assert ghcm_lib.ghcm_create(ctypes.byref(c), ctypes.byref(h)) == _lib.GHCM_ERR_BAD_ARG, bad
