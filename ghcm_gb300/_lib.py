"""ctypes binding of libghcm.so (the C ABI declared in include/ghcm.h)."""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libghcm.so"

GHCM_OK = 0
GHCM_ERR_BAD_ARG = -1
GHCM_ERR_BAD_INPUT = -2
GHCM_ERR_OOM = -3
GHCM_ERR_CUDA = -4
GHCM_ERR_TIMEOUT = -5
GHCM_ERR_NOT_CONVERGED = -6
GHCM_ERR_UNSUPPORTED = -7
GHCM_ERR_INTERNAL = -8
GHCM_ERR_TOO_LARGE = -9
GHCM_NOALLOC_MAX_TILES = 262144

GHCM_KERNEL_SYSTOLIC = 0
GHCM_KERNEL_FIM = 1
GHCM_SCHEDULE_PLAIN = 0
GHCM_SCHEDULE_LEARNED = 1
GHCM_KEY_BOUNDARY_MIN = 0
GHCM_KEY_BLOCK_MIN = 1

# Every entry point include/ghcm.h declares.
EXPORTS = (
    "ghcm_config_default",
    "ghcm_create",
    "ghcm_destroy",
    "ghcm_solve",
    "ghcm_solve_device",
    "ghcm_device_sm_count",
    "ghcm_status_string",
    "ghcm_abi_version",
    "ghcm_selftest_wait_timeout",
    "ghcm_selftest_sqrt",
    "ghcm_solve_device_noalloc",
    "ghcm_batch_create",
    "ghcm_batch_run",
    "ghcm_batch_query",
    "ghcm_batch_destroy",
    "ghcm_solve_batched",
    "ghcm_autotune_batch",
    "ghcm_trace_enable",
    "ghcm_trace_read",
    "ghcm_set_schedule_model",
    "ghcm_set_schedule_policy",
    "ghcm_schedule_counters",
    "ghcm_mlp_forward",
    "ghcm_mlp_grad",
    "ghcm_train_config_default",
    "ghcm_mlp_train",
)

GHCM_MLP_FEATURES = 12
GHCM_MLP_HIDDEN = 64
GHCM_MLP_PARAMS = 5057
GHCM_REFRESH_OFF = 0xFFFFFFFF
GHCM_REFRESH_IN_SOLVE = 0xFFFFFFFE
GHCM_POLICY_SCORE = 0
GHCM_POLICY_VETO = 1


class GhcmConfig(ctypes.Structure):
    _fields_ = [
        ("block_size", ctypes.c_uint32),
        ("max_jobs", ctypes.c_uint32),
        ("eps", ctypes.c_float),
        ("kernel", ctypes.c_uint32),
        ("schedule", ctypes.c_uint32),
        ("key_mode", ctypes.c_uint32),
        ("max_sweeps", ctypes.c_uint32),
        ("max_waves", ctypes.c_uint32),
        ("wait_timeout_ms", ctypes.c_uint32),
        ("device", ctypes.c_int32),
        ("use_tma", ctypes.c_uint32),
        ("fallback_jobs", ctypes.c_uint32),
        ("cost_cap", ctypes.c_float),
        ("refresh_solves", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32 * 2),
    ]


class GhcmStats(ctypes.Structure):
    _fields_ = [
        ("block_solves", ctypes.c_uint64),
        ("cells", ctypes.c_uint64),
        ("bytes_alg", ctypes.c_uint64),
        ("waves", ctypes.c_uint32),
        ("residual_passes", ctypes.c_uint32),
        ("max_active", ctypes.c_uint32),
        ("tiles", ctypes.c_uint32),
        ("device_ms", ctypes.c_double),
        ("total_ms", ctypes.c_double),
        ("kernel_ms", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class GhcmInstance(ctypes.Structure):
    _fields_ = [
        ("field", ctypes.c_void_p),
        ("time_out", ctypes.c_void_p),
        ("seeds_xy", ctypes.c_void_p),
        ("n_seeds", ctypes.c_uint32),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
        ("h", ctypes.c_float),
        ("input_is_speed", ctypes.c_int32),
        ("reserved", ctypes.c_uint32),
    ]


class GhcmBatchInfo(ctypes.Structure):
    _fields_ = [
        ("instances", ctypes.c_uint32),
        ("tiles", ctypes.c_uint32),
        ("cells", ctypes.c_uint64),
        ("block_size", ctypes.c_uint32),
        ("max_jobs", ctypes.c_uint32),
        ("max_sweeps", ctypes.c_uint32),
        ("graph", ctypes.c_uint32),
        ("grid", ctypes.c_uint32),
        ("tma_instances", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32 * 2),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class GhcmTuneTrial(ctypes.Structure):
    _fields_ = [
        ("block_size", ctypes.c_uint32),
        ("max_jobs", ctypes.c_uint32),
        ("max_sweeps", ctypes.c_uint32),
        ("status", ctypes.c_int32),
        ("ms", ctypes.c_double),
        ("block_solves", ctypes.c_uint64),
        ("kernel", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class GhcmTraceRecord(ctypes.Structure):
    _fields_ = [
        ("features", ctypes.c_float * 12),
        ("tile", ctypes.c_uint32),
        ("wave", ctypes.c_uint32),
        ("useful", ctypes.c_uint32),
        ("sweeps", ctypes.c_uint32),
    ]


class GhcmTrainConfig(ctypes.Structure):
    _fields_ = [
        ("epochs", ctypes.c_uint32),
        ("batch", ctypes.c_uint32),
        ("lr", ctypes.c_float),
        ("beta1", ctypes.c_float),
        ("beta2", ctypes.c_float),
        ("adam_eps", ctypes.c_float),
        ("pos_weight", ctypes.c_float),
        ("reserved", ctypes.c_uint32 * 5),
    ]


class GhcmError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({status})" if what else f"{status_string(status)} ({status})")


_lib = None


def load(path: Path | None = None):
    """Loads libghcm.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build it with `python -m ghcm_gb300.build`")
    lib = ctypes.CDLL(str(p))
    f32p = ctypes.POINTER(ctypes.c_float)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    cfgp = ctypes.POINTER(GhcmConfig)
    stp = ctypes.POINTER(GhcmStats)
    vp = ctypes.c_void_p
    lib.ghcm_config_default.argtypes = [cfgp]
    lib.ghcm_create.argtypes = [cfgp, ctypes.POINTER(vp)]
    lib.ghcm_destroy.argtypes = [vp]
    lib.ghcm_solve.argtypes = [vp, f32p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, u32p,
                               ctypes.c_uint32, f32p, stp]
    lib.ghcm_solve_device.argtypes = [vp, vp, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, vp,
                                      ctypes.c_uint32, vp, vp, stp]
    lib.ghcm_device_sm_count.argtypes = [vp, u32p]
    lib.ghcm_status_string.argtypes = [ctypes.c_int]
    lib.ghcm_status_string.restype = ctypes.c_char_p
    lib.ghcm_abi_version.argtypes = []
    lib.ghcm_selftest_wait_timeout.argtypes = [vp, ctypes.c_uint32]
    lib.ghcm_selftest_sqrt.argtypes = [vp, ctypes.POINTER(ctypes.c_ulonglong)]
    lib.ghcm_solve_device_noalloc.argtypes = [cfgp, vp, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                              vp, ctypes.c_uint32, vp, vp]
    instp = ctypes.POINTER(GhcmInstance)
    lib.ghcm_batch_create.argtypes = [vp, instp, ctypes.c_uint32, ctypes.POINTER(vp)]
    lib.ghcm_batch_run.argtypes = [vp, vp, stp]
    lib.ghcm_batch_query.argtypes = [vp, ctypes.POINTER(GhcmBatchInfo)]
    lib.ghcm_batch_destroy.argtypes = [vp]
    lib.ghcm_solve_batched.argtypes = [vp, instp, ctypes.c_uint32, vp, stp]
    lib.ghcm_autotune_batch.argtypes = [cfgp, instp, ctypes.c_uint32, vp, ctypes.c_uint32, cfgp,
                                        ctypes.POINTER(GhcmTuneTrial), ctypes.c_uint32, u32p]
    lib.ghcm_trace_enable.argtypes = [vp, ctypes.c_uint32]
    lib.ghcm_trace_read.argtypes = [vp, ctypes.c_void_p, ctypes.c_uint32, u32p, u32p]
    lib.ghcm_set_schedule_model.argtypes = [vp, f32p, ctypes.c_uint32, ctypes.c_float]
    lib.ghcm_schedule_counters.argtypes = [vp, u32p]
    lib.ghcm_set_schedule_policy.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32]
    lib.ghcm_mlp_forward.argtypes = [vp, vp, ctypes.c_uint32, vp, vp]
    lib.ghcm_mlp_grad.argtypes = [vp, vp, vp, ctypes.c_uint32, ctypes.c_float, vp, vp, vp]
    tcp = ctypes.POINTER(GhcmTrainConfig)
    lib.ghcm_train_config_default.argtypes = [tcp]
    lib.ghcm_mlp_train.argtypes = [vp, vp, ctypes.c_uint32, vp, tcp, vp, f32p]
    for name in EXPORTS:
        if name != "ghcm_status_string":
            getattr(lib, name).restype = ctypes.c_int
    if path is None:
        _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load().ghcm_status_string(int(status)).decode()
    except FileNotFoundError:
        return "library not built"
