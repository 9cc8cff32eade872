"""GB300-native gHCM: block-scheduled eikonal solver with device-side scheduling.

The compute path is libghcm.so (CUDA, sm_103a) behind the C ABI in
include/ghcm.h; this package holds its build recipe, a ctypes binding, the
Python mirror of the reference's solver interface and synthetic workloads.
"""
from ._lib import GhcmError, load as load_library  # noqa: F401
from .eikonal import (  # noqa: F401
    CacheMode,
    EikonalResult,
    HcmConfig,
    HcmSetup,
    Kernel,
    KeyMode,
    Schedule,
    eikonal_hcm_cuda,
    eikonal_hcm_cuda_ex,
    eikonal_hcm_cuda_setup,
    solve_device,
)
from .batch import (  # noqa: F401
    Batch,
    DeviceInstance,
    autotune_batch,
    shard_instances,
    solve_batched,
    solve_sharded,
)
from . import learned  # noqa: F401
