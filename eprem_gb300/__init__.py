"""GB300 (sm_103a) implementation of EPREM's per-timestep energetic-particle
update behind a C ABI (include/eprem_gpu.h).

* ``libeprem_gpu.so`` (csrc/) -- the CUDA kernels and the C ABI;
* ``runtime.EpremRun``        -- the reference's verbs over that ABI;
* ``runtime.Ensemble``        -- many runs stepped by one graph launch;
* ``workloads``               -- synthetic run states of the measured sizes;
* ``host/eprem_dropin.c``     -- the C shim that puts the ABI behind the
  reference's own entry points inside its driver.
"""
from . import abi, workloads  # noqa: F401
from .runtime import Ensemble, EpremGpuError, EpremRun, load_library  # noqa: F401

__all__ = ["abi", "workloads", "EpremRun", "Ensemble", "EpremGpuError", "load_library"]
