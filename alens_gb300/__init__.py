"""GB300-native rod collision-and-constraint step (the SylinderSystem::runStep
hot path of aLENS/SimToolbox) behind a C ABI (``include/alens_gpu.h``).

Python is the test and benchmark harness; the product is the CUDA library
``alens_gb300/lib/libalens_gpu.so`` and the C++ ``SylinderSystem`` facade in
``alens_gb300/csrc/facade``.
"""
from .capi import (AlensBlock, AlensConfig, AlensError, AlensStepStats, GpuSystem, RodState,
                   load_library, make_config)

__all__ = ["AlensBlock", "AlensConfig", "AlensError", "AlensStepStats", "GpuSystem", "RodState",
           "load_library", "make_config"]
