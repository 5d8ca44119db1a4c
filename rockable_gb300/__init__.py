"""GB300-native engine for Rockable's per-step DEM hot path.

The compute lives in librk_gpu.so (rockable_gb300/csrc, C ABI in
include/rk_gpu.h); `rockable_gb300.abi` binds it from Python and
`rockable_gb300.scenes` builds the benchmark scenes.
"""
__all__ = ["abi", "scenes", "build_ext"]
