"""GB300-native contact pipeline for Jitter Physics 2 worlds.

The compute lives in libjitter_gpu.so (hand-written sm_103a kernels behind the C ABI of
include/jitter_gpu.h); this package binds it (abi), mirrors the reference's World API
(world) and generates the seeded workloads (scenes).
"""
from . import abi  # noqa: F401

__all__ = ["abi", "world", "scenes", "build"]
