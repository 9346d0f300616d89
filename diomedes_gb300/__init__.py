"""diomedes_gb300 -- GB300-native (sm_103a) rigid-body step of Diomedes.

The compute path is libdio_cuda.so (hand-written CUDA behind the C ABI in
include/dio_cuda.h).  This package holds the ctypes binding (`abi`), the
host-side mirror of the reference's physics API (`physics`), the compute
objects (`compute`: NarrowPhaseCompute, AvbdCompute, World) and seeded
scene generators (`scenes`).
"""
from . import abi, physics, scenes  # noqa: F401
from .compute import AvbdCompute, Context, NarrowPhaseCompute, World, capacity, decode_contacts  # noqa: F401

__all__ = ["abi", "physics", "scenes", "AvbdCompute", "Context", "NarrowPhaseCompute", "World", "capacity",
           "decode_contacts"]
