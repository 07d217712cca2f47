"""GB300-native FLIP step behind the reference's FluidSimulation API.

The compute lives in libflip3d_gb300.so (hand-written CUDA for sm_103a,
flipengine3d_gb300/csrc); `FluidSimulation` mirrors the reference class over
its C ABI (include/flip3d.h).
"""
from .fluidsimulation import (FluidRuntime, FluidSimulation, FlipCudaError, FlipDeviceTimeout,  # noqa: F401
                              compute_domain_solid, estimate_device_bytes, load_library)
from . import scenes  # noqa: F401
