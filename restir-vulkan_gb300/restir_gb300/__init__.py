"""GB300-native ReSTIR direct-lighting path (Python side of the C ABI).

The compute runs in librestir_gb300.so (hand-written sm_103a kernels behind
include/restir_gb300.h); this package binds it with ctypes, generates the
seeded synthetic workloads and drives frames the way the reference's
App::_recordMainCommandBuffers orders its passes.
"""
from ._lib import RestirError, lib  # noqa: F401
from .camera import CameraModel  # noqa: F401
from .scenes import CONFIGS, Scene, config1, config2, config3  # noqa: F401
