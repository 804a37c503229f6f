"""GB300-native UPPE propagator: a drop-in for the unidirectional pulse propagation z-step of
SeaRay (``modules/uppe_kernel.py``), computed by hand-written sm_103a CUDA kernels behind a C ABI
(``include/searay_uppe.h``, ``libsearay_uppe.so``)."""
from .uppe import track, propagator, DeviceGrid, Material  # noqa: F401
from .grid import VolumeGrid  # noqa: F401

__all__ = ["track", "propagator", "DeviceGrid", "Material", "VolumeGrid"]
