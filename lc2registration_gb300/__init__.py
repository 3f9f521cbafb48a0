"""GB300-native LC2 similarity hot path of LC2Registration.

``capi``      ctypes binding of liblc2.so (CUDA kernels behind include/lc2.h)
``geometry``  image geometry and the reference's transform builders
``synth``     seeded synthetic MR/US workloads
``build``     nvcc build of liblc2.so (sm_103a)
"""
from .geometry import Geometry, affine2d, affine3d, virtual_geometry  # noqa: F401

__all__ = ["Geometry", "affine2d", "affine3d", "virtual_geometry"]
