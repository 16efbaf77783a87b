"""GB300-native wavefront path tracer: a drop-in for KiRaRay's
WavefrontPathTracer render pass (src/render/wavefront/integrator.h:24-104).

The compute path is libkrr_gb300.so (hand-written CUDA for sm_103a) behind the
C ABI in include/krr_gb300.h; this package is a thin host-side mirror of the
reference's pass interface over that ABI.  Nothing here computes on the CPU
in place of the GPU: if the library is missing, the entry points raise.
"""
from . import _lib, scenes
from ._lib import KrrError

__all__ = ["_lib", "scenes", "KrrError", "build"]


def build(force: bool = False):
    from .build import build as _build
    return _build(force=force)
