"""GB300 (sm_103a) ray-casting hot path of iVR behind a C ABI.

``libivr_gpu.so`` (include/ivr_gpu.h) holds the CUDA kernels and the C
entry points; ``ivr_gb300.api`` wraps them for Python.  The library is built
in-tree with ``python -m ivr_gb300.build``.
"""
from .state import IvrState, orbit_state  # noqa: F401

__all__ = ["IvrState", "orbit_state"]
