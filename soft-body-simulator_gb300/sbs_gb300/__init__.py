"""GB300 XPBD soft-body solver: Python side of libsbs_gpu.so.

``capi`` binds the C ABI (include/sbs_gpu.h); ``scenes`` generates the
synthetic tetrahedral workloads; ``build`` compiles the CUDA library.
"""
from . import scenes  # noqa: F401

__all__ = ["scenes", "capi", "build"]
