"""MoreFit likelihood engine for GB300 (sm_103a): CUDA C-ABI backend and its Python mirror.

Submodules: ``backend`` (CUDABackend / CUDABlock mirroring the reference's
ComputeBackend / ComputeBlock), ``_lib`` (ctypes binding of
include/morefit_cuda.h), ``build`` (in-tree native build).
"""
__all__ = ["backend", "build"]
