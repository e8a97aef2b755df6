"""fastem_gb300 -- GB300 (sm_103a) backend for FastEM's EM and k-means hot path.

The compute path is libfastem_gpu.so (CUDA kernels behind the C-ABI of
include/fastem_gpu.h).  This package holds its ctypes binding, thin Python
mirrors of the reference's EMAlgorithm / GaussianMixture / KMeansAlgorithm
classes, the .bin / .cmp file formats and seeded synthetic workloads.
"""
from .em import CudaMatrixEM, GaussianMixture  # noqa: F401
from .kmeans import CudaKMA  # noqa: F401
from .batch import CudaBatchEM  # noqa: F401

__all__ = ["CudaMatrixEM", "GaussianMixture", "CudaKMA", "CudaBatchEM"]
