"""GB300-native compute kernel for ReaDDy (particle-based reaction-diffusion).

The hot path (cell list, pair and bonded forces, Euler Brownian dynamics, uncontrolled-approximation
and Gillespie reaction handlers) runs as hand-written sm_103a CUDA in libreaddy_cuda_core.so, reached
through the C ABI of include/readdy_cuda.h.  There is no CPU fallback.
"""
from ._native import CapacityError, CudaKernelError, GILLESPIE, UNCONTROLLED_APPROXIMATION, load
from .kernel import KERNEL_NAME, CUDAKernel, Context

__all__ = ["Context", "CUDAKernel", "KERNEL_NAME", "GILLESPIE", "UNCONTROLLED_APPROXIMATION",
           "CapacityError", "CudaKernelError", "load"]
