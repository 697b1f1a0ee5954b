"""GB300-native doubly periodic Stokes mobility operator (Mdot): open, bottom
wall and slit geometries, and the triply periodic box; forces and torques
(derivative-kernel or regular-kernel coupling); FP64 and mixed precision;
batched, multi-column and differentiable forms.

Hand-written sm_103a CUDA kernels behind a C ABI (libdpstokes_gb300.so,
include/dpstokes_gb300.h), driven from Python on torch tensors.
"""
from .operator import DPStokes, DPStokesBatch, StokesParams  # noqa: F401
from .autograd import mdot  # noqa: F401
from . import workloads  # noqa: F401

__all__ = ["DPStokes", "DPStokesBatch", "StokesParams", "mdot", "workloads"]
