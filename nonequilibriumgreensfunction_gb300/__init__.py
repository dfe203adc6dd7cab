"""GB300-native (sm_103a) per-energy NEGF solve of brian-dellabetta/nonEquilibriumGreensFunction.

The compute path is libnegf_gb300.so (CUDA kernels + C ABI, include/negf.h); this package
holds its ctypes binding, the host-side mirror of the reference's subroutine interface
and the wire Hamiltonian builder.
"""
from . import capi, hamiltonian  # noqa: F401
from .negf import Solver  # noqa: F401

__all__ = ["capi", "hamiltonian", "Solver"]
