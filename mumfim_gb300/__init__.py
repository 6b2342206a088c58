"""GB300-native batched explicit fiber-network RVE solve.

A from-scratch implementation of MuMFiM's batched microscale analysis
(``mumfim::BatchedFiberRVEAnalysisExplicit``): per-RVE deformation-gradient
increment in, homogenised Cauchy stress and updated RVE state out. The
compute path is libmumfim_gpu.so (hand-written sm_103a CUDA behind the C ABI
of include/mumfim_gpu.h); this package only binds it.
"""
from ._abi import RVE_STATUS_DTYPE
from .batched import (NOALLOC_SCRATCH_BYTES, BatchedFiberRVEAnalysisExplicit, MumfimGpuError,
                      load_library)
from .network_io import FiberNetwork, Reaction, load_network
from .strategy import SolutionStrategy

__all__ = ["BatchedFiberRVEAnalysisExplicit", "MumfimGpuError", "load_library", "FiberNetwork",
           "Reaction", "load_network", "SolutionStrategy", "RVE_STATUS_DTYPE",
           "NOALLOC_SCRATCH_BYTES"]
