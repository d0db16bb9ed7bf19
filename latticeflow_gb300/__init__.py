"""GB300-native lattice max-flow: push-relabel min cuts, parametric flow and
TV denoising on one GPU, behind latticeflow's solver interface.

The compute path is the native library ``_lib/liblatticeflow_gpu.so`` (CUDA
for sm_103a, C ABI in ``include/latticeflow_gpu.h``); this package is its
Python surface.
"""
from .interface import (LatticeBatch, LatticeFlow, LatticeServer, calculate2dTV, calculate2dTVBatch,  # noqa: F401
                        calculate2dTVPath, isValidKernel, isValidSolver,
                        kernelDimension, kernelInfo, validKernelNames, validSolverNames)
from ._native import BadSolverOrKernelName, LatticeFlowError, NativeLibraryMissing  # noqa: F401
