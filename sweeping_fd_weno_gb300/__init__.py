"""GB300-native sweeping positivity-preserving FD-WENO Euler time step.

The compute path is the CUDA library ``_lib/libswfd.so`` (C ABI in
include/swfd.h); this package is the host side over it.
"""
from . import abi
from .batch import Batch
from .problems import make_config, reference_defaults, workload
from .solver import Solver

__all__ = ["abi", "Batch", "Solver", "make_config", "reference_defaults", "workload"]
