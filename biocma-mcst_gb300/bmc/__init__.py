"""bmc -- GB300-native Monte Carlo cycle of BioCMA-MCST.

The compute path is libbmc.so (hand-written CUDA for sm_103a behind the
C-ABI of include/bmc.h).  This package holds its build step, the ctypes
binding, the host-side scenario objects and the synthetic scenario
generators.
"""
from . import networks, scenarios  # noqa: F401

__all__ = ["networks", "scenarios", "sim", "build"]
