"""fluid-sim_gb300: the stable-fluids step of fluid-sim on one GB300.

The compute path is libfluidcuda.so (hand-written CUDA for sm_103a behind the
C ABI in include/fluid.h); this package builds it and mirrors the reference's
GPUFluidSolver API on top of it.
"""
from ._lib import FluidError, build, load, LIB_PATH  # noqa: F401
from .solver import GPUFluidBatch, GPUFluidSolver, make_params  # noqa: F401
from . import forced, workload  # noqa: F401
from .guess import PressureGuess, normalize_pair, read_pair_file, write_pair_file  # noqa: F401

__all__ = ["GPUFluidSolver", "GPUFluidBatch", "make_params", "PressureGuess", "FluidError", "build", "load", "LIB_PATH", "normalize_pair",
           "read_pair_file", "write_pair_file", "workload", "forced"]
