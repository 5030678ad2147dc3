"""GB300-native engine for FluidFlowSimulation.jl's pseudo-spectral solver step.

The compute path is libffs.so (hand-written sm_103a CUDA behind a C ABI, include/ffs.h);
this package is the host-side mirror of the reference's Julia interface:
``run_simulation``, ``readglobal``, ``parameters``, ``Simulation.initialize`` /
``advance_in_time`` and the reference file formats.
"""
from ._lib import (EXPORTS, FFS_AB3, FFS_ETD3, FFS_EULER, FFS_FP32, FFS_FP64, FFSError, FFSParams, LIB_PATH,
                   lib_available, load)
from .fields import random_spectrum, read_field, taylor_green, write_field
from .globalfile import parameters, parse_number, readglobal
from .server import Server
from .simulation import Simulation, julia_float, run_simulation, stats_line, write_dlm

__all__ = [
    "EXPORTS", "FFS_AB3", "FFS_ETD3", "FFS_EULER", "FFS_FP32", "FFS_FP64", "FFSError", "FFSParams", "LIB_PATH",
    "lib_available", "load", "random_spectrum", "read_field", "taylor_green", "write_field", "parameters",
    "parse_number", "readglobal", "Server", "Simulation", "julia_float", "run_simulation", "stats_line",
    "write_dlm",
]
