"""seidart_gpu -- GB300-native CPML-FDTD solvers with the SeidarT-Backend interface.

The compute path is libseidart_gpu.so (hand-written sm_103a CUDA behind a
C ABI, include/seidart_gpu.h); this package is its Python host side:

  api        numpy-level Problem / Solver / run
  cpmlfdtd   drop-in module with the reference's Python entry points
  cpml       C-PML coefficient grids (Komatitsch & Martin 2007)
  models     seeded synthetic models of the benchmark configurations
  fortran_io Fortran sequential-unformatted record files (.dat contract)
"""
from ._lib import (ELECTROMAG2, ELECTROMAG3, ELECTROMAG25, FP32, FP64, FP64_FAST, SEISMIC2, SEISMIC3, SEISMIC25,
                   SeidartError, UnstableError)
from .api import FIELD_SLOTS, MODEL_SLOTS, SRC_SLOTS, Problem, Solver, layout, run

__all__ = ["SEISMIC2", "SEISMIC25", "SEISMIC3", "ELECTROMAG2", "ELECTROMAG25", "ELECTROMAG3", "FP64", "FP32", "FP64_FAST",
           "SeidartError", "UnstableError", "Problem", "Solver", "run", "layout",
           "MODEL_SLOTS", "SRC_SLOTS", "FIELD_SLOTS"]
