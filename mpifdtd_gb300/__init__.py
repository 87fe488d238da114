"""mpifdtd_gb300 -- GB300 (sm_103a) engine for rennone/mpiFDTD's UPML time-stepping path.

The CUDA engine is a C-ABI shared library (include/mpifdtd_gb300.h); this
package builds it in-tree and binds it with ctypes.  The reference's own entry
points (mpi_fdtdTM_upml_get*, ...) are provided by the drop-in library
libmpifdtd_upml.so (include/mpifdtd_upml.h).
"""
from .engine import (F32, F64, LAYOUT_GLOBAL, LAYOUT_SOLVER, MODEL_CIRCLE, MODEL_MORPHO, MODEL_NONE, MODEL_ZIGZAG,  # noqa: F401
                     MPI_TE_UPML_2D, MPI_TM_UPML_2D, OPT_NTFF_BLOCK, OPT_NTFF_CHUNK, OPT_NTFF_MODE, OPT_ROWS, OPT_TBLOCK,
                     OPT_DFT_STRIDE, OPT_TBLOCK_COLS, OPT_TBLOCK_ROWS, SOLVERS, STATUS_NONFINITE, STATUS_NTFF_RANGE, TE_UPML_2D,
                     TM_UPML_2D, Batch, FdtdError, FieldInfo, Simulation, geometry_of, load)

__all__ = ["Simulation", "Batch", "FieldInfo", "FdtdError", "geometry_of", "load", "SOLVERS"]
