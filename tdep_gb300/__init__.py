"""GB300 (sm_103a) implementation of the three/four-phonon scattering path of TDEP's
thermal_conductivity program, behind a C-ABI (include/tdep_gb300.h).

Python users drive it through tdep_gb300.scattering (Problem, Options, QLists,
ScatteringRates); Fortran or C callers bind the C-ABI directly.
"""
from .scattering import (KAPPA_AU_TO_SI, Options, Problem, QLists, ScatteringRates, device_count,  # noqa: F401
                         release_cached_memory, write_grid_hdf5, write_outfile)

__all__ = ["Problem", "Options", "QLists", "ScatteringRates", "write_outfile", "write_grid_hdf5", "device_count",
           "release_cached_memory",
           "KAPPA_AU_TO_SI"]
