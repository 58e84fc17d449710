"""GB300-native reconstruction path of a tomographic diffractive microscope.

Off-axis hologram extraction, Volkov phase unwrapping, aberration correction,
Born/Rytov fields and Ewald-cap mapping with the 3D inverse FFT, as sm_103a
CUDA kernels behind the C ABI declared in include/tdm.h.
"""
from .api import (  # noqa: F401
    Batch, Context, Derived, Geometry, TdmError, derive, extract_string, extract_val, lib, read_geom, read_pgm,
    write_tiff,
)
