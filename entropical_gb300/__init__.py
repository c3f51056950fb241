"""entropical_gb300 -- GB300-native (sm_103a) density hot path of lettis/entropical.

The compute path is the CUDA library built from ``csrc/`` and bound through
the C ABI in ``include/entropical_gb300.h``. This package is its host-side
mirror: the reference's density interface (``combined_densities``,
``epa_convolution``), the bandwidth estimators and the information measures
built on them. There is no CPU implementation of any of these here.
"""
from ._build import build, lib_path  # noqa: F401
from ._native import NativeError  # noqa: F401
from .densities import (COMPAT_NORM, Context, as_colmajor, combined_densities,  # noqa: F401
                        coords_file_shape, default_context, is_xtc, read_coords, write_xtc,
                        xtc_file_shape)

__all__ = [
    "build",
    "lib_path",
    "NativeError",
    "COMPAT_NORM",
    "Context",
    "as_colmajor",
    "combined_densities",
    "coords_file_shape",
    "read_coords",
    "is_xtc",
    "xtc_file_shape",
    "write_xtc",
    "default_context",
]
