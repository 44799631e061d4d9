"""GB300-native VL+CT MHD step (drop-in for Enzo-E's Method "mhd_vlct").

The numerics live in libmhdvlct_gb300.so (CUDA for sm_103a behind a C ABI,
include/mhdvlct_gb300.h).  This package is the Python side of that boundary:
ctypes bindings, a device-resident block container, the Method mirror and the
synthetic initial conditions.
"""
from . import capi  # noqa: F401
from .capi import MhdError  # noqa: F401

__all__ = ["capi", "MhdError"]
