"""ctypes wrapper of the C oracle's skewer read + FGPA (oracle/csrc/skewers_ref.c).
TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import cbuild

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(cbuild.build())
        f = _lib.oracle_skewer_flux
        f.restype = None
        f.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                      C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                      C.c_double, C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double,
                      C.c_double, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_double,
                      C.c_void_p, C.c_int32]
    return _lib


def skewer_flux(start, direction, npix, offset, dpix, delta_pad, eta_pad, nz, dcell, *,
                ds=None, abc_mode=0, a=0.1, b=1.6, c=0.5, zref1=3.2, power=4.5, z_lo=1.8,
                z_hi=3.6, growth_mode=0, growth24=0.0, nthreads=None):
    """Flux of every pixel (packed float32) from padded float32 boxes [nx, ny, pitch]."""
    lib = _load()
    start = np.ascontiguousarray(start, np.float32)
    direction = np.ascontiguousarray(direction, np.float32)
    npix = np.ascontiguousarray(npix, np.int32)
    offset = np.ascontiguousarray(offset, np.int64)
    delta_pad = np.ascontiguousarray(delta_pad, np.float32)
    nx, ny, pitch = delta_pad.shape
    eta_pad = None if eta_pad is None else np.ascontiguousarray(eta_pad, np.float32)
    total = int(npix.astype(np.int64).sum())
    flux = np.empty(total, np.float32)
    ds = None if ds is None else np.ascontiguousarray(ds, np.float64)
    ptr = lambda x: None if x is None else x.ctypes.data  # noqa: E731
    lib.oracle_skewer_flux(len(npix), ptr(start), ptr(direction), ptr(npix), ptr(offset), float(dpix),
                           ptr(delta_pad), ptr(eta_pad), nx, ny, int(nz), pitch, float(dcell), ptr(ds),
                           int(abc_mode), a, b, c, zref1, power, z_lo, z_hi, int(growth_mode),
                           float(growth24), ptr(flux), int(nthreads or os.cpu_count() or 1))
    return flux
