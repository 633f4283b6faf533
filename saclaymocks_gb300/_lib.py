"""ctypes binding of libsmk.so (the C ABI declared in include/smk.h).

The library is loaded from ``saclaymocks_gb300/_build/libsmk.so`` (built in-tree by
``saclaymocks_gb300.build``).  There is no fallback: if the library is missing or does not
load, every entry point raises :class:`SmkError`.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

SMK_OK = 0
SMK_EINVAL = -1
SMK_ENOTSUPP = -2
SMK_ECUDA = -3
SMK_EWORKSPACE = -4
SMK_ENULLBOX = -5

SMK_NOISE_HOST, SMK_NOISE_PHILOX = 0, 1
SMK_PK_ANALYTIC, SMK_PK_GRID = 0, 1
SMK_INTERP_TRILINEAR, SMK_INTERP_PIXELS, SMK_INTERP_GAUSS343 = 0, 1, 2
SMK_SS_NONE, SMK_SS_HOST, SMK_SS_PHILOX = 0, 1, 2
SMK_ABC_CONST, SMK_ABC_POWERLAW, SMK_ABC_TABLE = 0, 1, 2
SMK_G_ONE, SMK_G_MERGE = 0, 1
SMK_SS_SET_FLOATS = 3973
SMK_ETA = {"zz": 0, "xx": 1, "yy": 2, "xy": 3, "xz": 4, "yz": 5, "vx": 6, "vy": 7, "vz": 8}
SMK_PASS_ZFWD, SMK_PASS_LINE, SMK_PASS_XPASS, SMK_PASS_XGEN, SMK_PASS_ZINV = 0, 1, 2, 3, 4


class SmkError(RuntimeError):
    """A libsmk call returned a non-zero status (``.status`` holds the code)."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class SmkGrfParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("batch", C.c_int32),
                ("dcell", C.c_double), ("pk_mode", C.c_int32), ("k0", C.c_double),
                ("amp", C.c_double), ("pk_grid", C.c_void_p), ("noise_mode", C.c_int32),
                ("noise", C.c_void_p), ("seed", C.c_uint64), ("want_eta", C.c_int32),
                ("pass_events", C.c_void_p), ("n_pass_events", C.c_int32), ("eta_comp", C.c_int32),
                ("vel_factor", C.c_double), ("xi_chunk_kz", C.c_int32)]


class SmkSkewers(C.Structure):
    _fields_ = [("n", C.c_int64), ("start", C.c_void_p), ("dir", C.c_void_p),
                ("npix", C.c_void_p), ("offset", C.c_void_p), ("dpix", C.c_double),
                ("order", C.c_void_p), ("n_slots", C.c_int64),
                ("pix_delta", C.c_void_p), ("pix_eta", C.c_void_p), ("pix_z", C.c_void_p),
                ("forest", C.c_void_p), ("start64", C.c_void_p), ("dir64", C.c_void_p)]


class SmkSpectraParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("pitch", C.c_int64),
                ("dcell", C.c_double), ("interp", C.c_int32), ("eta6", C.c_void_p * 6),
                ("obs", C.c_double * 3), ("ss_mode", C.c_int32), ("ss_nz", C.c_int32), ("ss_scale", C.c_void_p),
                ("ss_noise", C.c_void_p), ("ss_noise_offset", C.c_void_p), ("seed", C.c_uint64),
                ("abc_mode", C.c_int32), ("a", C.c_float), ("b", C.c_float), ("c", C.c_float),
                ("a_zref1", C.c_float), ("a_power", C.c_float), ("abc_tab", C.c_void_p),
                ("n_tab", C.c_int32), ("z_tab0", C.c_float), ("dz_tab", C.c_float),
                ("z_lo", C.c_float), ("z_hi", C.c_float), ("growth_mode", C.c_int32),
                ("growth24", C.c_float), ("ss_nztab", C.c_int32), ("ss_ztab", C.c_void_p),
                ("ss_zsigma", C.c_void_p), ("gauss_dmax", C.c_int32)]


class SmkFitProblem(C.Structure):
    _fields_ = [("delta", C.c_void_p), ("eta", C.c_void_p), ("G", C.c_void_p), ("zbin", C.c_void_p),
                ("offset", C.c_void_p), ("npix", C.c_void_p), ("order", C.c_void_p),
                ("n_slots", C.c_int64), ("n_total", C.c_int64), ("nzb", C.c_int32), ("nkb", C.c_int32),
                ("kedges", C.c_void_p), ("dx", C.c_double), ("chirp", C.c_void_p), ("chirp_off", C.c_void_p),
                ("n_max", C.c_int32), ("spectrum", C.c_void_p)]


# (name, restype, argtypes) of every exported entry point
_SIGS = [
    ("smk_strerror", C.c_char_p, [C.c_int]),
    ("smk_last_error", C.c_char_p, []),
    ("smk_version", C.c_int, []),
    ("smk_fft_supported", C.c_int, [C.c_int32]),
    ("smk_grf_pitch", C.c_int64, [C.c_int32]),
    ("smk_grf_box_floats", C.c_int64, [C.POINTER(SmkGrfParams)]),
    ("smk_grf_workspace_size", C.c_size_t, [C.POINTER(SmkGrfParams)]),
    ("smk_grf_boxes", C.c_int, [C.POINTER(SmkGrfParams), C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_size_t, C.c_void_p]),
    ("smk_grf_check", C.c_int, [C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double)]),
    ("smk_pk_normalisation", C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                       C.c_void_p, C.c_void_p]),
    ("smk_tune_count", C.c_int, [C.c_int32]),
    ("smk_tune_info", C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32)]),
    ("smk_tune_set", C.c_int, [C.c_int32, C.c_int32, C.c_int32]),
    ("smk_tune_get", C.c_int, [C.c_int32, C.c_int32]),
    ("smk_tune_flag", C.c_int, [C.c_int32, C.c_int32, C.c_void_p]),
    ("smk_skewer_schedule", C.c_int, [C.c_int64, C.c_void_p, C.c_int32, C.c_void_p,
                                      C.POINTER(C.c_int64)]),
    ("smk_skewers_workspace_size", C.c_size_t, [C.POINTER(SmkSkewers), C.POINTER(SmkSpectraParams)]),
    ("smk_skewers_flux", C.c_int, [C.POINTER(SmkSkewers), C.POINTER(SmkSpectraParams), C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_size_t, C.c_void_p]),
    ("smk_skewers_flux_static", C.c_int, [C.POINTER(SmkSkewers), C.c_void_p, C.POINTER(SmkSpectraParams),
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    ("smk_fit_schedule", C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    ("smk_fit_acc_len", C.c_int, [C.c_int32, C.c_int32]),
    ("smk_fit_bluestein_m", C.c_int, [C.c_int32]),
    ("smk_fit_chirps", C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("smk_fit_forward", C.c_int, [C.POINTER(SmkFitProblem), C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_size_t, C.c_void_p]),
    ("smk_fit_backward", C.c_int, [C.POINTER(SmkFitProblem), C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("smk_fgpa", C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p,
                           C.c_float, C.c_void_p, C.c_float, C.c_void_p, C.c_float, C.c_void_p,
                           C.c_void_p]),
]

EXPORTED = tuple(name for name, _, _ in _SIGS)

_lib = None


def library_path() -> str:
    return _build.LIB


def load(path: str | None = None):
    """Load libsmk.so once and declare the prototypes; raise SmkError if it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or _build.LIB
    if not os.path.exists(p):
        raise SmkError(SMK_ECUDA, f"libsmk.so not built ({p}); run saclaymocks_gb300.build.build() "
                       "or __graft_entry__.build() first")
    try:
        lib = C.CDLL(p)
    except OSError as e:
        raise SmkError(SMK_ECUDA, f"cannot load {p}: {e}") from e
    for name, res, args in _SIGS:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


SMK_TUNE_XGEN_SPLIT, SMK_TUNE_PREFETCH, SMK_TUNE_TMA, SMK_TUNE_TMA_WAIT_TEST = 0, 1, 3, 4
SMK_TUNE_SKEWER_BLOCKS = 5


def tune_flag(flag: int, value: int) -> int:
    """smk_tune_flag: set a process-wide switch; returns its previous value."""
    prev = C.c_int32(0)
    check(load().smk_tune_flag(int(flag), int(value), C.byref(prev)), "smk_tune_flag")
    return prev.value


def xgen_split(mode: int) -> int:
    """x-pass launch mode (-1 by footprint, 0 one launch, 1 two launches); returns the previous."""
    return tune_flag(SMK_TUNE_XGEN_SPLIT, mode)


def check(status: int, what: str = ""):
    """Raise SmkError for a non-zero status, with the library's message."""
    if status != SMK_OK:
        lib = load()
        msg = lib.smk_last_error().decode(errors="replace")
        name = lib.smk_strerror(status).decode(errors="replace")
        raise SmkError(status, f"{what}: {name}: {msg}" if what else f"{name}: {msg}")
