"""Import shims that let the reference's own Python run in this container.

Used only by ``make_golden.py`` when the fixtures are regenerated.  The reference
(igmhub/SaclayMocks, pure Python) needs pyfftw, numba, fitsio, healpy, iminuit,
matplotlib and h5py, none of which is installed, and it uses numpy aliases that
scipy 1.18 no longer exports (``sp.pi``, ``sp.array``...).  Each shim reproduces
the published semantics of the missing call closely enough for the hot path:

* ``pyfftw.FFTW`` (r2c forward / c2r backward, both unnormalised, FFTW convention)
  -> numpy.fft in float64, result rounded to the output array's dtype;
* ``pyfftw.interfaces.numpy_fft`` -> numpy.fft (``threads=`` dropped);
* ``numba.jit`` -> identity decorator (the jitted code runs as plain Python);
* ``fitsio`` -> reads real FITS files with ``saclaymocks_gb300.fits``; writes are
  captured in ``FITS_CAPTURE`` instead of touching the disk; reads of names listed
  in ``FITS_SERVE`` return the served object (used to feed a P(k) grid file and
  synthetic spectra files);
* ``healpy.ang2pix`` -> pixel 0 for every object (one healpix pixel).
"""
from __future__ import annotations

import ast
import os
import sys
import types

import numpy as np

# checkout of the reference (igmhub/SaclayMocks), from SACLAYMOCKS_REF or make_golden.py --ref
REF = os.environ.get("SACLAYMOCKS_REF", "")
REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)

from saclaymocks_gb300 import fits as _fits  # noqa: E402

FITS_CAPTURE: dict = {}
FITS_SERVE: dict = {}


# ----------------------------------------------------------------------------- pyfftw
class _FFTW:
    def __init__(self, a, b, axes=(0, 1, 2), direction="FFTW_FORWARD", threads=1, flags=()):
        self.a, self.b, self.axes, self.direction = a, b, tuple(axes), direction

    def execute(self):
        if self.direction == "FFTW_FORWARD":
            res = np.fft.rfftn(self.a.astype(np.float64), axes=self.axes)
        else:
            s = [self.b.shape[ax] for ax in self.axes]
            res = np.fft.irfftn(self.a.astype(np.complex128), s=s, axes=self.axes)
            res *= float(np.prod(s))
        self.b[...] = res.astype(self.b.dtype)
        return self.b


def _np_fft_wrapper(name):
    f = getattr(np.fft, name)

    def g(*args, threads=None, **kw):
        return f(*args, **kw)
    return g


# ----------------------------------------------------------------------------- fitsio
class _HDUProxy:
    def __init__(self, owner, key):
        self.owner, self.key = owner, key

    def write_key(self, name, value, comment=""):
        self.owner.record["hdus"][self.key]["header"][name] = value

    def read(self):
        return self.owner.served[self.key]["data"]

    def read_header(self):
        return self.owner.served[self.key].get("header", {})


class _FITS:
    def __init__(self, path, mode="r", clobber=False):
        self.path = os.path.expandvars(path)
        self.served = None
        base = os.path.basename(self.path)
        if base in FITS_SERVE:
            self.served = FITS_SERVE[base]
        elif "w" not in mode:
            hdus = _fits.read_fits(self.path)
            self.served = {}
            for i, h in enumerate(hdus):
                self.served[i] = {"data": h.data, "header": h.header}
                if h.name:
                    self.served[h.name] = self.served[i]
        self.record = {"hdus": []}
        if "w" in mode:
            FITS_CAPTURE[base] = self.record

    def write(self, data, header=None, extname=None, names=None):
        hdr = {}
        if isinstance(header, dict):
            hdr.update(header)
        elif isinstance(header, list):
            for item in header:
                hdr[item["name"]] = item["value"]
        if names is not None:
            data = dict(zip(names, data))
        self.record["hdus"].append({"data": data, "header": hdr, "extname": extname})

    def __getitem__(self, key):
        if self.served is not None:
            return _HDUProxy(self, key)
        if key == -1:
            key = len(self.record["hdus"]) - 1
        return _HDUProxy(self, key)

    def close(self):
        pass


def _fitsio_read(path, ext=None, **kw):
    path = os.path.expandvars(path)
    base = os.path.basename(path)
    if base in FITS_SERVE:
        obj = FITS_SERVE[base]
        if not isinstance(obj, dict):
            return obj
        v = obj[ext]
        return v["data"] if isinstance(v, dict) and "data" in v else v
    return _fits.read(path, ext)


def _fitsio_read_header(path, ext=0):
    return _fits.read_header(os.path.expandvars(path), ext)


# ----------------------------------------------------------------------------- install
def install():
    if not REF or not os.path.isdir(os.path.join(REF, "py", "SaclayMocks")):
        raise SystemExit("set SACLAYMOCKS_REF (or make_golden.py --ref) to a checkout of igmhub/SaclayMocks")
    import scipy
    for name in ("pi", "array", "exp", "ones_like", "zeros_like", "sqrt", "indices",
                 "arange", "log", "zeros", "ones", "cos", "sin", "mean", "where",
                 "concatenate", "float32", "int32", "float64", "log10", "absolute", "power",
                 "interp", "radians", "degrees", "arctan", "tan", "floor"):
        if not hasattr(scipy, name):
            setattr(scipy, name, getattr(np, name))
    scipy.save = lambda *a, **k: None          # only ever used for FFTW wisdom files
    scipy.load = np.load
    scipy.random = np.random
    sys.modules["scipy.random"] = np.random
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid

    pyfftw = types.ModuleType("pyfftw")
    pyfftw.FFTW = _FFTW
    pyfftw.empty_aligned = lambda shape, dtype="float32", n=None: np.empty(shape, dtype=dtype)
    pyfftw.export_wisdom = lambda: ()
    pyfftw.import_wisdom = lambda w: None
    interfaces = types.ModuleType("pyfftw.interfaces")
    npfft = types.ModuleType("pyfftw.interfaces.numpy_fft")
    for n in ("rfftn", "irfftn", "rfft", "irfft", "fft", "ifft", "fftn", "ifftn"):
        setattr(npfft, n, _np_fft_wrapper(n))
    interfaces.numpy_fft = npfft
    pyfftw.interfaces = interfaces
    sys.modules.update({"pyfftw": pyfftw, "pyfftw.interfaces": interfaces,
                        "pyfftw.interfaces.numpy_fft": npfft})

    numba = types.ModuleType("numba")

    def jit(*args, **kw):
        if len(args) == 1 and callable(args[0]) and not kw:
            return args[0]
        return lambda f: f
    numba.jit = jit
    sys.modules["numba"] = numba

    fitsio = types.ModuleType("fitsio")
    fitsio.FITS = _FITS
    fitsio.FITSHDR = dict
    fitsio.read = _fitsio_read
    fitsio.read_header = _fitsio_read_header
    sys.modules["fitsio"] = fitsio

    hp = types.ModuleType("healpy")
    hp.ang2pix = lambda nside, theta, phi, nest=True: np.zeros(np.shape(theta), dtype=np.int64)
    sys.modules["healpy"] = hp
    for name in ("iminuit", "h5py", "matplotlib", "matplotlib.pyplot"):
        sys.modules[name] = types.ModuleType(name)
    sys.modules["iminuit"].Minuit = None
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]

    os.environ["SACLAYMOCKS_BASE"] = REF
    if os.path.join(REF, "py") not in sys.path:
        sys.path.insert(0, os.path.join(REF, "py"))


def load_script(name: str) -> types.ModuleType:
    """Import ``bin/<name>.py`` of the reference as a module (its ``main`` is not run)."""
    path = os.path.join(REF, "bin", name + ".py")
    mod = types.ModuleType("ref_" + name)
    mod.__file__ = path
    src = open(path).read()
    exec(compile(src, path, "exec"), mod.__dict__)
    return mod


def load_nested(script: str, outer: str, names: tuple) -> dict:
    """Compile the functions ``names`` that the reference defines inside ``outer`` of
    ``bin/<script>.py`` (e.g. ReadSpec inside make_spectra.main) into one namespace."""
    import scipy
    path = os.path.join(REF, "bin", script + ".py")
    tree = ast.parse(open(path).read(), path)
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == outer)
    defs = [n for n in fn.body if isinstance(n, ast.FunctionDef) and n.name in names]
    mod = ast.Module(body=defs, type_ignores=[])
    ns = {"np": np, "sp": scipy, "sys": sys, "jit": sys.modules["numba"].jit}
    exec(compile(mod, path, "exec"), ns)
    return ns
