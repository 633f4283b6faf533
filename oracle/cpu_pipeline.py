"""The reference's CPU path restated for timing (bench.py's CPU baseline and reference arm).
TEST INFRASTRUCTURE ONLY.

The reference itself cannot run on the GPU machine (pyfftw, numba, fitsio, healpy and iminuit are
absent, and numpy 2 / scipy 1.18 break its imports), so this port times the same algorithm
with the fastest CPU libraries present:

* white noise: numpy's legacy MT19937 normal drawn plane by plane, as bin/make_boxes.py:46-48
  (single thread, exactly the reference's generator);
* 3D r2c / c2r: scipy.fft (pocketfft) in float32 on all host threads (the reference uses FFTW
  with -ncpu threads, bin/make_boxes.py:53, :87);
* sqrt(P/Vcell) multiply and kz^2/k^2 split in float32 numpy (bin/make_boxes.py:290, :350);
* small scales: batched scipy.fft rfft/irfft per skewer length class on all threads
  (bin/merge_spectra.py:308-322), legacy normal noise per skewer;
* trilinear read + FGPA: the C oracle with OpenMP over skewers (oracle/csrc/skewers_ref.c).
"""
from __future__ import annotations

import os
import time

import numpy as np
import scipy.fft as sfft

from . import cskewers, grf, skewers


def grf_cpu(nx, ny, nz, dcell, seed, k0=0.02, workers=None):
    """delta and eta_zz (float32, padded [nx, ny, 2*(nz//2+1)] rows) on the CPU; returns
    (delta_pad, eta_pad, seconds by stage)."""
    workers = workers or os.cpu_count()
    t = {}
    t0 = time.perf_counter()
    noise = grf.draw_noise(nx, ny, nz, seed)
    t["noise"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    nk = sfft.rfftn(noise, workers=workers, overwrite_x=True)
    del noise
    t["r2c"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    P0 = grf.sqrt_pk_grid(nx, ny, nz, dcell, k0)
    kx, ky, kz = grf.k_components(nx, ny, nz, dcell)
    nk *= P0
    del P0
    ek = nk * grf.eta_factor("zz", kx, ky, kz)
    t["scale"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    delta = sfft.irfftn(nk, s=(nx, ny, nz), workers=workers, overwrite_x=True)  # includes 1/N
    eta = sfft.irfftn(ek, s=(nx, ny, nz), workers=workers, overwrite_x=True)
    t["c2r"] = time.perf_counter() - t0
    return delta.astype(np.float32, copy=False), eta.astype(np.float32, copy=False), t


def skewers_cpu(delta, eta, dcell, start, direction, npix, dpix, ss_nz, pmiss, seed,
                a0=0.1, zref1=3.2, power=4.5, b=1.58, c=0.6, workers=None):
    """Flux of every pixel (packed float32) with small scales on an ss_nz grid."""
    workers = workers or os.cpu_count()
    t = {}
    nx, ny, nz = delta.shape
    t0 = time.perf_counter()
    rs = np.random.RandomState(seed)
    nsk = len(npix)
    offset = np.concatenate([[0], np.cumsum(npix[:-1], dtype=np.int64)]).astype(np.int64)
    total = int(np.sum(npix, dtype=np.int64))
    ds = np.empty(total, np.float64)
    scale = skewers.small_scale_scale(ss_nz, 0.2, pmiss)
    chunk = 4096
    for s0 in range(0, nsk, chunk):
        s1 = min(nsk, s0 + chunk)
        noise = rs.normal(size=(s1 - s0, ss_nz))
        f = sfft.irfft(sfft.rfft(noise, axis=1, workers=workers) * scale, n=ss_nz, axis=1,
                       workers=workers)
        for j, s in enumerate(range(s0, s1)):
            ds[offset[s]:offset[s] + npix[s]] = f[j, :npix[s]]
    t["small_scales"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    F = cskewers.skewer_flux(start, direction, npix, offset, dpix, delta, eta, nz, dcell, ds=ds,
                             abc_mode=1, a=a0, b=b, c=c, zref1=zref1, power=power,
                             nthreads=workers)
    t["gather_fgpa"] = time.perf_counter() - t0
    return F, t
