"""Lines of sight of make_spectra from a QSO catalogue (host side, numpy).

Restates bin/make_spectra.py:286-321 (the pixel grid in comoving distance, its wavelength and
redshift, the cut below lambda_min) and :384-472 (per quasar: position from (RA, DEC, z),
slice cut, forest limits imin/imax), with the distance-redshift tables of util.cosmo
(py/SaclayMocks/util.py:793-833) and box.ComputeXYZ2 (py/SaclayMocks/box.py:240-250).  The
result is a skewer table in the box-corner frame for ``smk_skewers_flux`` (FP64 start points
and directions) plus, per quasar, its slice of the common pixel grid, so the Gaussian 7^3 read
of every quasar runs in one GPU launch.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# py/SaclayMocks/constant.py
C_KMS = 299792.458            # speed of light, km/s (scipy.constants.speed_of_light / 1000)
LYA = 1215.67
LYLIMIT = 0.0
LAMBDA_MIN = 3476.0
H = 0.6731
OMEGA_M_0 = 0.31457
OMEGA_K_0 = 0.0
Z0 = 1.70975268202


class Cosmo:
    """Comoving distance tables of util.cosmo: hubble(z) on 10000 bins of dz = 1e-3 up to z = 10,
    chi by the cumulative trapezoid rule, linear interpolation both ways (Mpc, H0 in km/s/Mpc)."""

    def __init__(self, Om=OMEGA_M_0, Ok=OMEGA_K_0, Or=0.0, wl=-1.0, H0=100.0 * H):
        Ol = 1.0 - Ok - Om - Or
        nbins, zmax = 10000, 10.0
        dz = zmax / nbins
        z = np.arange(nbins) * dz
        hub = H0 * np.sqrt(Ol * (1.0 + z) ** (3.0 * (1.0 + wl)) + Ok * (1.0 + z) ** 2 + Om * (1.0 + z) ** 3
                           + Or * (1.0 + z) ** 4)
        inc = C_KMS * (1.0 / hub[:-1] + 1.0 / hub[1:]) / 2.0 * dz
        chi = np.concatenate([[0.0], np.cumsum(inc)])        # the sequential sum of the loop
        self.z, self.chi, self.hub = z, chi, hub

    @staticmethod
    def _lin(x, xp, fp):
        x = np.asarray(x, np.float64)
        if np.any(x < xp[0]) or np.any(x > xp[-1]):
            raise ValueError("value outside the interpolation range")   # interp1d's bounds_error
        return np.interp(x, xp, fp)

    def r_comoving(self, z):
        return self._lin(z, self.z, self.chi)

    def r_2_z(self, r):
        return self._lin(r, self.chi, self.z)

    def dist_hubble(self, z):
        return self._lin(z, self.z, C_KMS / self.hub)


def compute_xyz2(ra, dec, R, ra0, dec0):
    """Observer-frame position of (ra, dec, R) for a box centred on (ra0, dec0), radians
    (box.ComputeXYZ2)."""
    x = R * (np.cos(ra0) * np.cos(dec) * np.sin(ra) - np.sin(ra0) * np.cos(dec) * np.cos(ra))
    y = R * (-np.sin(ra0) * np.sin(dec0) * np.cos(dec) * np.sin(ra) + np.cos(dec0) * np.sin(dec)
             - np.cos(ra0) * np.sin(dec0) * np.cos(dec) * np.cos(ra))
    z = R * (np.cos(dec0) * np.sin(ra0) * np.cos(dec) * np.sin(ra) + np.sin(dec0) * np.sin(dec)
             + np.cos(ra0) * np.cos(dec0) * np.cos(dec) * np.cos(ra))
    return x, y, z


@dataclass
class PixelGrid:
    """The pixel grid shared by every line of sight (bin/make_spectra.py:306-321)."""
    R: np.ndarray          # comoving distance of each pixel, Mpc/h
    lam: np.ndarray        # wavelength lya (1 + z(R)), Angstrom
    R0: float              # distance of the box centre, Mpc/h


def pixel_grid(cosmo: Cosmo, zmin: float, zmax: float, pixel: float) -> PixelGrid:
    R0 = H * cosmo.r_comoving(Z0)
    Rmin = H * cosmo.r_comoving(zmin)
    Rmax = H * cosmo.r_comoving(zmax)
    n = int((Rmax - Rmin) / pixel + 0.5)
    R = Rmin + np.arange(n) * pixel
    lam = LYA * (1 + cosmo.r_2_z(R / H))
    cut = lam > LAMBDA_MIN
    return PixelGrid(R=R[cut], lam=lam[cut], R0=float(R0))


@dataclass
class QsoLines:
    """Lines of sight of one slice: for quasar q (row qso_index[q] of the catalogue) the pixels
    [r0[q], r0[q] + npix[q]) of the grid, of which [imin[q], imax[q]) (relative) are read."""
    qso_index: np.ndarray   # [n] int64
    r0: np.ndarray          # [n] int64 first grid pixel in the slice
    npix: np.ndarray        # [n] int32 pixels in the slice
    imin: np.ndarray        # [n] int32
    imax: np.ndarray        # [n] int32
    unit: np.ndarray        # [n, 3] float64 unit vector observer -> quasar
    zqso: np.ndarray        # [n] float64 redshift used (Z_QSO_RSD with RSD, else Z_QSO_NO_RSD)


def qso_lines(cosmo: Cosmo, grid: PixelGrid, qsos, ra0: float, dec0: float, box_len, dx: float,
              n_hdu: int, i_slice: int, n_slice: int, zmin: float, zmax: float, rsd: bool = True,
              nqso_max: int = -1) -> QsoLines:
    """The per-quasar loop of bin/make_spectra.py:429-472 without the read.  box_len = (LX, LY,
    LZ) with LX = dx * n_hdu; qsos a structured array with RA, DEC (degrees), Z_QSO_RSD,
    Z_QSO_NO_RSD."""
    LX, LY, LZ = (float(v) for v in box_len)
    R0 = grid.R0
    x_lo = LX * i_slice / n_slice - LX / 2
    x_hi = LX * (i_slice + 1) / n_slice - LX / 2
    if i_slice >= n_slice // 2:
        tanx_max = (dx * (n_hdu / n_slice) * (i_slice + 1) - LX / 2) / (R0 - LZ / 2)
    else:
        tanx_max = abs((dx * (n_hdu / n_slice) * i_slice - LX / 2) / (R0 - LZ / 2))
    out = {k: [] for k in ("qso_index", "r0", "npix", "imin", "imax", "unit", "zqso")}
    kept = 0
    for q in range(len(qsos)):
        if nqso_max > 0 and kept >= nqso_max:
            break
        zq = float(qsos["Z_QSO_RSD"][q] if rsd else qsos["Z_QSO_NO_RSD"][q])
        Rq = H * float(cosmo.r_comoving(zq)) if 0.0 <= zq <= cosmo.z[-1] else np.nan
        if not np.isfinite(Rq):
            continue
        X, Y, Z = compute_xyz2(np.radians(float(qsos["RA"][q])), np.radians(float(qsos["DEC"][q])), Rq,
                               np.radians(ra0), np.radians(dec0))
        if abs(X / Z) > tanx_max:
            continue
        if zq < zmin or zq > zmax:
            continue
        sel = np.nonzero((grid.R * X / Rq > x_lo) & (grid.R * X / Rq <= x_hi))[0]
        if len(sel) < 1:
            continue
        lam = grid.lam[sel]
        a = np.nonzero(lam > LYLIMIT * (1 + zq))[0]
        imin = a[0] if len(a) else len(lam)
        b = np.nonzero(lam < LYA * (1 + zq))[0]
        imax = b[-1] + 1 if len(b) else 0
        kept += 1
        out["qso_index"].append(q)
        out["r0"].append(sel[0])
        out["npix"].append(len(sel))
        out["imin"].append(imin)
        out["imax"].append(imax)
        out["unit"].append(np.array([X, Y, Z]) / Rq)
        out["zqso"].append(zq)
    return QsoLines(qso_index=np.array(out["qso_index"], np.int64), r0=np.array(out["r0"], np.int64),
                    npix=np.array(out["npix"], np.int32), imin=np.array(out["imin"], np.int32),
                    imax=np.array(out["imax"], np.int32),
                    unit=np.array(out["unit"], np.float64).reshape(-1, 3),
                    zqso=np.array(out["zqso"], np.float64))
