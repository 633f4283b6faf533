"""Oracle for the reductions: 1D power spectrum estimator, profile histogram, mean flux.

Restates py/SaclayMocks/powerspectrum.py (P1D_1spectrum :204-208, ComputeP1D
:212-238), py/SaclayMocks/util.py (MakeProfileHisto :46-75) and the mean flux per
redshift window of analysis/compute_p1d.py:37-45 / transmissions.trans_of_z
(py/SaclayMocks/transmissions.py:98-118).  TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import numpy as np


def p1d_1spectrum(delta, dx: float):
    """|rfft(delta)|^2 * dx / len(delta) (powerspectrum.py:204-208)."""
    z = np.fft.rfft(np.asarray(delta, np.float64))
    return (z.real ** 2 + z.imag ** 2) * dx / len(delta)


def p1d_k(n: int, dx: float):
    """rfftfreq(n) * 2 * k_ny, k_ny = pi/dx (powerspectrum.py:231)."""
    return np.fft.rfftfreq(n) * 2 * (np.pi / dx)


def bin_index(x, edges):
    """scipy.stats.binned_statistic bin of each x: [e_i, e_i+1), last bin closed; -1 outside."""
    x = np.asarray(x)
    nb = len(edges) - 1
    idx = np.searchsorted(edges, x, side="right") - 1
    idx = np.where(x == edges[-1], nb - 1, idx)
    return np.where((idx >= 0) & (idx < nb), idx, -1)


def profile_histo(x, y, edges, err: bool = True):
    """Binned mean of y, with rms/sqrt(n) (err=True) or rms (err=False), empty bins dropped
    (util.py:46-75).  Returns (mean x, mean y, error) over non-empty bins."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    ok = ~(np.isnan(x) | np.isnan(y))
    x, y = x[ok], y[ok]
    nb = len(edges) - 1
    idx = bin_index(x, edges)
    m = idx >= 0
    cnt = np.bincount(idx[m], minlength=nb).astype(np.float64)
    sx = np.bincount(idx[m], x[m], nb)
    sy = np.bincount(idx[m], y[m], nb)
    sy2 = np.bincount(idx[m], y[m] ** 2, nb)
    keep = cnt > 0
    mx, my, my2 = sx[keep] / cnt[keep], sy[keep] / cnt[keep], sy2[keep] / cnt[keep]
    e = np.sqrt(np.maximum(my2 - my ** 2, 0))
    if err:
        e = e / np.sqrt(cnt[keep])
    return mx, my, e


def binned_p1d(spectra, dx: float, edges):
    """ComputeP1D: add every spectrum's (k, P) then profile_histo (powerspectrum.py:221-238)."""
    ks = np.concatenate([p1d_k(len(s), dx) for s in spectra])
    ps = np.concatenate([p1d_1spectrum(s, dx) for s in spectra])
    return profile_histo(ks, ps, edges)


def mean_flux_bins(F, z, edges):
    """Mean of F per redshift window [e_i, e_i+1) (analysis/compute_p1d.py:37-45);
    returns (mean, count) per bin (NaN mean where empty)."""
    F = np.concatenate(F) if isinstance(F, (list, tuple)) else np.asarray(F)
    z = np.concatenate(z) if isinstance(z, (list, tuple)) else np.asarray(z)
    idx = bin_index(z, edges)
    m = idx >= 0
    nb = len(edges) - 1
    cnt = np.bincount(idx[m], minlength=nb).astype(np.float64)
    s = np.bincount(idx[m], F[m].astype(np.float64), nb)
    with np.errstate(invalid="ignore", divide="ignore"):
        return s / cnt, cnt
