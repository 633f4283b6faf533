"""Oracle for the skewer stage: box read along skewers, missing small-scale power, FGPA.

Restates bin/make_spectra.py (ComputeWeight :39-62, computeRho :66-68, ReadSpec
:90-139), bin/merge_spectra.py (small-scale loop :303-331, nz rule :308-309, growth
:91 and :296, FGPA :336-339), py/SaclayMocks/util.py (fgrowth :123-134, fgpa
:421-433, sigma_p1d :372-398, InterpP1Dmissing :448-474).  The trilinear read has no
reference code: it is the read the configs ask for, defined here on the same
cell-centred grid as ComputeWeight (centre of cell i at (i+0.5)*DX, :54-55) with
periodic wrap.  TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).
"""
from __future__ import annotations

import numpy as np

OMEGA_M_0 = 0.31457          # py/SaclayMocks/constant.py:23
LYA = 1215.67                # py/SaclayMocks/constant.py:12


# ----------------------------------------------------------------------------- geometry
def skewer_positions(start, direction, npix: int, dpix: float) -> np.ndarray:
    """Pixel positions p_i = start + i * dpix * direction, i = 0..npix-1 (float64)."""
    t = np.arange(npix, dtype=np.float64) * dpix
    return np.asarray(start, np.float64)[None, :] + t[:, None] * np.asarray(direction, np.float64)[None, :]


def trilinear(box: np.ndarray, pos: np.ndarray, dcell: float) -> np.ndarray:
    """Trilinear read of a periodic box at corner-frame positions ``pos`` [..., 3]
    (float64 arithmetic, float32 box).  Cell i is centred at (i+0.5)*dcell."""
    NX, NY, NZ = box.shape
    u = pos / dcell - 0.5
    i0 = np.floor(u).astype(np.int64)
    f = u - i0
    out = np.zeros(pos.shape[:-1])
    for cx in (0, 1):
        wx = f[..., 0] if cx else 1 - f[..., 0]
        ix = (i0[..., 0] + cx) % NX
        for cy in (0, 1):
            wy = f[..., 1] if cy else 1 - f[..., 1]
            iy = (i0[..., 1] + cy) % NY
            for cz in (0, 1):
                wz = f[..., 2] if cz else 1 - f[..., 2]
                iz = (i0[..., 2] + cz) % NZ
                out += wx * wy * wz * box[ix, iy, iz]
    return out


def gauss343(boxes: list, pos: np.ndarray, dcell: float, dmax: int = 3) -> list:
    """Gaussian-weighted read of ReadSpec (bin/make_spectra.py:39-68, 104-112): for the
    cell holding p, weights exp(-|r_c - p|^2 / (2 dcell^2)) over the (2*dmax+1)^3 cells
    around it, result sum(w*rho)/sum(w).  ``pos`` is in the corner frame, i.e. the
    reference's (X+LX/2, Y+LY/2, Z+LZ/2-R0) (:47-49); indices wrap periodically (the
    reference reads a halo instead, which gives the same values inside the box)."""
    NX, NY, NZ = boxes[0].shape
    sig2 = 2.0 * dcell * dcell
    r = np.arange(-dmax, dmax + 1)
    cx, cy, cz = np.meshgrid(r, r, r, indexing="ij")
    cells = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1)          # (343, 3)
    grid = cells * dcell
    outs = [np.zeros(len(pos)) for _ in boxes]
    for n, p in enumerate(pos):
        ixyz = (p // dcell).astype(np.int64)
        centre = (ixyz + 0.5) * dcell
        xx = (grid + centre - p) ** 2
        w = np.exp(-(xx[:, 0] + xx[:, 1] + xx[:, 2]) / sig2)
        li = (cells + ixyz) % np.array([NX, NY, NZ])
        for b, box in enumerate(boxes):
            rho = box[li[:, 0], li[:, 1], li[:, 2]]
            outs[b][n] = (w * rho).sum() / w.sum()
    return outs


def eta_par_projection(eta6: dict, rvec: np.ndarray) -> np.ndarray:
    """r_i r_j eta_ij / r^2 with r the observer->pixel vector (bin/make_spectra.py:114-129)."""
    X, Y, Z = rvec[..., 0], rvec[..., 1], rvec[..., 2]
    RR = X ** 2 + Y ** 2 + Z ** 2
    return (X * eta6["xx"] * X + Y * eta6["yy"] * Y + Z * eta6["zz"] * Z
            + 2 * X * eta6["xy"] * Y + 2 * X * eta6["xz"] * Z + 2 * Y * eta6["yz"] * Z) / RR


# ----------------------------------------------------------------------------- small scales
def nz_rule(length: int) -> int:
    """FFT length of the small-scale field: 256 * 2^n >= length + 50 (merge_spectra.py:308-309)."""
    nz = 256
    while nz < length + 50:
        nz *= 2
    return nz


def pmiss_analytic(k, amp: float = 0.05, kscale: float = 2.0):
    """P1D_miss(k) = amp * exp(-(k/kscale)^2) of the production config."""
    return amp * np.exp(-(np.asarray(k, np.float64) / kscale) ** 2)


def small_scale_scale(nz: int, pixsize: float, pmiss) -> np.ndarray:
    """sqrt(max(P1Dmiss(k),0)/pixsize) at k = rfftfreq(nz)*2*k_ny (merge_spectra.py:312-320;
    negative P1Dmiss is clipped as in the non-fit branch :319)."""
    k = np.fft.rfftfreq(nz) * 2 * (np.pi / pixsize)
    return np.sqrt(np.maximum(pmiss(k), 0.0) / pixsize)


def small_scales(noise: np.ndarray, length: int, scale: np.ndarray) -> np.ndarray:
    """delta_s = irfft(rfft(noise) * scale)[:length] in float64 (merge_spectra.py:310-322)."""
    return np.fft.irfft(np.fft.rfft(noise) * scale, n=len(noise))[:length]


# ----------------------------------------------------------------------------- FGPA
def fgrowth(z, Om0: float = OMEGA_M_0, unnormed: bool = False):
    """Linear growth factor normalised at z=0 (py/SaclayMocks/util.py:123-134)."""
    Om = 1 / (1 + (1 - Om0) / (Om0 * (1 + z) ** 3))
    Ol = 1 - Om
    a = 1 / (1 + z)
    norm = 1.0 if unnormed else 1.0 / fgrowth(0.0, Om0, unnormed=True)
    return norm * (5. / 2.) * a * Om / (Om ** (4. / 7.) - Ol + (1. + Om / 2.) * (1. + Ol / 70.))


def growth_merge(z, Om0: float = OMEGA_M_0):
    """G(z) = fgrowth(2.4) * (1+2.4) / (1+z) as bin/merge_spectra.py:91, 296 apply it."""
    return fgrowth(2.4, Om0) * (1 + 2.4) / (1 + z)


def fgpa(delta, eta_par, growthf, a, b, c):
    """F = exp(-a exp(b G (delta + c eta_par))) (py/SaclayMocks/util.py:421-433)."""
    tau_over_a = np.exp(b * growthf * (delta + c * eta_par))
    return np.exp(-a * tau_over_a)


def a_powerlaw(z, a0: float = 0.1, zref1: float = 3.2, power: float = 4.5):
    """a(z) = a0 * ((1+z)/zref1)^power of the production config."""
    return a0 * ((1 + np.asarray(z, np.float64)) / zref1) ** power


def z_along_x(x, lx: float, z_lo: float = 1.8, z_hi: float = 3.6):
    """Redshift mapped linearly along the box x axis (production config)."""
    xw = np.mod(x, lx)
    return z_lo + (z_hi - z_lo) * xw / lx


def sigma_p1d(pmiss, pixel: float = 0.2, N: int = 10000) -> float:
    """Analytic sigma of delta_s for a P1Dmiss function (py/SaclayMocks/util.py:372-398)."""
    L = N * pixel
    kj = 2 * np.pi / L * np.arange(1, N / 2)
    var_s = 2 * pmiss(kj).sum() / L
    var_s += pmiss(0) / L
    var_s += pmiss(np.pi / pixel) / L
    return float(np.sqrt(var_s))


def interp_table(ztab, ytab, z):
    """Linear interpolation on a table, raising outside it (util.InterpFitsTable :300-314)."""
    z = np.asarray(z)
    if z.min() < ztab.min() or z.max() > ztab.max():
        raise ValueError("redshift out of the table range")
    return np.interp(z, ztab, ytab)


# ----------------------------------------------------------------------------- pipeline
def skewer_flux(delta_box, eta_box, skewers: dict, dcell: float, *, dpix: float,
                fgpa_mode: dict, small: dict | None = None, noise1d=None, pitch=None):
    """Reference pipeline for a synthetic skewer list (float64 throughout).

    skewers: dict(start [n,3], dir [n,3], npix [n]) in the corner frame (Mpc/h).
    fgpa_mode: {"kind": "const", a, b, c} or {"kind": "powerlaw_x", a0, zref1, power,
               b, c, z_lo, z_hi}; optional "G": "one" | "merge".
    small: None, or {"pixsize", "nz" (int or "rule"), "pmiss" (callable)} with
           noise1d[s] the white noise of skewer s (length nz of that skewer).
    Returns dict(F=list of float64 arrays, delta=..., eta=..., z=...).
    """
    NX = delta_box.shape[0]
    lx = NX * dcell
    out = {"F": [], "delta": [], "eta": [], "z": [], "delta_s": []}
    scale_cache = {}
    for s in range(len(skewers["npix"])):
        n = int(skewers["npix"][s])
        pos = skewer_positions(skewers["start"][s], skewers["dir"][s], n, dpix)
        dl = trilinear(delta_box, pos, dcell)
        et = trilinear(eta_box, pos, dcell) if eta_box is not None else np.zeros(n)
        ds = np.zeros(n)
        if small is not None:
            nz = nz_rule(n) if small["nz"] == "rule" else int(small["nz"])
            if nz not in scale_cache:
                scale_cache[nz] = small_scale_scale(nz, small["pixsize"], small["pmiss"])
            ds = small_scales(np.asarray(noise1d[s], np.float64), n, scale_cache[nz])
        z = z_along_x(pos[:, 0], lx, fgpa_mode.get("z_lo", 1.8), fgpa_mode.get("z_hi", 3.6))
        G = growth_merge(z) if fgpa_mode.get("G", "one") == "merge" else np.ones(n)
        if fgpa_mode["kind"] == "const":
            a, b, c = fgpa_mode["a"], fgpa_mode["b"], fgpa_mode["c"]
        else:
            a = a_powerlaw(z, fgpa_mode["a0"], fgpa_mode["zref1"], fgpa_mode["power"])
            b, c = fgpa_mode["b"], fgpa_mode["c"]
        out["F"].append(fgpa(dl + ds, et, G, a, b, c))
        out["delta"].append(dl)
        out["eta"].append(et)
        out["z"].append(z)
        out["delta_s"].append(ds)
    return out


def merge_spectra_loop(spectra: list, rs: np.random.RandomState, *, pixsize: float = 0.2,
                       pmiss_fit=None, ptab: dict | None = None, abc=(0.1, 1.6, 0.5),
                       rsd: bool = True, addnoise: bool = True, lylimit: float = 0.0):
    """The per-spectrum loop of bin/merge_spectra.py (:303-339) in float64.

    spectra: list of dicts (wav, delta_l, eta_par, z, zq) in the loop's order, wavelengths
    ascending.  rs: the RandomState the loop draws from (np.random.seed(seed + i), :75-79).
    pmiss_fit: callable P1Dmiss(k) of the --fit-p1d branch (no clip, no sigma rescale); else
    ptab = dict(z, k, pk, sigma) of the default branch (util.InterpP1Dmissing, util.py:448-474:
    nearest-z table, linear in k; negative values clipped, :319; delta_s rescaled by
    sigma(z)/sigma(zeff), :324-325).  abc: a, b, c scalars or callables of z.
    A spectrum without forest pixels (lylimit < lambda/(1+zq) < lya) draws nothing and gets
    delta_s = 0 (:327-330).  Returns (flux list, delta_s list).
    """
    fl, dsl = [], []
    for sp in spectra:
        wav = np.asarray(sp["wav"], np.float64)
        z = np.asarray(sp["z"])
        n = len(wav)
        dl = np.asarray(sp["delta_l"], np.float64)
        ds = np.zeros(n)
        if addnoise:
            wav_rf = wav / (1 + sp["zq"])
            mmm = np.where((wav_rf < LYA) & (wav_rf > lylimit))[0]
            if len(mmm) > 0:
                nz = nz_rule(n)
                noise = rs.normal(size=nz)
                k = np.fft.rfftfreq(nz) * 2 * (np.pi / pixsize)
                zeff = z[mmm].mean()
                if pmiss_fit is not None:
                    pm = np.asarray(pmiss_fit(k), np.float64)
                else:
                    iz = np.argsort(np.abs(np.asarray(ptab["z"]) - zeff))[0]
                    pm = np.interp(k, ptab["k"], ptab["pk"][iz])
                    pm[pm < 0] = 0
                ds = np.fft.irfft(np.fft.rfft(noise) * np.sqrt(pm / pixsize), n=nz)[:n]
                if pmiss_fit is None and ptab.get("sigma") is not None:
                    ds = ds * np.interp(z, ptab["z"], ptab["sigma"]) / np.interp(zeff, ptab["z"], ptab["sigma"])
        a, b, c = (p(z) if callable(p) else p for p in abc)
        G = growth_merge(np.asarray(z, np.float64))
        eta = np.asarray(sp["eta_par"], np.float64) if rsd else 0.0
        fl.append(fgpa(dl + ds, eta, G, a, b, c))
        dsl.append(ds)
    return fl, dsl


def merge_forest(sp: dict, lylimit: float = 0.0) -> np.ndarray:
    """Indices of the forest pixels of a spectrum: lylimit < lambda/(1+zq) < lya
    (bin/merge_spectra.py:305-306)."""
    wav_rf = np.asarray(sp["wav"], np.float64) / (1 + sp["zq"])
    return np.where((wav_rf < LYA) & (wav_rf > lylimit))[0]
