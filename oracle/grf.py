"""Oracle for the GRF step: white noise -> x sqrt(P/Vcell) -> c2r -> delta, eta_ij.

Restates bin/make_boxes.py (DrawGRF_boxk :40-72, P0 multiply :288-292,
FFTandStore :77-125, k grids :299-306, eta_ij :315-391) and the P-grid of
bin/interpolate_pk.py:23-26, 63-77 for the analytic spectrum of the configs,
P(k) = A * k / (1 + (k/k0)^2)^2 with A fixed so that E[var(delta)] = 1.
TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).
"""
from __future__ import annotations

import numpy as np

ETA_COMPONENTS = ("xx", "yy", "zz", "xy", "xz", "yz")


def draw_noise(NX: int, NY: int, NZ: int, seed: int) -> np.ndarray:
    """N(0,1) float32 box drawn plane by plane with the legacy MT19937 stream,
    exactly as bin/make_boxes.py:46-48 after np.random.seed(seed) (:170)."""
    rs = np.random.RandomState(seed)
    box = np.zeros((NX, NY, NZ), dtype=np.float32)
    for iz in range(NZ):
        box[:, :, iz] = np.float32(rs.normal(size=[NX, NY]))
    return box


def k_components(NX: int, NY: int, NZ: int, dcell: float):
    """float32 kx (NX,1,1), ky (NY,1), kz (NZ/2+1,) in h/Mpc: bin/make_boxes.py:299-303."""
    k_ny = np.pi / dcell
    kx = np.float32(np.fft.fftfreq(NX) * 2 * k_ny).reshape(-1, 1, 1)
    ky = np.float32(np.fft.fftfreq(NY) * 2 * k_ny).reshape(-1, 1)
    kz = np.float32(np.fft.rfftfreq(NZ) * 2 * k_ny)
    return kx, ky, kz


def pk_shape(k, k0: float):
    """Unnormalised analytic spectrum k / (1 + (k/k0)^2)^2 (P(0) = 0)."""
    k = np.asarray(k, dtype=np.float64)
    return k / (1.0 + (k / k0) ** 2) ** 2


def half_weights(NZ: int) -> np.ndarray:
    """Multiplicity of each kz plane of the half spectrum in the full spectrum."""
    w = np.full(NZ // 2 + 1, 2.0)
    w[0] = 1.0
    if NZ % 2 == 0:
        w[-1] = 1.0
    return w


def pk_normalisation(NX: int, NY: int, NZ: int, dcell: float, k0: float) -> float:
    """A such that E[var delta] = sum_k P(k) / Volume = 1 (full-grid sum, FP64).
    With the make_boxes normalisation (unnormalised r2c, c2r divided by N), the
    variance of delta is sum_{k != 0} P(k) / (N * Vcell)."""
    kx, ky, kz = k_components(NX, NY, NZ, dcell)
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    vcell = float(np.float32(dcell ** 3))
    s = float((pk_shape(k, k0) * half_weights(NZ)).sum())
    return NX * NY * NZ * vcell / s


def sqrt_pk_grid(NX: int, NY: int, NZ: int, dcell: float, k0: float, A: float | None = None):
    """float32 sqrt(P(k)/Vcell) on the half spectrum, as bin/interpolate_pk.py:23-26
    stores it (P rounded to float32, divided by float32 Vcell, float32 sqrt)."""
    if A is None:
        A = pk_normalisation(NX, NY, NZ, dcell, k0)
    kx, ky, kz = k_components(NX, NY, NZ, dcell)
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    P = np.float32(A * pk_shape(k, k0))
    vcell = np.float32(dcell ** 3)
    return np.float32(np.sqrt(P / vcell))


def eta_factor(comp: str, kx, ky, kz):
    """k_i k_j / k^2 in float32 with k^2[0,0,0] = 1: bin/make_boxes.py:305-306, 324-389."""
    kk = kx * kx + ky * ky + kz * kz
    kk[0, 0, 0] = 1
    ki = {"x": kx, "y": ky, "z": kz}
    return ki[comp[0]] * ki[comp[1]] / kk


VELOCITY_COMPONENTS = ("vx", "vy", "vz")


def velocity_factor(comp: str, kx, ky, kz, H0: float, dgrowth0: float):
    """-i k_i / k^2 * H0 * dD/dz(0) with numpy's promotion of the reference's expression
    (bin/make_boxes.py:393-431): complex64 up to the H0 product, complex128 after the
    float64 growth-rate scalar."""
    kk = kx * kx + ky * ky + kz * kz
    kk[0, 0, 0] = 1
    ki = {"vx": kx, "vy": ky, "vz": kz}[comp]
    return -1j * ki / kk * H0 * np.float64(dgrowth0)


def grf_boxes(noise: np.ndarray, dcell: float, k0: float = 0.02, A: float | None = None,
              eta=("zz",), precision: str = "f32") -> dict:
    """delta and eta_ij boxes from a white-noise box.

    precision="f32" reproduces the reference's arrays: forward r2c rounded to
    complex64 (:52-54), times the float32 P0 grid in complex64 (:290), c2r rounded to
    float32 then divided by N in float32 (:86-89).  precision="f64" keeps every step
    in float64 (the FP64 oracle the FP32 kernels are measured against).
    Returns dict(delta=..., eta_<ij>=..., sigma=std(delta) as float64).
    """
    NX, NY, NZ = noise.shape
    if NZ % 2:
        raise ValueError("NZ must be even (the c2r output length is 2*(NZ/2))")
    nk = np.fft.rfftn(noise.astype(np.float64))
    return grf_from_modes(nk, NZ, dcell, k0, A, eta, precision)


def grf_from_modes(nk: np.ndarray, NZ: int, dcell: float, k0: float = 0.02, A: float | None = None,
                   eta=("zz",), precision: str = "f32", P0=None, velocity=None) -> dict:
    """The GRF step from the (unnormalised) Fourier transform nk [NX, NY, NZ//2+1] of the
    white noise: everything of grf_boxes after the forward r2c.  P0: a sqrt(P/Vcell) grid to
    use instead of the analytic one (the lognormal boxes multiply by the Pln grids,
    bin/make_boxes.py:241-275).  velocity: (H0, dD/dz(0)) adds vx, vy, vz."""
    NX, NY = nk.shape[:2]
    N = NX * NY * NZ
    if P0 is None:
        P0 = sqrt_pk_grid(NX, NY, NZ, dcell, k0, A)
    kx, ky, kz = k_components(NX, NY, NZ, dcell)
    if precision == "f32":
        dk = nk.astype(np.complex64) * P0
    else:
        dk = nk * P0.astype(np.float64)

    def c2r(spec):
        r = np.fft.irfftn(spec.astype(np.complex128), s=(NX, NY, NZ), axes=(0, 1, 2)) * N
        if precision == "f32":
            return r.astype(np.float32) / np.float32(N)
        return r / N

    out = {"delta": c2r(dk)}
    for comp in eta:
        f = eta_factor(comp, kx, ky, kz)
        if precision == "f32":
            out["eta_" + comp] = c2r((dk * f).astype(np.complex64))
        else:
            out["eta_" + comp] = c2r(dk * f.astype(np.float64))
    if velocity is not None:
        for comp in VELOCITY_COMPONENTS:
            f = velocity_factor(comp, kx, ky, kz, *velocity)
            if precision == "f32":
                out[comp] = c2r((dk * f).astype(np.complex64))
            else:
                out[comp] = c2r(dk * f.astype(np.complex128))
    out["sigma"] = float(np.std(out["delta"].astype(np.float64)))
    return out


def measured_pk(box: np.ndarray, dcell: float, kbins: np.ndarray, pk=None):
    """Binned power of a box, P(k) = |FFT|^2 * Vcell / N (inverse of the generator's
    normalisation), averaged over modes in each |k| bin; returns (k_mean, P_mean, n_modes),
    plus the mode-averaged pk(k) of each bin when a spectrum function is given."""
    NX, NY, NZ = box.shape
    bk = np.fft.rfftn(box.astype(np.float64))
    kx, ky, kz = k_components(NX, NY, NZ, dcell)
    k = np.sqrt(kx.astype(np.float64) ** 2 + ky.astype(np.float64) ** 2
                + kz.astype(np.float64) ** 2)
    w = np.broadcast_to(half_weights(NZ), k.shape)
    p = np.abs(bk) ** 2 * (dcell ** 3) / (NX * NY * NZ)
    idx = np.digitize(k.ravel(), kbins) - 1
    ok = (idx >= 0) & (idx < len(kbins) - 1) & (k.ravel() > 0)
    wn = np.bincount(idx[ok], w.ravel()[ok], len(kbins) - 1)
    pk_ = np.bincount(idx[ok], (w * p).ravel()[ok], len(kbins) - 1)
    km = np.bincount(idx[ok], (w * k).ravel()[ok], len(kbins) - 1)
    with np.errstate(invalid="ignore", divide="ignore"):
        if pk is None:
            return km / wn, pk_ / wn, wn
        pe = np.bincount(idx[ok], (w * pk(k)).ravel()[ok], len(kbins) - 1)
        return km / wn, pk_ / wn, wn, pe / wn
