"""Skewer stage on the GPU: the host side of ``smk_skewers_flux``.

Mirrors the per-quasar loop of bin/make_spectra.py (:412-522, ReadSpec :90-139) followed by
the per-skewer loop of bin/merge_spectra.py (:267-339): read delta_l and eta_par along each
line of sight, add the missing small-scale power delta_s (a Gaussian field of 1D spectrum
P1D_miss drawn through an FFT of length nz), apply the FGPA.  Skewers are given as a
:class:`SkewerTable` in the box-corner frame (start point, unit direction, pixel count,
pixel spacing); outputs are packed: skewer s owns pixels [offset[s], offset[s]+npix[s]).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .grf import stream_handle
from .util import fgrowth

SS_CLASSES = tuple(256 << j for j in range(5))   # small-scale FFT lengths the kernel handles


def nz_rule(npix: int) -> int:
    """256 * 2^n >= npix + 50 (bin/merge_spectra.py:308-309)."""
    nz = 256
    while nz < npix + 50:
        nz *= 2
    return nz


def ss_scale_tables(pmiss, pixsize: float = 0.2) -> np.ndarray:
    """sqrt(max(P1Dmiss(k), 0) / pixsize) at k = rfftfreq(nz) * 2 k_ny for every nz class,
    concatenated (merge_spectra.py:312-320; negative P1Dmiss clipped as at :319)."""
    out = []
    for nz in SS_CLASSES:
        k = np.fft.rfftfreq(nz) * 2 * (np.pi / pixsize)
        out.append(np.sqrt(np.maximum(np.asarray(pmiss(k), np.float64), 0.0) / pixsize))
    return np.concatenate(out).astype(np.float32)


class P1DMissTable:
    """P1D_miss tabulated on a redshift grid, as util.InterpP1Dmissing reads it
    (py/SaclayMocks/util.py:448-474: extensions ``z`` [nz], ``k`` [nk], ``pk`` [nz, nk]) plus the
    ``sigma`` extension merge_spectra interpolates in z (bin/merge_spectra.py:118).  Each
    skewer takes the table nearest to the mean redshift of its forest pixels, interpolated
    linearly in k and clipped at 0, and, with sigma, its delta_s is rescaled pixel by pixel by
    sigma(z)/sigma(zeff) (bin/merge_spectra.py:305-325)."""

    def __init__(self, z, k, pk, sigma=None):
        z = np.asarray(z, np.float64).reshape(-1)
        order = np.argsort(z, kind="stable")
        self.z = z[order]
        self.k = np.asarray(k, np.float64).reshape(-1)
        self.pk = np.asarray(pk, np.float64).reshape(len(z), -1)[order]
        self.sigma = None if sigma is None else np.asarray(sigma, np.float64).reshape(-1)[order]
        if self.pk.shape[1] != len(self.k):
            raise ValueError("pk must be [len(z), len(k)]")

    @classmethod
    def from_fits(cls, path):
        from . import fits
        return cls(fits.read(path, "z"), fits.read(path, "k"), fits.read(path, "pk"), fits.read(path, "sigma"))

    def scale_sets(self, pixsize: float = 0.2) -> np.ndarray:
        """Table sets of smk_skewers_flux (ss_nztab of them, SMK_SS_SET_FLOATS floats each)."""
        return np.concatenate([ss_scale_tables(lambda kk, j=j: np.interp(kk, self.k, self.pk[j]), pixsize)
                               for j in range(len(self.z))])


def forest_ranges(wav, zqso, lya: float = 1215.67, lylimit: float = 0.0) -> np.ndarray:
    """[n, 2] pixel range [f0, f1) of the Lya forest of each skewer: the pixels with
    lylimit < lambda/(1+z_qso) < lya (bin/merge_spectra.py:305-306), wavelengths ascending."""
    out = np.zeros((len(wav), 2), np.int32)
    for s, (w, zq) in enumerate(zip(wav, zqso)):
        rf = np.asarray(w, np.float64) / (1.0 + float(zq))
        idx = np.nonzero((rf < lya) & (rf > lylimit))[0]
        if len(idx):
            if idx[-1] - idx[0] + 1 != len(idx):
                raise ValueError(f"skewer {s}: forest pixels are not contiguous (wavelengths unsorted?)")
            out[s] = idx[0], idx[-1] + 1
    return out


def pmiss_gauss(amp: float = 0.05, kscale: float = 2.0):
    """P1D_miss(k) = amp * exp(-(k/kscale)^2) (k in h/Mpc)."""
    return lambda k: amp * np.exp(-(np.asarray(k, np.float64) / kscale) ** 2)


@dataclass
class SkewerTable:
    start: np.ndarray              # [n, 3] float32, Mpc/h, box-corner frame
    direction: np.ndarray          # [n, 3] float32 unit vectors
    npix: np.ndarray               # [n] int32
    dpix: float = 0.2
    offset: np.ndarray = field(default=None)   # [n] int64 (filled by __post_init__)
    forest: np.ndarray | None = None           # [n, 2] int32 forest pixel range, None: all pixels
    start64: np.ndarray | None = None          # [n, 3] float64 start points (override start)
    dir64: np.ndarray | None = None            # [n, 3] float64 unit directions (override direction)

    def __post_init__(self):
        self.start = np.ascontiguousarray(self.start, dtype=np.float32).reshape(-1, 3)
        self.direction = np.ascontiguousarray(self.direction, dtype=np.float32).reshape(-1, 3)
        self.npix = np.ascontiguousarray(self.npix, dtype=np.int32).reshape(-1)
        if self.offset is None:
            self.offset = np.concatenate([[0], np.cumsum(self.npix[:-1], dtype=np.int64)]).astype(np.int64) \
                if len(self.npix) else np.zeros(0, np.int64)
        if not (len(self.start) == len(self.direction) == len(self.npix) == len(self.offset)):
            raise ValueError("skewer table arrays differ in length")
        for name in ("start64", "dir64"):
            v = getattr(self, name)
            if v is not None:
                v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
                if len(v) != len(self.npix):
                    raise ValueError(f"{name} and skewers differ in length")
                setattr(self, name, v)
        if self.forest is not None:
            self.forest = np.ascontiguousarray(self.forest, dtype=np.int32).reshape(-1, 2)
            if len(self.forest) != len(self.npix):
                raise ValueError("forest ranges and skewers differ in length")

    @property
    def n(self) -> int:
        return len(self.npix)

    @property
    def total_pixels(self) -> int:
        return int(self.npix.astype(np.int64).sum())

    def schedule(self, ss_nz: int, pair: bool = True) -> np.ndarray:
        """Work schedule of smk_skewers_flux (pairs of equal small-scale FFT length).
        pair=False gives every skewer a work item of its own (the other slot empty): the
        one-skewer-per-block layout, kept as the baseline the paired schedule is measured
        against."""
        lib = _lib.load()
        order = np.empty(2 * self.n + 16, dtype=np.int32)
        nslots = C.c_int64(0)
        _lib.check(lib.smk_skewer_schedule(self.n, self.npix.ctypes.data, int(ss_nz),
                                           order.ctypes.data, C.byref(nslots)), "smk_skewer_schedule")
        order = order[:nslots.value].copy()
        if not pair:
            ids = order[order >= 0]
            order = np.stack([ids, np.full_like(ids, -1)], 1).ravel().copy()
        return order


def skewers_parallel_z(n: int, nx: int, ny: int, npix: int, dcell: float, seed: int = 0,
                       dpix: float | None = None) -> SkewerTable:
    """n skewers along +z at uniform random (x, y), starting at z = 0."""
    rs = np.random.RandomState(seed)
    x = rs.uniform(0, nx * dcell, n)
    y = rs.uniform(0, ny * dcell, n)
    start = np.stack([x, y, np.zeros(n)], 1)
    d = np.tile([0.0, 0.0, 1.0], (n, 1))
    return SkewerTable(start, d, np.full(n, npix), dpix=dcell if dpix is None else dpix)


def skewers_cone(n: int, box_len, seed: int = 1, max_angle_deg: float = 10.0,
                 npix_range=(400, 1200), dpix: float = 0.2, log_uniform: bool = False) -> SkewerTable:
    """n skewers with start points uniform in the box, directions uniform on the cap within
    max_angle of +z, lengths uniform (or log-uniform) in npix_range (inclusive)."""
    rs = np.random.RandomState(seed)
    L = np.broadcast_to(np.asarray(box_len, np.float64), (3,))
    start = rs.uniform(0, 1, (n, 3)) * L
    cosmax = np.cos(np.radians(max_angle_deg))
    cz = rs.uniform(cosmax, 1.0, n)
    phi = rs.uniform(0, 2 * np.pi, n)
    sz = np.sqrt(1 - cz ** 2)
    d = np.stack([sz * np.cos(phi), sz * np.sin(phi), cz], 1)
    lo, hi = npix_range
    if log_uniform:
        npix = np.floor(np.exp(rs.uniform(np.log(lo), np.log(hi + 1), n))).astype(np.int32)
        npix = np.clip(npix, lo, hi)
    else:
        npix = rs.randint(lo, hi + 1, n).astype(np.int32)
    return SkewerTable(start, d, npix, dpix=dpix)


@dataclass
class SpectraConfig:
    """Small-scale and FGPA settings of :func:`skewer_flux` (see include/smk.h)."""
    ss_mode: int = _lib.SMK_SS_NONE
    ss_nz: int = 0                    # 0: reference rule 256*2^n >= npix+50
    pmiss: object = None              # callable P1Dmiss(k) (default 0.05 exp(-(k/2)^2)), or a
                                      # P1DMissTable (redshift-dependent, merge_spectra's default)
    pixsize: float = 0.2
    seed: int = 0
    abc_mode: int = _lib.SMK_ABC_CONST
    a: float = 0.1
    b: float = 1.6
    c: float = 0.5
    a_zref1: float = 3.2
    a_power: float = 4.5
    abc_table: np.ndarray | None = None   # [n, 4] rows (z, a, b, c) on a uniform z grid
    z_lo: float = 1.8
    z_hi: float = 3.6
    growth: int = _lib.SMK_G_ONE
    read: str = "trilinear"           # "trilinear" or "gauss343" (the reference's 7^3 read)
    observer: tuple = (0.0, 0.0, 0.0)  # gauss343: observer in the box-corner frame (Mpc/h)
    dmax: int = 3                     # gauss343: half-width of the read in cells (1..4)


class SkewerRunner:
    """Device copies of a skewer table + schedule + tables, reusable across calls."""

    def __init__(self, table: SkewerTable, cfg: SpectraConfig, device="cuda", pixels=None, pair: bool = True):
        self.table = table
        self.cfg = cfg
        self.device = torch.device(device)
        order = table.schedule(cfg.ss_nz if cfg.ss_mode != _lib.SMK_SS_NONE else -1, pair=pair)
        dv = self.device
        self.d_start = torch.from_numpy(table.start).to(dv)
        self.d_dir = torch.from_numpy(table.direction).to(dv)
        self.d_npix = torch.from_numpy(table.npix).to(dv)
        self.d_off = torch.from_numpy(table.offset).to(dv)
        self.d_order = torch.from_numpy(order).to(dv)
        self.n_slots = len(order)
        pm = cfg.pmiss if cfg.pmiss is not None else pmiss_gauss()
        self.nztab, self.d_ztab, self.d_zsig = 0, None, None
        if isinstance(pm, P1DMissTable):
            self.d_scale = torch.from_numpy(pm.scale_sets(cfg.pixsize)).to(dv)
            self.nztab = len(pm.z)
            self.d_ztab = torch.from_numpy(pm.z.astype(np.float32)).to(dv)
            if pm.sigma is not None:
                self.d_zsig = torch.from_numpy(pm.sigma.astype(np.float32)).to(dv)
        else:
            self.d_scale = torch.from_numpy(ss_scale_tables(pm, cfg.pixsize)).to(dv)
        self.d_forest = torch.from_numpy(table.forest).to(dv) if table.forest is not None else None
        self.d_start64 = torch.from_numpy(table.start64).to(dv) if table.start64 is not None else None
        self.d_dir64 = torch.from_numpy(table.dir64).to(dv) if table.dir64 is not None else None
        self.d_tab = None
        if cfg.abc_mode == _lib.SMK_ABC_TABLE:
            t = np.asarray(cfg.abc_table, np.float64)
            self.tab_z0, self.tab_dz, self.tab_n = float(t[0, 0]), float(t[1, 0] - t[0, 0]), len(t)
            self.d_tab = torch.from_numpy(np.ascontiguousarray(t[:, 1:4], dtype=np.float32)).to(dv)
        self.ws = torch.zeros(32, dtype=torch.int64, device=dv)
        self.pixels = pixels     # (delta_l, eta_par or None, z) packed CUDA tensors for SMK_INTERP_PIXELS

    def structs(self, nx, ny, nz, pitch, dcell, noise=None, eta6=None):
        cfg = self.cfg
        sk = _lib.SmkSkewers()
        sk.n = self.table.n
        sk.start = self.d_start.data_ptr()
        sk.dir = self.d_dir.data_ptr()
        sk.npix = self.d_npix.data_ptr()
        sk.offset = self.d_off.data_ptr()
        sk.dpix = float(self.table.dpix)
        sk.order = self.d_order.data_ptr()
        sk.n_slots = self.n_slots
        sk.forest = self.d_forest.data_ptr() if self.d_forest is not None else None
        sk.start64 = self.d_start64.data_ptr() if self.d_start64 is not None else None
        sk.dir64 = self.d_dir64.data_ptr() if self.d_dir64 is not None else None
        p = _lib.SmkSpectraParams()
        p.interp = _lib.SMK_INTERP_TRILINEAR
        if cfg.read == "gauss343":
            p.interp = _lib.SMK_INTERP_GAUSS343
            p.obs[:] = [float(v) for v in cfg.observer]
            p.gauss_dmax = int(cfg.dmax)
            if eta6 is not None:
                if len(eta6) != 6:
                    raise ValueError("eta6: six boxes eta_xx, yy, zz, xy, xz, yz")
                p.eta6[:] = [t.data_ptr() for t in eta6]
        elif cfg.read != "trilinear":
            raise ValueError(f"unknown read {cfg.read!r}")
        if self.pixels is not None:
            p.interp = _lib.SMK_INTERP_PIXELS
            sk.pix_delta = self.pixels[0].data_ptr()
            sk.pix_eta = self.pixels[1].data_ptr() if self.pixels[1] is not None else None
            sk.pix_z = self.pixels[2].data_ptr()
        p.nx, p.ny, p.nz, p.pitch, p.dcell = int(nx), int(ny), int(nz), int(pitch), float(dcell)
        p.ss_mode = cfg.ss_mode
        p.ss_nz = int(cfg.ss_nz)
        p.ss_scale = self.d_scale.data_ptr()
        if self.nztab:
            p.ss_nztab = self.nztab
            p.ss_ztab = self.d_ztab.data_ptr()
            p.ss_zsigma = self.d_zsig.data_ptr() if self.d_zsig is not None else None
        if cfg.ss_mode == _lib.SMK_SS_HOST:
            p.ss_noise = noise[0].data_ptr()
            p.ss_noise_offset = noise[1].data_ptr()
        p.seed = int(cfg.seed) & 0xFFFFFFFFFFFFFFFF
        p.abc_mode = cfg.abc_mode
        p.a, p.b, p.c = cfg.a, cfg.b, cfg.c
        p.a_zref1, p.a_power = cfg.a_zref1, cfg.a_power
        if self.d_tab is not None:
            p.abc_tab = self.d_tab.data_ptr()
            p.n_tab, p.z_tab0, p.dz_tab = self.tab_n, self.tab_z0, self.tab_dz
        p.z_lo, p.z_hi = cfg.z_lo, cfg.z_hi
        p.growth_mode = cfg.growth
        p.growth24 = float(fgrowth(2.4))
        return sk, p

    def run(self, delta_box=None, eta_box=None, *, nx=1, ny=1, nz=1, pitch=1, dcell=1.0,
            noise=None, want_fields=False, flux=None, stream=None, eta6=None):
        """Launch the fused kernel; boxes are padded CUDA tensors [nx, ny, pitch] (or None in
        pixel mode).  noise = (packed float32 tensor, int64 offsets tensor) for SMK_SS_HOST.
        eta6: for read="gauss343", the six eta_ij boxes (xx, yy, zz, xy, xz, yz) whose
        projection on the line of sight from cfg.observer gives eta_par (None: no RSD)."""
        lib = _lib.load()
        sk, p = self.structs(nx, ny, nz, pitch, dcell, noise, eta6)
        npx = self.table.total_pixels
        dv = self.device
        if flux is None:
            flux = torch.empty(npx, dtype=torch.float32, device=dv)
        extra = [torch.empty(npx, dtype=torch.float32, device=dv) for _ in range(3)] if want_fields else [None] * 3
        ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
        rc = lib.smk_skewers_flux(C.byref(sk), C.byref(p), ptr(delta_box), ptr(eta_box), flux.data_ptr(),
                                  ptr(extra[0]), ptr(extra[1]), ptr(extra[2]), self.ws.data_ptr(),
                                  self.ws.numel() * 8, stream_handle(stream))
        _lib.check(rc, "smk_skewers_flux")
        if want_fields:
            return flux, extra[0], extra[1], extra[2]
        return flux


def split(packed, table: SkewerTable) -> list:
    """Packed per-pixel array -> list of per-skewer arrays (numpy)."""
    a = packed.detach().cpu().numpy() if isinstance(packed, torch.Tensor) else np.asarray(packed)
    return [a[o:o + n] for o, n in zip(table.offset, table.npix)]
