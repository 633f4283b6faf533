"""GRF boxes on the GPU: the host side of ``smk_grf_boxes`` (the make_boxes hot path).

Mirrors bin/make_boxes.py: ``DrawGRF_boxk`` (:40-72) draws white noise and takes its r2c
transform, the P0 multiply (:288-292) scales it by sqrt(P(k)/Vcell), ``FFTandStore``
(:77-125) takes the c2r transform, divides by N, and records sigma and the null/NaN check;
eta_zz (:341-352) is the same c2r of kz^2/k^2 delta_k.  Here all of it is one call on device
memory: the boxes stay in HBM in the padded layout ``[batch][nx][ny][pitch]`` and are returned
as torch views ``[..., :nz]`` (no copy).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib


def pitch_of(nz: int) -> int:
    """Row pitch (floats) of the padded box layout."""
    return int(_lib.load().smk_grf_pitch(int(nz)))


def fft_supported(n: int) -> bool:
    return bool(_lib.load().smk_fft_supported(int(n)))


def stream_handle(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


@dataclass
class GrfBoxes:
    """Output of :func:`make_boxes`.  ``delta`` / ``eta`` are views [batch, nx, ny, nz] of the
    padded storage ``delta_pad`` / ``eta_pad`` ([batch, nx, ny, pitch])."""
    delta: torch.Tensor
    eta: torch.Tensor | None
    delta_pad: torch.Tensor
    eta_pad: torch.Tensor | None
    pitch: int
    stats: torch.Tensor          # [batch, 2, 4] FP64 (sum, sum^2, non-finite, 0) for delta, eta
    dcell: float

    def sigma(self, field: int = 0) -> np.ndarray:
        """Standard deviation of each box (FFTandStore's ``sigma`` header key)."""
        st = self.stats.double().cpu().numpy()
        n = self.delta.shape[1] * self.delta.shape[2] * self.delta.shape[3]
        out = []
        for b in range(st.shape[0]):
            rec = np.ascontiguousarray(st[b, field])
            sig = C.c_double(0.0)
            _lib.load().smk_grf_check(rec.ctypes.data_as(C.POINTER(C.c_double)), n, C.byref(sig))
            out.append(sig.value)
        return np.array(out)

    def check(self):
        """Raise SmkError(SMK_ENULLBOX) if a box is all zero or non-finite
        (bin/make_boxes.py:100-105)."""
        st = self.stats.double().cpu().numpy()
        n = self.delta.shape[1] * self.delta.shape[2] * self.delta.shape[3]
        lib = _lib.load()
        fields = [0] + ([1] if self.eta is not None else [])
        for b in range(st.shape[0]):
            for f in fields:
                rec = np.ascontiguousarray(st[b, f])
                _lib.check(lib.smk_grf_check(rec.ctypes.data_as(C.POINTER(C.c_double)), n, None),
                           f"box {b} field {f}")


def alloc_boxes(nx: int, ny: int, nz: int, batch: int = 1, want_eta: bool = True, device="cuda"):
    """Padded output storage for :func:`make_boxes` (reusable across calls)."""
    p = pitch_of(nz)
    d = torch.empty((batch, nx, ny, p), dtype=torch.float32, device=device)
    e = torch.empty((batch, nx, ny, p), dtype=torch.float32, device=device) if want_eta else None
    return d, e


class GrfWorkspace:
    """Device workspace + stats buffer reused by repeated calls (the workspace grows on
    demand to smk_grf_workspace_size)."""

    def __init__(self, batch: int, device="cuda"):
        self.device = device
        self.ws = torch.zeros(256 // 8, dtype=torch.float64, device=device)
        self.stats = torch.zeros((batch, 2, 4), dtype=torch.float64, device=device)

    def ensure(self, nbytes: int):
        if self.ws.numel() * 8 < nbytes:
            self.ws = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=self.ws.device)
        return self.ws


# Above this footprint of delta + eta the in-place x pass of GPU noise writes each field in
# its own launch (address-translation reach; the library's default rule, smk_tune_flag).
SPLIT_MIN_PAIR_BYTES = 64 * 2 ** 30


def make_boxes(nx: int, ny: int | None = None, nz: int | None = None, dcell: float = 2.19,
               seed: int = 0, *, noise: torch.Tensor | None = None, k0: float = 0.02,
               amp: float | None = None, pk_grid: torch.Tensor | None = None,
               want_eta: bool = True, batch: int = 1, out=None, workspace: GrfWorkspace | None = None,
               stream=None, pass_events=None, eta_comp: str = "zz",
               vel_factor: float | None = None, xi_chunk_kz: int = 128) -> GrfBoxes:
    """Draw delta (and eta_zz) boxes on the current CUDA device.

    noise:   None -> Philox white noise drawn on the GPU from ``seed`` (box b: seed + b);
             else a float32 CUDA tensor [batch, nx, ny, nz] (or [nx, ny, nz]) of white noise,
             e.g. the reference's ``RandomState(seed)`` plane-order draws.
    pk_grid: None -> analytic P(k) = amp*k/(1+(k/k0)^2)^2 (amp None: E[var delta] = 1);
             else a float32 CUDA tensor [nx, ny, nz//2+1] of sqrt(P/Vcell) (the P0 grid of
             bin/interpolate_pk.py).
    out:     optional (delta_pad, eta_pad) from :func:`alloc_boxes` to reuse storage.
    pass_events: optional list of 6 recorded torch.cuda.Event, marked before the first HBM
             pass and after each of the five (per-pass timing).
    xi_chunk_kz: > 0 runs the x pass into a blocked intermediate in the workspace (both fields
             from one launch, GPU-noise modes drawn once, the y pass reading contiguous runs),
             that many k_z columns at a time (the workspace grows to about
             16 * batch * nx * ny * xi_chunk_kz bytes with eta: 13 GB at 2560 x 2560 for the
             default 128); 0 writes the boxes in place.  Same boxes, bit for bit.
    eta_comp: which eta_ij = irfftn(k_i k_j / k^2 delta_k) the eta box holds ("zz", "xx",
             "yy", "xy", "xz", "yz"; bin/make_boxes.py:315-391), or a velocity
             v_i = irfftn(-i k_i / k^2 * vel_factor * delta_k) ("vx", "vy", "vz";
             bin/make_boxes.py:393-431, vel_factor = H0 * dD/dz(z=0)).
    """
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    lib = _lib.load()
    p = _lib.SmkGrfParams()
    p.nx, p.ny, p.nz, p.batch = int(nx), int(ny), int(nz), int(batch)
    p.dcell = float(dcell)
    p.k0 = float(k0)
    p.amp = float(amp) if amp is not None else 0.0
    p.want_eta = 1 if want_eta else 0
    p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    p.eta_comp = _lib.SMK_ETA[eta_comp]
    p.xi_chunk_kz = int(xi_chunk_kz)
    if eta_comp in ("vx", "vy", "vz"):
        if vel_factor is None:
            raise ValueError("velocity boxes need vel_factor = H0 * dD/dz(z=0)")
        p.vel_factor = float(vel_factor)
    keep = []
    if noise is not None:
        if noise.dtype != torch.float32 or not noise.is_cuda or not noise.is_contiguous():
            raise ValueError("noise must be a contiguous float32 CUDA tensor")
        if noise.numel() != batch * nx * ny * nz:
            raise ValueError("noise has the wrong number of cells")
        p.noise_mode = _lib.SMK_NOISE_HOST
        p.noise = noise.data_ptr()
        keep.append(noise)
    else:
        p.noise_mode = _lib.SMK_NOISE_PHILOX
    if pk_grid is not None:
        if pk_grid.dtype != torch.float32 or not pk_grid.is_cuda or not pk_grid.is_contiguous():
            raise ValueError("pk_grid must be a contiguous float32 CUDA tensor")
        if tuple(pk_grid.shape) != (nx, ny, nz // 2 + 1):
            raise ValueError("pk_grid must be [nx, ny, nz//2+1]")
        p.pk_mode = _lib.SMK_PK_GRID
        p.pk_grid = pk_grid.data_ptr()
    else:
        p.pk_mode = _lib.SMK_PK_ANALYTIC
    device = noise.device if noise is not None else torch.device("cuda", torch.cuda.current_device())
    if out is None:
        dpad, epad = alloc_boxes(nx, ny, nz, batch, want_eta, device)
    else:
        dpad, epad = out
    if workspace is None:
        workspace = GrfWorkspace(batch, device)
    workspace.ensure(lib.smk_grf_workspace_size(C.byref(p)))
    if pass_events is not None:
        handles = (C.c_void_p * 6)(*[int(e.cuda_event) for e in pass_events])
        keep.append(handles)
        p.pass_events = C.cast(handles, C.c_void_p)
        p.n_pass_events = 6
    st = stream_handle(stream)
    rc = lib.smk_grf_boxes(C.byref(p), dpad.data_ptr(), epad.data_ptr() if want_eta else None,
                           workspace.stats.data_ptr(), workspace.ws.data_ptr(),
                           workspace.ws.numel() * 8, st)
    _lib.check(rc, "smk_grf_boxes")
    return GrfBoxes(delta=dpad[..., :nz], eta=epad[..., :nz] if want_eta else None,
                    delta_pad=dpad, eta_pad=epad, pitch=dpad.shape[-1], stats=workspace.stats,
                    dcell=float(dcell))


def grf_launches(nx: int, ny: int, nz: int, batch: int = 1, want_eta: bool = True, gpu_noise: bool = True,
                 xi_chunk_kz: int = 128) -> int:
    """Kernel launches of one smk_grf_boxes call as make_boxes issues it (x pass in place: x, y
    inverse, z inverse, the GPU-noise x pass in two launches when delta + eta exceed
    SPLIT_MIN_PAIR_BYTES, and host noise adding the z and y forward passes; blocked
    intermediate: one x launch and one y launch per chunk of xi_chunk_kz columns rounded up to
    16, then the z inverse)."""
    fwd = 0 if gpu_noise else 2
    if xi_chunk_kz > 0:
        nzh = nz // 2 + 1
        cols = min((xi_chunk_kz + 15) // 16 * 16, (nzh + 15) // 16 * 16)
        return fwd + 2 * (-(-nzh // cols)) + 1
    if not gpu_noise:
        return 5
    pair = 2 * 4 * batch * nx * ny * pitch_of(nz)
    return 4 if want_eta and pair > SPLIT_MIN_PAIR_BYTES else 3


def pk_normalisation(nx: int, ny: int, nz: int, dcell: float = 2.19, k0: float = 0.02) -> float:
    """A with E[var delta] = 1 for the analytic spectrum, summed on the GPU in FP64."""
    lib = _lib.load()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    _lib.check(lib.smk_pk_normalisation(int(nx), int(ny), int(nz), float(dcell), float(k0),
                                        out.data_ptr(), stream_handle()), "smk_pk_normalisation")
    return float(out.item())
