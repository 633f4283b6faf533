"""Host-facing helpers with the reference's names: ``fgpa`` (the GPU drop-in for
py/SaclayMocks/util.py:421-433), ``fgrowth`` (:123-134) and ``sigma_p1d`` (:372-398).

``fgpa`` runs the smk_fgpa kernel in float32; ``fgrowth`` and ``sigma_p1d`` are scalar
cosmology formulas evaluated on the host (they configure the kernels, they are not
per-pixel work).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .grf import stream_handle

OMEGA_M_0 = 0.31457   # py/SaclayMocks/constant.py:23
LYA = 1215.67         # py/SaclayMocks/constant.py:12


def fgrowth(z, Om0: float = OMEGA_M_0, unnormed: bool = False):
    """Carroll-Press-Turner linear growth factor normalised at z = 0 (flat LCDM)."""
    Om = 1 / (1 + (1 - Om0) / (Om0 * (1 + np.asarray(z, np.float64)) ** 3))
    Ol = 1 - Om
    a = 1 / (1 + np.asarray(z, np.float64))
    norm = 1.0 if unnormed else 1.0 / fgrowth(0.0, Om0, unnormed=True)
    return norm * (5. / 2.) * a * Om / (Om ** (4. / 7.) - Ol + (1. + Om / 2.) * (1. + Ol / 70.))


def sigma_p1d(p1dmiss, pixel: float = 0.2, N: int = 10000) -> float:
    """sigma of delta_s for a P1D_miss(k) function: 2 sum_j P(k_j)/L + P(0)/L + P(k_N)/L."""
    L = N * pixel
    kj = 2 * np.pi / L * np.arange(1, N / 2)
    var = 2 * np.sum(p1dmiss(kj)) / L + p1dmiss(0.0) / L + p1dmiss(np.pi / pixel) / L
    return float(np.sqrt(var))


def _as_param(x, n, device, keep):
    """(device pointer or None, scalar) for a fgpa parameter given as scalar or array."""
    if np.isscalar(x) or (isinstance(x, np.ndarray) and x.ndim == 0) or \
            (isinstance(x, torch.Tensor) and x.dim() == 0):
        return None, float(x)
    t = torch.as_tensor(np.asarray(x) if not isinstance(x, torch.Tensor) else x)
    t = t.to(device=device, dtype=torch.float32).contiguous()
    if t.numel() == 1:
        return None, float(t.item())
    if t.numel() != n:
        t = t.broadcast_to(keep[0].shape).contiguous()
    keep.append(t)
    return t.data_ptr(), 0.0


def fgpa(delta, eta_par, growthf, a, b, c, out=None):
    """F = exp(-a exp(b G (delta + c eta_par))) on the GPU (float32).

    Same call as py/SaclayMocks/util.py:421 ``fgpa(delta, eta_par, growthf, a, b, c)``:
    delta is an array (numpy or CUDA tensor); eta_par, growthf, a, b, c are arrays
    broadcastable to it or scalars; eta_par=None gives the no-RSD form
    exp(-a exp(b G delta)) of bin/merge_spectra.py:339.  Returns a numpy float32 array for
    numpy input, a CUDA float32 tensor for tensor input.
    """
    lib = _lib.load()
    as_numpy = not isinstance(delta, torch.Tensor)
    device = torch.device("cuda", torch.cuda.current_device()) if as_numpy else delta.device
    d = torch.as_tensor(np.asarray(delta) if as_numpy else delta).to(device=device, dtype=torch.float32)
    shape = d.shape
    d = d.contiguous().reshape(-1)
    n = d.numel()
    keep = [d.reshape(shape)]
    ep, _ = (None, 0.0) if eta_par is None else _as_param(eta_par, n, device, keep)
    if eta_par is not None and ep is None:     # scalar eta: broadcast
        e = torch.full((n,), float(eta_par), dtype=torch.float32, device=device)
        keep.append(e)
        ep = e.data_ptr()
    gp, g0 = _as_param(growthf, n, device, keep)
    ap, a0 = _as_param(a, n, device, keep)
    bp, b0 = _as_param(b, n, device, keep)
    cp, c0 = _as_param(c, n, device, keep)
    f = out if out is not None else torch.empty(n, dtype=torch.float32, device=device)
    rc = lib.smk_fgpa(n, d.data_ptr(), ep, gp, g0, ap, a0, bp, b0, cp, c0, f.data_ptr(), stream_handle())
    _lib.check(rc, "smk_fgpa")
    f = f.reshape(shape)
    return f.cpu().numpy() if as_numpy else f
