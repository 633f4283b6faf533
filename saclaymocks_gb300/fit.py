"""The (a,b,c) fit on the GPU with an adjoint gradient (host side of smk_fit_*).

The reference fits a(z) with iminuit's Migrad on fit_az.Fitter.chi2 (py/SaclayMocks/fit_az.py
:194-279): every call recomputes the FGPA of all stored pixels, <F>, dF = F/<F> - 1 per
spectrum and the binned P1D, and Migrad takes its derivatives by finite differences.  Here the
same kind of objective, per redshift bin j with parameters theta_j = (a_j, b_j, c_j),

    L(theta) = sum_j (<F>_j - Fbar*_j)^2 + sum_b ((P_b - P*_b) / P*_b)^2,

is evaluated by two GPU passes (mean flux per z bin; P1D of dF by Bluestein DFTs per pair of
equal-length skewers) and differentiated exactly by one adjoint pass that recomputes the
pixels instead of storing them.  Reductions are FP64; the loss and its gradient are assembled
in FP64 on the host from the reductions.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _lib
from .grf import stream_handle


def bin_index(x, edges):
    """scipy binned_statistic bins: [e_i, e_i+1), the last one closed; -1 outside."""
    x = np.asarray(x)
    nb = len(edges) - 1
    idx = np.searchsorted(edges, x, side="right") - 1
    idx = np.where(x == edges[-1], nb - 1, idx)
    return np.where((idx >= 0) & (idx < nb), idx, -1)


class FitProblem:
    """Fixed fields of the fit on the GPU: per-pixel delta (= delta_l + delta_s), eta_par,
    growth G and redshift, skewer lengths (packed layout), z and log-k bin edges."""

    def __init__(self, delta, eta, G, z, lengths, zedges, kedges, dx=0.2, device="cuda", store_spectrum=True):
        dv = torch.device(device)
        self.device = dv
        to_dev = lambda x, dt: None if x is None else torch.as_tensor(x).to(device=dv, dtype=dt).contiguous()  # noqa: E731
        self.delta = to_dev(delta, torch.float32)
        self.eta = to_dev(eta, torch.float32)
        self.G = to_dev(G, torch.float32)
        self.zedges = np.asarray(zedges, np.float64)
        self.kedges = np.asarray(kedges, np.float64)
        self.nzb, self.nkb = len(self.zedges) - 1, len(self.kedges) - 1
        zt = torch.as_tensor(z).to(device=dv, dtype=torch.float64)
        zb = torch.searchsorted(torch.as_tensor(self.zedges, device=dv), zt, right=True) - 1
        self.zbin = zb.clamp(0, self.nzb - 1).to(torch.int16).contiguous()
        self.lengths = np.ascontiguousarray(lengths, np.int32)
        self.offset = np.concatenate([[0], np.cumsum(self.lengths[:-1], dtype=np.int64)]).astype(np.int64)
        self.n_total = int(self.lengths.astype(np.int64).sum())
        self.dx = float(dx)
        lib = _lib.load()
        order = np.empty(2 * len(self.lengths) + 16, np.int32)
        ns = C.c_int64()
        _lib.check(lib.smk_fit_schedule(len(self.lengths), self.lengths.ctypes.data, order.ctypes.data,
                                        C.byref(ns)), "smk_fit_schedule")
        self.d_order = torch.from_numpy(order[:ns.value].copy()).to(dv)
        self.d_off = torch.from_numpy(self.offset).to(dv)
        self.d_npix = torch.from_numpy(self.lengths).to(dv)
        self.d_kedges = torch.from_numpy(self.kedges).to(dv)
        # chirp spectra and chirps of every distinct length (independent of theta): one table,
        # built once, M + N complex values per length
        uniq = np.unique(self.lengths).astype(np.int32)
        msz = np.array([lib.smk_fit_bluestein_m(int(N)) + int(N) for N in uniq], np.int64)
        offs = np.concatenate([[0], np.cumsum(msz[:-1])]).astype(np.int64)
        self.chirp = torch.empty(2 * int(msz.sum()), dtype=torch.float32, device=dv)
        off_by_n = np.full(2049, -1, np.int64)
        off_by_n[uniq] = offs
        self.d_chirp_off = torch.from_numpy(off_by_n).to(dv)
        d_uniq, d_offs = torch.from_numpy(uniq).to(dv), torch.from_numpy(offs).to(dv)
        _lib.check(lib.smk_fit_chirps(len(uniq), d_uniq.data_ptr(), d_offs.data_ptr(), self.chirp.data_ptr(),
                                      stream_handle()), "smk_fit_chirps")
        self.acc = torch.zeros(lib.smk_fit_acc_len(self.nzb, self.nkb), dtype=torch.float64, device=dv)
        self.ws = torch.zeros(32, dtype=torch.int64, device=dv)
        self.d_gM = torch.zeros(self.nzb, dtype=torch.float64, device=dv)
        self.d_gP = torch.zeros(self.nkb, dtype=torch.float64, device=dv)
        self.d_theta = torch.zeros((self.nzb, 3), dtype=torch.float32, device=dv)
        # fixed counts: pixels per z bin, (skewer, mode) pairs per k bin
        self.cnt_z = torch.bincount(self.zbin.long(), minlength=self.nzb).double().cpu().numpy()
        cnt_k = np.zeros(self.nkb)
        ksum = np.zeros(self.nkb)
        for N, mult in zip(*np.unique(self.lengths, return_counts=True)):
            k = np.fft.rfftfreq(int(N)) * 2 * (np.pi / self.dx)
            b = bin_index(k, self.kedges)
            cnt_k += mult * np.bincount(b[b >= 0], minlength=self.nkb)
            ksum += mult * np.bincount(b[b >= 0], weights=k[b >= 0], minlength=self.nkb)
        self.cnt_k = cnt_k
        with np.errstate(invalid="ignore", divide="ignore"):
            self.k_mean = ksum / cnt_k        # mean k of the (skewer, mode) pairs per bin
        self.fp = _lib.SmkFitProblem(
            delta=self.delta.data_ptr(), eta=self.eta.data_ptr() if self.eta is not None else None,
            G=self.G.data_ptr() if self.G is not None else None, zbin=self.zbin.data_ptr(),
            offset=self.d_off.data_ptr(), npix=self.d_npix.data_ptr(), order=self.d_order.data_ptr(),
            n_slots=ns.value, n_total=self.n_total, nzb=self.nzb, nkb=self.nkb,
            kedges=self.d_kedges.data_ptr(), dx=self.dx, chirp=self.chirp.data_ptr(),
            chirp_off=self.d_chirp_off.data_ptr(), n_max=int(self.lengths.max()))
        # the forward pass's pair spectra (8 B per pixel), read back by the backward of the same
        # theta instead of a second forward transform
        self.spec = torch.empty(2 * self.n_total, dtype=torch.float32, device=dv) if store_spectrum else None
        self.fp.spectrum = self.spec.data_ptr() if store_spectrum else None
        self._spec_theta = None

    def without_chirp_table(self):
        """Let the kernels compute the chirp spectra themselves (the form without the table)."""
        self.fp.chirp = None
        self.fp.chirp_off = None
        return self

    def without_spectrum_store(self):
        """Let the backward transform every pair again (the form without the stored spectra)."""
        self.fp.spectrum = None
        self.spec = None
        self._spec_theta = None
        return self

    # ---------------------------------------------------------------- passes
    def _set_theta(self, theta):
        t = torch.as_tensor(np.asarray(theta, np.float32).reshape(self.nzb, 3))
        self.d_theta.copy_(t)

    def reductions(self, theta):
        """(<F>_j, P_b, <F>) in FP64 from the GPU forward passes."""
        lib = _lib.load()
        self._set_theta(theta)
        _lib.check(lib.smk_fit_forward(C.byref(self.fp), self.d_theta.data_ptr(), self.acc.data_ptr(),
                                       self.ws.data_ptr(), self.ws.numel() * 8, stream_handle()),
                   "smk_fit_forward")
        self._spec_theta = np.asarray(theta, np.float32).reshape(self.nzb, 3).copy() if self.spec is not None else None
        acc = self.acc.cpu().numpy()
        nzb, nkb = self.nzb, self.nkb
        with np.errstate(invalid="ignore", divide="ignore"):
            mz = acc[:nzb] / self.cnt_z
            pk = acc[nzb + 1:nzb + 1 + nkb] / self.cnt_k
        return mz, pk, acc[nzb] / self.n_total

    def p1d_profile(self, theta):
        """util.MakeProfileHisto of the mock P1D (py/SaclayMocks/util.py:46-75 applied as in
        powerspectrum.ComputeP1D.P1D, :231-238): per non-empty k bin the mean k, the mean
        power and rms / sqrt(n), from the GPU sums of P and P^2 (FP64)."""
        self.reductions(theta)
        acc = self.acc.cpu().numpy()
        nzb, nkb = self.nzb, self.nkb
        s1 = acc[nzb + 1:nzb + 1 + nkb]
        s2 = acc[7 * nzb + 2 + nkb:7 * nzb + 2 + 2 * nkb]
        ok = self.cnt_k > 0
        n = self.cnt_k[ok]
        m1, m2 = s1[ok] / n, s2[ok] / n
        err = np.sqrt(np.maximum(m2 - m1 * m1, 0.0)) / np.sqrt(n)
        return self.k_mean[ok], m1, err

    def loss(self, theta, target_mz, target_pk) -> float:
        mz, pk, _ = self.reductions(theta)
        return float(((mz - target_mz) ** 2).sum() + (((pk - target_pk) / target_pk) ** 2).sum())

    def forward(self, theta, target_mz, target_pk):
        """Loss and the state the adjoint pass needs (small host arrays, no pixels)."""
        mz, pk, fbar = self.reductions(theta)
        L = float(((mz - target_mz) ** 2).sum() + (((pk - target_pk) / target_pk) ** 2).sum())
        state = dict(theta=np.asarray(theta, np.float64).reshape(self.nzb, 3).copy(), mz=mz, pk=pk,
                     fbar=fbar, target_mz=target_mz, target_pk=target_pk)
        return L, state

    def backward(self, state):
        """dL/dtheta [nzb, 3] by the adjoint pass; the pixels are recomputed on the GPU.  The
        accumulators must still hold this state's forward reductions (<F>)."""
        lib = _lib.load()
        mz, pk = state["mz"], state["pk"]
        gM = 2 * (mz - state["target_mz"]) / self.cnt_z
        gP = 2 * (pk - state["target_pk"]) / state["target_pk"] ** 2 / self.cnt_k
        self.d_gM.copy_(torch.from_numpy(np.nan_to_num(gM)))
        self.d_gP.copy_(torch.from_numpy(np.nan_to_num(gP)))
        self._set_theta(state["theta"])
        self.acc[self.nzb] = state["fbar"] * self.n_total   # <F> of this state's forward pass
        fp = self.fp
        th32 = np.asarray(state["theta"], np.float32).reshape(self.nzb, 3)
        if self.spec is not None and (self._spec_theta is None or not np.array_equal(self._spec_theta, th32)):
            # the stored spectra belong to another theta's forward: transform again
            fp = type(self.fp).from_buffer_copy(self.fp)
            fp.spectrum = None
        _lib.check(lib.smk_fit_backward(C.byref(fp), self.d_theta.data_ptr(), self.acc.data_ptr(),
                                        self.d_gM.data_ptr(), self.d_gP.data_ptr(), self.ws.data_ptr(),
                                        self.ws.numel() * 8, stream_handle()), "smk_fit_backward")
        acc = self.acc.cpu().numpy()
        nzb, nkb = self.nzb, self.nkb
        A = acc[nzb + 1 + nkb:nzb + 1 + nkb + 3 * nzb].reshape(nzb, 3)
        B = acc[4 * nzb + 1 + nkb:7 * nzb + 1 + nkb].reshape(nzb, 3)
        S = acc[7 * nzb + 1 + nkb]
        return A - S * B / (self.n_total * state["fbar"] ** 2)

    def loss_grad(self, theta, target_mz, target_pk):
        """(L, dL/dtheta [nzb, 3]) by the forward passes + one adjoint pass."""
        L, state = self.forward(theta, target_mz, target_pk)
        return L, self.backward(state)

    def fd_grad(self, theta, target_mz, target_pk, h=1e-4, points=2):
        """Finite differences of the GPU loss with relative step h: the derivative-free way
        Migrad proceeds.  points=2: central (f(x+h) - f(x-h)) / 2h, 2 * 3 * nzb loss
        evaluations; points=4: fourth-order stencil (8 f(x+h) - 8 f(x-h) - f(x+2h) + f(x-2h))
        / 12h, twice the evaluations and O(h^4) truncation, which lets h be large enough for the
        float32 rounding of the loss not to matter."""
        theta = np.asarray(theta, np.float64).reshape(self.nzb, 3)
        g = np.zeros_like(theta)

        def f(j, p, d):
            t = theta.copy()
            t[j, p] += d
            return self.loss(t, target_mz, target_pk)
        for j in range(self.nzb):
            for p in range(3):
                st = h * max(abs(theta[j, p]), 1e-3)
                if points == 4:
                    g[j, p] = (8 * f(j, p, st) - 8 * f(j, p, -st) - f(j, p, 2 * st) + f(j, p, -2 * st)) / (12 * st)
                else:
                    g[j, p] = (f(j, p, st) - f(j, p, -st)) / (2 * st)
        return g


class FgpaP1DLoss(torch.autograd.Function):
    """L(theta) as a torch autograd Function: forward = GPU reductions (saves only the bin
    means and <F>), backward = the adjoint pass, which recomputes every pixel."""

    @staticmethod
    def forward(ctx, theta, problem, target_mz, target_pk):
        L, state = problem.forward(theta.detach().cpu().numpy(), target_mz, target_pk)
        ctx.problem = problem
        ctx.state = state
        return theta.new_tensor(L)

    @staticmethod
    def backward(ctx, gL):
        g = ctx.problem.backward(ctx.state)
        return gL * torch.as_tensor(g, dtype=gL.dtype, device=gL.device), None, None, None


def adam_fit(problem: FitProblem, theta0, target_mz, target_pk, steps=50, lr=0.02, grad="adjoint",
             h=1e-4, eps_rel=0.0, points=2):
    """Adam on log-parameters (all of a, b, c are positive).  grad: "adjoint" or "fd".
    eps_rel sets Adam's epsilon relative to the largest first-step gradient component, which
    damps the steps of directions the loss barely constrains (the 30-parameter problem is
    badly conditioned).  Returns (theta, losses, seconds, gradient evaluations)."""
    theta0 = np.asarray(theta0, np.float64).reshape(problem.nzb, 3)
    x = np.log(theta0)
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    b1, b2, eps = 0.9, 0.999, 1e-12
    eps_set = eps_rel <= 0
    losses = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(1, steps + 1):
        th = np.exp(x)
        if grad == "adjoint":
            L, g = problem.loss_grad(th, target_mz, target_pk)
        else:
            L = problem.loss(th, target_mz, target_pk)
            g = problem.fd_grad(th, target_mz, target_pk, h, points)
        losses.append(L)
        gx = g * th                      # d/dlog(theta)
        if not eps_set:
            eps = max(eps_rel * float(np.abs(gx).max()), 1e-12)
            eps_set = True
        m = b1 * m + (1 - b1) * gx
        v = b2 * v + (1 - b2) * gx * gx
        mh = m / (1 - b1 ** it)
        vh = v / (1 - b2 ** it)
        x = x - lr * mh / (np.sqrt(vh) + eps)
    torch.cuda.synchronize()
    return np.exp(x), losses, time.perf_counter() - t0, steps
