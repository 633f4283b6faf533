"""Oracle for the (a,b,c) fit: the fit_az chi2 and the per-z-bin loss with its gradient.

* ``fit_az_chi2`` restates py/SaclayMocks/fit_az.py:194-264 (comp_spectra -> masked
  mean flux -> dF = F/<F> - 1 per spectrum -> ComputeP1D binned P1D -> chi2 vs data).
* ``zbin_loss`` is the differentiable loss of the fit the adjoint replaces: per-pixel
  parameters (a_j, b_j, c_j) of the redshift bin j of the pixel,
      L = sum_j (<F>_j - Fbar*_j)^2 + sum_b ((P_b - P*_b)/P*_b)^2,
  with <F>_j the mean flux of bin j and P_b the binned P1D of dF = F/<F> - 1
  (<F> over all pixels, as fit_az.compute_p1d :201-212) in log-k bins.
* ``zbin_loss_grad`` is its exact gradient written out by hand (FP64), and
  ``zbin_loss_fd_grad`` the central-difference gradient the adjoint is checked against.
TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import numpy as np

from . import p1d as _p1d
from .skewers import fgpa


def fit_az_chi2(a, bb, cc, delta_l, delta_s, eta, mask, growthf, bins, data_pk, data_err,
                pixel=0.2):
    """fit_az.Fitter.chi2(a) for masked [nspec, npix] fields (fit_az.py:194-264)."""
    F = fgpa(delta_l + delta_s, eta, growthf, a, bb, cc)
    Fmean = F[~mask].mean()
    spectra = [F[i][~mask[i]] / Fmean - 1 for i in range(F.shape[0]) if (~mask[i]).sum() >= 1]
    _, pk, _ = _p1d.binned_p1d(spectra, pixel, bins)
    return float((((pk - data_pk) / data_err) ** 2).sum())


class ZBinProblem:
    """Fixed fields of the fit: per-pixel delta (= delta_l + delta_s), eta, G, redshift,
    skewer segmentation, and the z and log-k bin edges."""

    def __init__(self, delta, eta, G, z, lengths, zedges, kedges, dx):
        self.delta = np.asarray(delta, np.float64)
        self.eta = np.asarray(eta, np.float64)
        self.G = np.asarray(G, np.float64)
        self.z = np.asarray(z, np.float64)
        self.lengths = np.asarray(lengths, np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.lengths)])
        self.zedges = np.asarray(zedges, np.float64)
        self.kedges = np.asarray(kedges, np.float64)
        self.dx = float(dx)
        nzb = len(zedges) - 1
        self.zbin = np.clip(np.searchsorted(self.zedges, self.z, side="right") - 1, 0, nzb - 1)
        self.nzb = nzb
        self.nkb = len(kedges) - 1

    def flux(self, theta):
        a, b, c = theta[self.zbin, 0], theta[self.zbin, 1], theta[self.zbin, 2]
        return fgpa(self.delta, self.eta, self.G, a, b, c)

    def reductions(self, F):
        nzb, nkb = self.nzb, self.nkb
        cnt_z = np.bincount(self.zbin, minlength=nzb).astype(np.float64)
        mz = np.bincount(self.zbin, F, nzb) / cnt_z
        fbar = F.mean()
        sp = np.zeros(nkb)
        cnt_k = np.zeros(nkb)
        X = []
        for s in range(len(self.lengths)):
            o, n = self.offsets[s], self.lengths[s]
            x = np.fft.rfft(F[o:o + n] / fbar - 1)
            X.append(x)
            k = _p1d.p1d_k(n, self.dx)
            idx = _p1d.bin_index(k, self.kedges)
            m = idx >= 0
            sp += np.bincount(idx[m], (np.abs(x[m]) ** 2) * self.dx / n, nkb)
            cnt_k += np.bincount(idx[m], minlength=nkb)
        return mz, sp / cnt_k, fbar, X, cnt_z, cnt_k

    def loss(self, theta, target_mz, target_pk):
        F = self.flux(theta)
        mz, pk, *_ = self.reductions(F)
        return float(((mz - target_mz) ** 2).sum() + (((pk - target_pk) / target_pk) ** 2).sum())

    def loss_grad(self, theta, target_mz, target_pk):
        """Exact gradient dL/dtheta [nzb, 3] by the chain rule through the reductions."""
        F = self.flux(theta)
        mz, pk, fbar, X, cnt_z, cnt_k = self.reductions(F)
        L = float(((mz - target_mz) ** 2).sum() + (((pk - target_pk) / target_pk) ** 2).sum())
        g_mz = 2 * (mz - target_mz) / cnt_z                     # dL/dF_p via <F>_j
        g_pk = 2 * (pk - target_pk) / target_pk ** 2 / cnt_k    # dL/dP_(s,m) for (s,m) in bin
        gdF = np.zeros_like(F)
        for s in range(len(self.lengths)):
            o, n = self.offsets[s], self.lengths[s]
            k = _p1d.p1d_k(n, self.dx)
            idx = _p1d.bin_index(k, self.kedges)
            w = np.where(idx >= 0, g_pk[np.maximum(idx, 0)], 0.0) * self.dx / n
            Y = np.zeros(n, complex)
            Y[:len(w)] = w * X[s]
            gdF[o:o + n] = 2 * n * np.fft.ifft(Y).real
        npx = len(F)
        gF = g_mz[self.zbin] + gdF / fbar - (gdF * F).sum() / (npx * fbar ** 2)
        a, b, c = theta[self.zbin, 0], theta[self.zbin, 1], theta[self.zbin, 2]
        g = self.delta + c * self.eta
        tau1 = np.exp(b * self.G * g)
        dFa = -tau1 * F
        dFb = -a * tau1 * self.G * g * F
        dFc = -a * tau1 * b * self.G * self.eta * F
        grad = np.stack([np.bincount(self.zbin, gF * d, self.nzb) for d in (dFa, dFb, dFc)], 1)
        return L, grad

    def fd_grad(self, theta, target_mz, target_pk, h=1e-4):
        """Central differences, relative step h on each parameter."""
        grad = np.zeros_like(theta)
        for j in range(theta.shape[0]):
            for p in range(3):
                step = h * max(abs(theta[j, p]), 1e-3)
                tp = theta.copy()
                tm = theta.copy()
                tp[j, p] += step
                tm[j, p] -= step
                grad[j, p] = (self.loss(tp, target_mz, target_pk)
                              - self.loss(tm, target_mz, target_pk)) / (2 * step)
        return grad


def torch_loss(problem: ZBinProblem, theta, target_mz, target_pk):
    """The same loss written with torch operations in float64, so that torch.autograd gives its
    gradient (the reference-autograd check of the adjoint): FGPA per pixel with the
    parameters of the pixel's z bin, <F>_j by scatter-add, dF = F/<F> - 1, |rfft|^2 dx/N per
    skewer (skewers of one length batched), binned as MakeProfileHisto bins them."""
    import torch
    th = theta if isinstance(theta, torch.Tensor) else torch.as_tensor(theta, dtype=torch.float64)
    p = problem
    zb = torch.as_tensor(p.zbin)
    delta, eta, G = (torch.as_tensor(x) for x in (p.delta, p.eta, p.G))
    a, b, c = th[zb, 0], th[zb, 1], th[zb, 2]
    F = torch.exp(-a * torch.exp(b * G * (delta + c * eta)))
    cnt_z = torch.bincount(zb, minlength=p.nzb).double()
    mz = torch.zeros(p.nzb, dtype=torch.float64).index_add(0, zb, F) / cnt_z
    dF = F / F.mean() - 1
    psum = torch.zeros(p.nkb, dtype=torch.float64)
    cnt_k = torch.zeros(p.nkb, dtype=torch.float64)
    for n in np.unique(p.lengths):
        rows = np.nonzero(p.lengths == n)[0]
        idx = torch.as_tensor((p.offsets[rows][:, None] + np.arange(n)[None, :]).ravel())
        X = torch.fft.rfft(dF[idx].reshape(len(rows), int(n)), dim=1)
        P = (X.real ** 2 + X.imag ** 2) * p.dx / n
        kb = _p1d.bin_index(_p1d.p1d_k(int(n), p.dx), p.kedges)
        m = kb >= 0
        kbt = torch.as_tensor(kb[m])
        psum = psum.index_add(0, kbt, P[:, torch.as_tensor(m)].sum(0))
        cnt_k = cnt_k.index_add(0, kbt, torch.full((int(m.sum()),), float(len(rows)), dtype=torch.float64))
    pk = psum / cnt_k
    tm = torch.as_tensor(np.asarray(target_mz, np.float64))
    tp = torch.as_tensor(np.asarray(target_pk, np.float64))
    return ((mz - tm) ** 2).sum() + (((pk - tp) / tp) ** 2).sum()
