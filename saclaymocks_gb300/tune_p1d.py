"""The P1D-missing tuning loop on the GPU: fit_az.Fitter.iterate / read_p1dmiss /
gen_small_scales / compute_p1d (py/SaclayMocks/fit_az.py:121-132, 169-219, 281-332).

The reference tunes the power spectrum P1Dmiss(k) of the small-scale field delta_s so that the
flux P1D of the mock, F = fgpa(delta_l + delta_s, eta_par, G, a, b, c), matches a model P1D:
each iteration multiplies P1Dmiss by 1 + lambda (r_smooth(k) - 1), r = P_model / P_mock
smoothed by a spline, regenerates delta_s with the new P1Dmiss and recomputes the mock P1D.

Here the per-pixel fields stay on the GPU: delta_s is drawn by the skewer kernel in pixel mode
(Philox Fourier modes, sqrt(P1Dmiss/pixel) tables rebuilt from the spline each iteration), and
mean flux + binned P1D (mean, rms/sqrt(n)) come from the fit kernels' FP64 reductions.  The
spline update itself is host work on a few dozen numbers and restates the reference's code.
"""
from __future__ import annotations

import numpy as np
import scipy.interpolate as si
import torch

from . import _lib, fit, spectra


def iterate_p1dmiss(k, p1d, err_p1d, model_interp, p1dmiss_interp, convergence_factor=1.0,
                    convergence_criterium=None):
    """One update of fit_az.Fitter.iterate (py/SaclayMocks/fit_az.py:281-329) on the mock
    P1D (k, p1d, err_p1d at the bin means).  Returns (converged, max|r - 1|, p1dmiss at k,
    the smoothing spline of the new P1Dmiss); when converged the last two are None."""
    k = np.asarray(k, np.float64)
    rr = model_interp(k) / p1d
    s = len(k) * (err_p1d.mean() / p1d.mean()) ** 2 * 0.5
    rr_smooth = si.UnivariateSpline(k[3:], rr[3:], s=s)
    p1dmiss = p1dmiss_interp(k) * (1 + convergence_factor * (rr_smooth(k) - 1))
    s = len(k) * err_p1d.mean() ** 2 * 3
    new_interp = si.UnivariateSpline(k, p1dmiss, s=s)
    dev = float(np.max(np.abs(rr - 1)))
    if convergence_criterium and dev < convergence_criterium:
        return True, dev, None, None
    return False, dev, p1dmiss, new_interp


class P1DMissTuner:
    """The tuning loop for one redshift: fixed per-pixel delta_l, eta_par, growth G of a set
    of skewers (packed, lengths `lengths`), FGPA parameters (a, b, c), a model P1D (model_k,
    model_p1d in h/Mpc units) and the starting table (kmiss, p1dmiss) of read_p1dmiss.

    ``compute_p1d()`` draws delta_s (seed + iteration) and measures the mock P1D in the k
    bins `kedges`; ``iterate()`` updates P1Dmiss and recomputes; ``run(n)`` iterates until
    convergence or n iterations."""

    def __init__(self, delta_l, eta_par, growthf, lengths, a, b, c, kmiss, p1dmiss, model_k, model_p1d,
                 kedges, pixel=0.2, ss_nz=0, seed=0, convergence_factor=1.0, convergence_criterium=None,
                 device="cuda"):
        dv = torch.device(device)
        self.device = dv
        self.lengths = np.ascontiguousarray(lengths, np.int32)
        n = len(self.lengths)
        zero3 = np.zeros((n, 3), np.float32)
        self.table = spectra.SkewerTable(zero3, zero3, self.lengths, dpix=pixel)
        def f32(x):
            if isinstance(x, torch.Tensor):
                return x.to(device=dv, dtype=torch.float32).contiguous()
            return torch.as_tensor(np.asarray(x, np.float32)).to(dv).contiguous()
        self.delta_l = f32(delta_l)
        self.eta = f32(eta_par) if eta_par is not None else None
        self.G = f32(growthf) if growthf is not None else None
        self.zpix = torch.zeros_like(self.delta_l)
        self.theta = np.array([[a, b, c]], np.float64)
        self.pixel = float(pixel)
        self.ss_nz = int(ss_nz)
        self.seed = int(seed)
        self.convergence_factor = float(convergence_factor)
        self.convergence_criterium = convergence_criterium
        self.model_interp = si.interp1d(np.asarray(model_k, np.float64), np.asarray(model_p1d, np.float64))
        self.kmiss = np.asarray(kmiss, np.float64)
        self.p1dmiss = np.asarray(p1dmiss, np.float64)
        self.p1dmiss_interp = si.InterpolatedUnivariateSpline(self.kmiss, self.p1dmiss)
        self.niter = 0
        self.converged = False
        self.history = []
        # the problem's own delta buffer receives delta_l + delta_s each iteration
        self.problem = fit.FitProblem(self.delta_l.clone(), self.eta, self.G, np.zeros(self.table.total_pixels),
                                      self.lengths, np.array([-1.0, 1.0]), kedges, dx=pixel, device=dv)

    def gen_small_scales(self):
        """delta_l + delta_s into the fit problem's delta buffer: Philox small scales with
        sqrt(max(P1Dmiss, 0)/pixel) (fit_az.py:169-192; negative P1Dmiss clipped as there)."""
        interp = self.p1dmiss_interp
        cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=self.ss_nz, pmiss=lambda kk: interp(kk),
                                    pixsize=self.pixel, seed=self.seed + self.niter)
        runner = spectra.SkewerRunner(self.table, cfg, device=self.device,
                                      pixels=(self.delta_l, None, self.zpix))
        _, dtot, _, _ = runner.run(want_fields=True)
        self.problem.delta.copy_(dtot)

    def compute_p1d(self):
        """Mock P1D after a fresh small-scale draw: (k mean, P, rms/sqrt(n)) per non-empty bin."""
        self.gen_small_scales()
        self.k, self.p1d, self.err_p1d = self.problem.p1d_profile(self.theta)
        return self.k, self.p1d, self.err_p1d

    def iterate(self):
        if not hasattr(self, "p1d"):
            self.compute_p1d()
        conv, dev, p1dmiss, interp = iterate_p1dmiss(self.k, self.p1d, self.err_p1d, self.model_interp,
                                                     self.p1dmiss_interp, self.convergence_factor,
                                                     self.convergence_criterium)
        self.history.append(dev)
        if conv:
            self.converged = True
            return
        self.p1dmiss = p1dmiss
        self.p1dmiss_interp = interp
        self.niter += 1
        self.compute_p1d()

    def run(self, n_iter: int):
        for _ in range(n_iter):
            self.iterate()
            if self.converged:
                break
        return self
