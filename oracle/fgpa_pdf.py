"""Analytic moments of the FGPA flux for a Gaussian field (known answers for the kernels).

Restates py/SaclayMocks/FGPApdf.py:11-58: for g ~ N(0,1) and F = exp(-exp(b g + ln a)),
<F> and <F^2> are integrals of the closed-form pdf of F, split at 1-1e-8 where the pdf
diverges.  bin/param_setting.py:112 records the pair (<F>, sigma_F) =
(0.791119, 0.360234) <-> (ln a, b sigma_g) = (-5.3199529, 5.71883103).
TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import numpy as np
from scipy import integrate, special


def f_pdf(F, ln_a, b):
    tau = -np.log(F)
    xx = np.log(tau) - ln_a
    return np.exp(-xx * xx / 2 / b / b) / (F * tau * np.sqrt(2 * np.pi) * b)


def _cdf(Fmax, ln_a, b):
    u = ln_a - np.log(-np.log(Fmax))
    return 0.5 * (1 + special.erf(u / b / np.sqrt(2)))


def f_moment(n: int, ln_a: float, b: float) -> float:
    """<F^n> = int_0^{1-eps} F^n pdf dF + P(F > 1-eps) (FGPApdf.py:39-55)."""
    eps = 1e-8
    v = integrate.quad(lambda F: F ** n * f_pdf(F, ln_a, b), 0, 1 - eps)[0]
    return v + 1 - _cdf(1 - eps, ln_a, b)


def f_mean(ln_a: float, b: float) -> float:
    return f_moment(1, ln_a, b)


def f_sig2(ln_a: float, b: float) -> float:
    return f_moment(2, ln_a, b) - f_mean(ln_a, b) ** 2
