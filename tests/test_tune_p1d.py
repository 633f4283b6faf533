"""The P1D-missing tuning loop (fit_az.Fitter.iterate, py/SaclayMocks/fit_az.py:281-332): the
host update against the reference's own iterate() (tests/golden/iterate.npz), and on the GPU
the mock P1D profile against the oracle and a tuning run toward a known P1Dmiss."""
import numpy as np
import pytest
import scipy.interpolate as si

from saclaymocks_gb300 import tune_p1d


@pytest.mark.parametrize("tag,cf,crit", [("cf1", 1.0, None), ("cf0.6", 0.6, None), ("cf1_conv", 1.0, 1e3)])
def test_iterate_update_matches_reference(golden, tag, cf, crit):
    g = golden("iterate.npz")
    conv, dev, p1dmiss, interp = tune_p1d.iterate_p1dmiss(
        g["k"], g["p1d"], g["err"], si.interp1d(g["model_k"], g["model_p"]),
        si.InterpolatedUnivariateSpline(g["kmiss"], g["pmiss"]), cf, crit)
    assert conv == bool(g[tag + "_converged"])
    if conv:
        assert int(g[tag + "_niter"]) == 0
        return
    np.testing.assert_allclose(p1dmiss, g[tag + "_p1dmiss"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(interp(g["kmiss"]), g[tag + "_interp_on_kmiss"], rtol=1e-10, atol=1e-14)


@pytest.mark.gpu
def test_gpu_profile_and_tuning_toward_known_p1dmiss():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import p1d as op1d
    from oracle import philox as ophilox
    from saclaymocks_gb300 import spectra
    rng = np.random.RandomState(4)
    lengths = rng.randint(300, 900, size=400).astype(np.int32)
    n = int(lengths.sum())
    delta_l = (0.8 * rng.normal(size=n)).astype(np.float32)
    eta = (0.3 * rng.normal(size=n)).astype(np.float32)
    kedges = np.linspace(0.1, 10.0, 25)
    kmiss = np.arange(0.0, 20.0, 0.01)
    true = 0.08 * np.exp(-(kmiss / 2.5) ** 2)
    a, b, c = 0.12, 1.58, 0.6
    # target: the P1D of the same fields with the true P1Dmiss
    ref = tune_p1d.P1DMissTuner(delta_l, eta, None, lengths, a, b, c, kmiss, true, kmiss, true + 1.0,
                                kedges, ss_nz=1024, seed=9)
    kt, pt, et = ref.compute_p1d()
    # the profile of the GPU reductions against the oracle on the same total field
    dtot = ref.problem.delta.cpu().numpy().astype(np.float64)
    offs = np.concatenate([[0], np.cumsum(lengths[:-1])])
    F = np.exp(-a * np.exp(b * (dtot + c * eta.astype(np.float64))))
    dF = F / F.mean() - 1
    ko, po, eo = op1d.profile_histo(*_modes(dF, offs, lengths, 0.2), kedges)
    np.testing.assert_allclose(kt, ko, rtol=1e-10)
    np.testing.assert_allclose(pt, po, rtol=2e-4)
    np.testing.assert_allclose(et, eo, rtol=2e-3)
    # tune from a P1Dmiss twice too large toward the target (same noise seed)
    model_k = np.concatenate([[0.0], kt, [20.0]])
    model_p = np.concatenate([[pt[0]], pt, [pt[-1]]])
    tuner = tune_p1d.P1DMissTuner(delta_l, eta, None, lengths, a, b, c, kmiss, 2.0 * true, model_k, model_p,
                                  kedges, ss_nz=1024, seed=9, convergence_factor=1.0)
    tuner.compute_p1d()
    tuner.seed = 9 - 1          # every iteration redraws with seed + niter: keep the target's noise
    tuner.run(4)
    assert tuner.history[-1] < 0.5 * tuner.history[0]


def _modes(dF, offs, lengths, dx):
    ks, ps = [], []
    for o, L in zip(offs, lengths):
        x = np.fft.rfft(dF[o:o + L])
        ks.append(np.fft.rfftfreq(L) * 2 * np.pi / dx)
        ps.append((x.real ** 2 + x.imag ** 2) * dx / L)
    return np.concatenate(ks), np.concatenate(ps)
