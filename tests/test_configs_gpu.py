"""Parity at the sizes of the configurations, against the FP64 oracle.

* The small plain configuration exactly as specified: 256^3 box of 2.19 Mpc/h cells, white
  noise drawn from numpy's RandomState(0) in the reference's plane order, P(k) = A k/(1 +
  (k/0.02)^2)^2 with E[var delta] = 1, delta and eta_par = irfftn(kz^2/k^2 delta_k); 1000
  skewers along z at uniform (x, y), 256 cells each, trilinear read; FGPA a = 0.1, b = 1.6,
  c = 0.5, G = 1.  Tolerances: boxes relative RMS <= 1e-6 and max |err| <= 1e-5 sigma, flux
  |dF| <= 2e-6.
* The batching configuration's skewers: 3000 of the 5e4 log-uniform 64..2048-pixel skewers
  through the 1024^3 box (GPU noise, seed 2), small scales on the 256*2^n rule from host
  noise, a(z) = 0.1((1+z)/3.2)^4.5, b = 1.58, c = 0.6: the oracle reads the GPU machine.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import grf as ograf          # noqa: E402
from oracle import skewers as osk        # noqa: E402

REL_RMS, MAX_SIGMA, F_ATOL = 1e-6, 1e-5, 2e-6


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from saclaymocks_gb300 import _lib, grf, spectra
    return _lib, grf, spectra


def _box_err(gpu, ref):
    d = gpu.astype(np.float64) - ref
    return np.sqrt((d ** 2).mean() / (ref ** 2).mean()), np.abs(d).max() / ref.std()


def test_small_plain_configuration_exact(env):
    _lib, grf, spectra = env
    n, dx = 256, 2.19
    noise = ograf.draw_noise(n, n, n, 0)
    out = grf.make_boxes(n, n, n, dx, noise=torch.from_numpy(noise).cuda(), k0=0.02)
    t = spectra.skewers_parallel_z(1000, n, n, 256, dx, seed=0)
    cfg = spectra.SpectraConfig(a=0.1, b=1.6, c=0.5)
    F = spectra.SkewerRunner(t, cfg).run(out.delta_pad[0], out.eta_pad[0], nx=n, ny=n, nz=n,
                                         pitch=out.pitch, dcell=dx)
    torch.cuda.synchronize()
    out.check()
    o = ograf.grf_boxes(noise, dx, 0.02, eta=("zz",), precision="f64")
    for name, gpu, ref in (("delta", out.delta[0], o["delta"]), ("eta_zz", out.eta[0], o["eta_zz"])):
        rr, ma = _box_err(gpu.cpu().numpy(), ref)
        assert rr <= REL_RMS, f"{name}: relative RMS {rr:.3e}"
        assert ma <= MAX_SIGMA, f"{name}: max |err| / sigma {ma:.3e}"
    # flux on the oracle's own FP64 boxes: every pixel of every skewer
    pos = np.concatenate([osk.skewer_positions(t.start[s].astype(np.float64), t.direction[s].astype(np.float64),
                                               int(t.npix[s]), t.dpix) for s in range(t.n)])
    dl = osk.trilinear(o["delta"], pos, dx)
    et = osk.trilinear(o["eta_zz"], pos, dx)
    Fo = osk.fgpa(dl, et, 1.0, 0.1, 1.6, 0.5)
    err = np.abs(F.cpu().numpy().astype(np.float64) - Fo).max()
    assert err <= F_ATOL, f"flux max |dF| {err:.3e}"


def test_batching_configuration_skewers_through_1024_box(env):
    _lib, grf, spectra = env
    n, dx = 1024, 2.19
    out = grf.make_boxes(n, n, n, dx, seed=2)
    torch.cuda.synchronize()
    out.check()
    full = spectra.skewers_cone(50_000, np.array([n, n, n]) * dx, seed=2, npix_range=(64, 2048), log_uniform=True)
    k = 3000
    t = spectra.SkewerTable(full.start[:k], full.direction[:k], full.npix[:k], dpix=0.2)
    rs = np.random.RandomState(5)
    draws = [rs.normal(size=osk.nz_rule(int(m))).astype(np.float32) for m in t.npix]
    offs = np.concatenate([[0], np.cumsum([len(d) for d in draws])[:-1]]).astype(np.int64)
    noise = (torch.from_numpy(np.concatenate(draws)).cuda(), torch.from_numpy(offs).cuda())
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_HOST, ss_nz=0, abc_mode=_lib.SMK_ABC_POWERLAW, a=0.1,
                                a_zref1=3.2, a_power=4.5, b=1.58, c=0.6, z_lo=1.8, z_hi=3.6)
    F, dtot, eta, z = spectra.SkewerRunner(t, cfg).run(out.delta_pad[0], out.eta_pad[0], nx=n, ny=n, nz=n,
                                                       pitch=out.pitch, dcell=dx, noise=noise, want_fields=True)
    torch.cuda.synchronize()
    d = out.delta[0].cpu().numpy()
    e = out.eta[0].cpu().numpy()
    ref = osk.skewer_flux(d, e, dict(start=t.start.astype(np.float64), dir=t.direction.astype(np.float64),
                                     npix=t.npix), dx, dpix=0.2,
                          fgpa_mode=dict(kind="powerlaw_x", a0=0.1, zref1=3.2, power=4.5, b=1.58, c=0.6,
                                         z_lo=1.8, z_hi=3.6),
                          small=dict(pixsize=0.2, nz="rule", pmiss=osk.pmiss_analytic),
                          noise1d=[x.astype(np.float64) for x in draws])
    sig = float(d.std())
    Fg, dg = spectra.split(F, t), spectra.split(dtot, t)
    for s in range(k):
        np.testing.assert_allclose(Fg[s], ref["F"][s], rtol=0, atol=F_ATOL, err_msg=f"skewer {s}")
        np.testing.assert_allclose(dg[s], ref["delta"][s] + ref["delta_s"][s], rtol=0, atol=1e-5 * sig,
                                   err_msg=f"skewer {s}")
