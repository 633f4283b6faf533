"""The CPU oracle against golden vectors produced by running the reference's own code
(tests/golden/make_golden.py).  These pin the restatement before it is trusted."""
import numpy as np
import pytest

from oracle import fgpa_pdf, fit, grf, p1d, skewers


@pytest.mark.parametrize("tag", ["cube16", "rect"])
def test_grf_bit_exact_vs_make_boxes(golden, tag):
    f = golden(f"grf_{tag}.npz")
    NX, NY, NZ = int(f["NX"]), int(f["NY"]), int(f["NZ"])
    dx, k0 = float(f["DX"]), float(f["k0"])
    assert grf.pk_normalisation(NX, NY, NZ, dx, k0) == pytest.approx(float(f["A"]), rel=1e-14)
    assert np.array_equal(grf.sqrt_pk_grid(NX, NY, NZ, dx, k0), f["P0"])
    noise = grf.draw_noise(NX, NY, NZ, int(f["seed"]))
    out = grf.grf_boxes(noise, dx, k0, eta=grf.ETA_COMPONENTS, precision="f32")
    assert np.array_equal(out["delta"], f["delta"])
    for c in grf.ETA_COMPONENTS:
        assert np.array_equal(out["eta_" + c], f["eta_" + c])
    assert out["sigma"] == pytest.approx(float(f["sigma"]), rel=1e-6)
    # the FP64 oracle differs from the reference's FP32 arrays only by FP32 rounding
    o64 = grf.grf_boxes(noise, dx, k0, eta=("zz",), precision="f64")
    d = o64["delta"] - f["delta"]
    assert np.sqrt((d ** 2).mean() / (o64["delta"] ** 2).mean()) < 2e-7


@pytest.mark.parametrize("tag", ["cube16", "rect"])
def test_lognormal_and_velocity_boxes_bit_exact(golden, tag):
    """boxln_1..3 (raw modes x Pln grids) and vx, vy, vz (-i k_i/k^2 H0 dD/dz(0) x P0-scaled
    modes) of the reference's main() (bin/make_boxes.py:241-275, 393-431)."""
    f = golden(f"grf_{tag}.npz")
    NX, NY, NZ = int(f["NX"]), int(f["NY"]), int(f["NZ"])
    dx, k0 = float(f["DX"]), float(f["k0"])
    noise = grf.draw_noise(NX, NY, NZ, int(f["seed"]))
    nk = np.fft.rfftn(noise.astype(np.float64))
    for i in (1, 2, 3):
        out = grf.grf_from_modes(nk, NZ, dx, k0, eta=(), P0=f[f"Pln{i}"])
        assert np.array_equal(out["delta"], f[f"boxln_{i}"]), i
    out = grf.grf_from_modes(nk, NZ, dx, k0, eta=(), velocity=(float(f["H0"]), float(f["dgrowth0"])))
    for c in grf.VELOCITY_COMPONENTS:
        assert np.array_equal(out[c], f[c]), c


def test_grf_scaled_k_box_matches_checkpoint(golden):
    """boxk.npy after the P0 multiply (bin/make_boxes.py:289-291)."""
    f = golden("grf_cube16.npz")
    noise = grf.draw_noise(16, 16, 16, int(f["seed"]))
    nk = np.fft.rfftn(noise.astype(np.float64)).astype(np.complex64) * f["P0"]
    assert np.array_equal(nk, f["boxk_scaled"])


def test_gauss343_matches_readspec(golden):
    g = golden("grf_cube16.npz")
    r = golden("readspec.npz")
    NX = int(g["NX"])
    dx = float(g["DX"])
    L = NX * dx
    R0 = float(r["R0"])
    for s in range(r["pos"].shape[0]):
        xyz = r["XYZ"][s]
        pos = np.stack([xyz[:, 0] + L / 2, xyz[:, 1] + L / 2, xyz[:, 2] + L / 2 - R0], 1)
        boxes = [g["delta"]] + [g["eta_" + c] for c in grf.ETA_COMPONENTS]
        vals = skewers.gauss343(boxes, pos, dx)
        np.testing.assert_allclose(vals[0], r["delta_l"][s], rtol=1e-12, atol=1e-14)
        eta6 = dict(zip(grf.ETA_COMPONENTS, vals[1:]))
        ep = skewers.eta_par_projection(eta6, xyz)
        np.testing.assert_allclose(ep, r["eta_par"][s], rtol=1e-11, atol=1e-14)


def _merge_restated(f, scale_fn):
    order = f["order"]
    rs = np.random.RandomState(int(f["seed"]))
    flux, ds_all = [], []
    z = f["redshift"]                                  # float32, as read from the file
    G = skewers.growth_merge(z)
    for s in order:
        n = len(z)
        nz = skewers.nz_rule(n)
        noise = rs.normal(size=nz)
        ds = skewers.small_scales(noise, n, scale_fn(nz, z))
        ds_all.append(ds)
        flux.append(skewers.fgpa(f["delta_l_in"][s] + ds, f["eta_par_in"][s], G, 0.1, 1.6, 0.5))
    return np.array(flux), np.array(ds_all)


def test_small_scales_and_fgpa_match_merge_spectra_fit_path(golden):
    f = golden("merge_fitp1d.npz")
    from scipy.interpolate import InterpolatedUnivariateSpline
    kt = np.linspace(0.0, float(f["pm_kmax"]), int(f["pm_n"]))
    pt = float(f["pm_amp"]) * np.exp(-(kt / float(f["pm_kscale"])) ** 2) + float(f["pm_floor"])
    spl = InterpolatedUnivariateSpline(kt, pt)

    def scale(nz, z):
        return skewers.small_scale_scale(nz, 0.2, spl)
    flux, ds = _merge_restated(f, scale)
    np.testing.assert_allclose(ds, f["delta_s"], rtol=0, atol=1e-6)     # stored as float32
    np.testing.assert_allclose(flux, f["flux"], rtol=2e-6, atol=1e-7)


def test_small_scales_table_path_with_sigma_correction(golden):
    """Non-fit branch: nearest-z table, interp1d in k, clip, sigma_s(z)/sigma_s(zeff)."""
    f = golden("merge_table.npz")
    zt, kt, pk, sig = f["pm_z"], f["pm_k"], f["pm_pk"], f["pm_sigma"]
    order = f["order"]
    rs = np.random.RandomState(int(f["seed"]))
    z = f["redshift"]
    wav = f["wav"]
    G = skewers.growth_merge(z)
    for row, s in enumerate(order):
        n = len(z)
        nz = skewers.nz_rule(n)
        noise = rs.normal(size=nz)
        wav_rf = wav / (1 + f["zq"][s])
        mmm = np.where((wav_rf < skewers.LYA) & (wav_rf > 0.0))[0]
        zeff = z[mmm].mean()
        iz = np.argsort(np.abs(zt - zeff))[0]
        pm = lambda k: np.interp(k, kt, pk[iz])   # noqa: E731
        ds = skewers.small_scales(noise, n, skewers.small_scale_scale(nz, 0.2, pm))
        ds = ds * np.interp(z, zt, sig) / np.interp(zeff, zt, sig)
        np.testing.assert_allclose(ds, f["delta_s"][row], rtol=0, atol=1e-6)
        F = skewers.fgpa(f["delta_l_in"][s] + ds, f["eta_par_in"][s], G, 0.1, 1.6, 0.5)
        np.testing.assert_allclose(F, f["flux"][row], rtol=2e-6, atol=1e-7)


def test_util_functions(golden):
    u = golden("util.npz")
    np.testing.assert_array_equal(skewers.fgpa(u["delta"], u["eta"], u["G"], 0.1, 1.6, 0.5),
                                  u["F_scalar"])
    np.testing.assert_array_equal(
        skewers.fgpa(u["delta"], u["eta"], u["G"], u["a_arr"], u["b_arr"], u["c_arr"]),
        u["F_array"])
    np.testing.assert_allclose(skewers.fgrowth(u["zg"], 0.31457), u["fg"], rtol=1e-14)
    assert skewers.sigma_p1d(skewers.pmiss_analytic, 0.2, 10000) == pytest.approx(
        float(u["sig_s"]), rel=1e-13)


def test_p1d_estimator_and_profile(golden):
    u = golden("util.npz")
    lens = u["spec_lens"]
    off = np.concatenate([[0], np.cumsum(lens)])
    specs = [u["specs"][off[i]:off[i + 1]] for i in range(len(lens))]
    np.testing.assert_allclose(p1d.p1d_1spectrum(specs[1], 0.2), u["one"], rtol=1e-12)
    k, pk, err = p1d.binned_p1d(specs, 0.2, u["p1d_bins"])
    np.testing.assert_allclose(k, u["k_b"], rtol=1e-12)
    np.testing.assert_allclose(pk, u["p_b"], rtol=1e-12)
    np.testing.assert_allclose(err, u["e_b"], rtol=1e-9)
    mx, my, me = p1d.profile_histo(u["xh"], u["yh"], np.linspace(0, 12, 13))
    np.testing.assert_allclose(mx, u["mx"], rtol=1e-12)
    np.testing.assert_allclose(my, u["my"], rtol=1e-12)
    np.testing.assert_allclose(me, u["me"], rtol=1e-9)


def test_fgpa_pdf_known_answer(golden):
    """bin/param_setting.py:112: (<F>, sigma_F) = (0.791119, 0.360234)."""
    u = golden("util.npz")
    m = fgpa_pdf.f_mean(float(u["fm_ln_a"]), float(u["fm_b"]))
    s2 = fgpa_pdf.f_sig2(float(u["fm_ln_a"]), float(u["fm_b"]))
    assert m == pytest.approx(float(u["fmean"]), rel=1e-10)
    assert s2 == pytest.approx(float(u["sig2F"]), rel=1e-9)
    assert m == pytest.approx(0.791119, abs=1e-6)
    assert np.sqrt(s2) == pytest.approx(0.360234, abs=1e-6)


def test_fit_az_chi2(golden):
    u = golden("util.npz")
    for a, ref in zip(u["fit_a"], u["fit_chi2"]):
        c = fit.fit_az_chi2(float(a), 1.6, 0.5, u["fit_dl"], u["fit_ds"], u["fit_eta"],
                            u["fit_mask"], u["fit_gf"], u["fit_bins"], u["fit_pk"],
                            u["fit_pkerr"])
        assert c == pytest.approx(float(ref), rel=1e-10)


def test_zbin_loss_gradient_matches_central_differences():
    rng = np.random.RandomState(0)
    lengths = rng.randint(40, 90, size=12)
    n = lengths.sum()
    z = np.concatenate([np.linspace(1.8, 3.6, L) for L in lengths])
    prob = fit.ZBinProblem(rng.normal(0, 1, n), rng.normal(0, 0.4, n), np.ones(n), z, lengths,
                           np.linspace(1.8, 3.6, 4), np.logspace(np.log10(0.3), np.log10(15.0), 6),
                           0.2)
    truth = np.tile([0.1, 1.58, 0.6], (3, 1))
    F = prob.flux(truth)
    mz, pk, *_ = prob.reductions(F)
    theta = np.tile([0.15, 1.3, 0.4], (3, 1))
    L, g = prob.loss_grad(theta, mz, pk)
    gfd = prob.fd_grad(theta, mz, pk, h=1e-5)
    np.testing.assert_allclose(g, gfd, rtol=2e-5, atol=1e-9 * np.abs(gfd).max())


def test_c_oracle_matches_numpy_oracle():
    """The C restatement (CPU baseline) against the numpy restatement on one box."""
    from oracle import cskewers
    rs = np.random.RandomState(4)
    nx, ny, nz, dx = 12, 10, 16, 2.19
    pitch = 24
    box = np.zeros((nx, ny, pitch), np.float32)
    eta = np.zeros((nx, ny, pitch), np.float32)
    box[..., :nz] = rs.normal(size=(nx, ny, nz))
    eta[..., :nz] = rs.normal(size=(nx, ny, nz)) * 0.3
    n = 7
    start = rs.uniform(0, 1, (n, 3)) * np.array([nx, ny, nz]) * dx
    d = rs.normal(size=(n, 3)) * 0.1 + np.array([0, 0, 1.0])
    d /= np.linalg.norm(d, axis=1)[:, None]
    npix = rs.randint(20, 200, n)
    off = np.concatenate([[0], np.cumsum(npix)[:-1]])
    st32, d32 = start.astype(np.float32), d.astype(np.float32)
    F = cskewers.skewer_flux(st32, d32, npix, off, 0.2, box, eta, nz, dx, abc_mode=1, a=0.1,
                             b=1.58, c=0.6, growth_mode=1, growth24=float(skewers.fgrowth(2.4)))
    ref = skewers.skewer_flux(box[..., :nz], eta[..., :nz],
                              dict(start=st32.astype(np.float64), dir=d32.astype(np.float64), npix=npix),
                              dx, dpix=0.2, fgpa_mode=dict(kind="powerlaw_x", a0=0.1, zref1=3.2,
                                                           power=4.5, b=1.58, c=0.6, G="merge"))
    np.testing.assert_allclose(F, np.concatenate(ref["F"]), rtol=0, atol=1e-6)
