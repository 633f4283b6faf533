"""Fused skewer kernel (trilinear read + small scales + FGPA) through the C ABI against the
oracle on the same boxes, skewers and noise; and the merge_spectra golden vectors.

Tolerances (FP32 kernel vs FP64 oracle): |dF| <= 2e-6 (F in [0,1]); delta_l + delta_s and
eta_par within 1e-5 * sigma_delta.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import grf as ograf          # noqa: E402
from oracle import philox as ophilox     # noqa: E402
from oracle import skewers as osk        # noqa: E402

F_ATOL = 2e-6
FIELD_TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from saclaymocks_gb300 import _lib, grf, spectra
    return _lib, grf, spectra


@pytest.fixture(scope="module")
def boxes(env):
    _, grf, _ = env
    nx, ny, nz, dx = 32, 24, 40, 2.19
    noise = np.random.RandomState(3).normal(size=(nx, ny, nz)).astype(np.float32)
    out = grf.make_boxes(nx, ny, nz, dx, noise=torch.from_numpy(noise).cuda())
    torch.cuda.synchronize()
    return dict(out=out, d=out.delta[0].cpu().numpy().astype(np.float64),
                e=out.eta[0].cpu().numpy().astype(np.float64), nx=nx, ny=ny, nz=nz, dx=dx)


def _run(env, boxes, table, cfg, noise=None):
    _lib, _, spectra = env
    r = spectra.SkewerRunner(table, cfg)
    out = boxes["out"]
    F, dtot, eta, z = r.run(out.delta_pad[0], out.eta_pad[0], nx=boxes["nx"], ny=boxes["ny"],
                            nz=boxes["nz"], pitch=out.pitch, dcell=boxes["dx"], noise=noise,
                            want_fields=True)
    torch.cuda.synchronize()
    sp = spectra.split
    return sp(F, table), sp(dtot, table), sp(eta, table), sp(z, table)


def _oracle(boxes, table, fg, small=None, noise1d=None):
    sk = dict(start=table.start.astype(np.float64), dir=table.direction.astype(np.float64),
              npix=table.npix)
    return osk.skewer_flux(boxes["d"], boxes["e"], sk, boxes["dx"], dpix=table.dpix,
                           fgpa_mode=fg, small=small, noise1d=noise1d)


def _cmp(gpu, ref, sig):
    for s in range(len(ref["F"])):
        np.testing.assert_allclose(gpu[0][s], ref["F"][s], rtol=0, atol=F_ATOL)
        np.testing.assert_allclose(gpu[1][s], ref["delta"][s] + ref["delta_s"][s], rtol=0,
                                   atol=FIELD_TOL * sig)
        np.testing.assert_allclose(gpu[2][s], ref["eta"][s], rtol=0, atol=FIELD_TOL * sig)
        np.testing.assert_allclose(gpu[3][s], ref["z"][s], rtol=0, atol=2e-6)


def test_parallel_z_trilinear_fgpa_const(env, boxes):
    """The small plain configuration: z-parallel skewers, trilinear read, a,b,c constant."""
    _lib, _, spectra = env
    t = spectra.skewers_parallel_z(40, boxes["nx"], boxes["ny"], 60, boxes["dx"], seed=0)
    cfg = spectra.SpectraConfig(a=0.1, b=1.6, c=0.5)
    g = _run(env, boxes, t, cfg)
    ref = _oracle(boxes, t, dict(kind="const", a=0.1, b=1.6, c=0.5))
    _cmp(g, ref, np.std(boxes["d"]))


def test_cone_skewers_host_noise_small_scales_powerlaw(env, boxes):
    """Tilted skewers wrapping through the periodic box, host white noise (reference rule
    nz = 256*2^n >= npix+50), a(z) power law with z along x, G = merge_spectra growth."""
    _lib, _, spectra = env
    L = np.array([boxes["nx"], boxes["ny"], boxes["nz"]]) * boxes["dx"]
    t = spectra.skewers_cone(25, L, seed=4, npix_range=(150, 700))
    pm = spectra.pmiss_gauss(0.05, 2.0)
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_HOST, ss_nz=0, pmiss=pm,
                                abc_mode=_lib.SMK_ABC_POWERLAW, a=0.1, a_zref1=3.2, a_power=4.5,
                                b=1.58, c=0.6, growth=_lib.SMK_G_MERGE)
    rs = np.random.RandomState(9)
    noises = [rs.normal(size=osk.nz_rule(int(n))) for n in t.npix]
    offs = np.concatenate([[0], np.cumsum([len(x) for x in noises])[:-1]]).astype(np.int64)
    packed = torch.from_numpy(np.concatenate(noises).astype(np.float32)).cuda()
    g = _run(env, boxes, t, cfg, noise=(packed, torch.from_numpy(offs).cuda()))
    fg = dict(kind="powerlaw_x", a0=0.1, zref1=3.2, power=4.5, b=1.58, c=0.6, G="merge")
    ref = _oracle(boxes, t, fg, small=dict(pixsize=0.2, nz="rule", pmiss=pm),
                  noise1d=[x.astype(np.float32).astype(np.float64) for x in noises])
    _cmp(g, ref, np.std(boxes["d"]))


def test_fixed_nz_philox_small_scales(env, boxes):
    """Fixed 2048-point small-scale grid with the GPU noise, against the numpy restatement of
    the same Philox stream."""
    _lib, _, spectra = env
    L = np.array([boxes["nx"], boxes["ny"], boxes["nz"]]) * boxes["dx"]
    t = spectra.skewers_cone(15, L, seed=8, npix_range=(400, 1200))
    pm = spectra.pmiss_gauss(0.05, 2.0)
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=2048, pmiss=pm, seed=77,
                                a=0.1, b=1.58, c=0.6)
    g = _run(env, boxes, t, cfg)
    scale = osk.small_scale_scale(2048, 0.2, pm)
    ref = _oracle(boxes, t, dict(kind="const", a=0.1, b=1.58, c=0.6))
    for s in range(t.n):
        ds = ophilox.skewer_small_scales(s, 2048, 77, scale, int(t.npix[s]))
        ref["delta_s"][s] = ds
        ref["F"][s] = osk.fgpa(ref["delta"][s] + ds, ref["eta"][s], 1.0, 0.1, 1.58, 0.6)
    _cmp(g, ref, np.std(boxes["d"]))


def test_philox_small_scale_variance_matches_sigma_p1d(env, boxes):
    """Statistical check of the GPU noise mode: std of delta_s vs util.sigma_p1d."""
    _lib, _, spectra = env
    n = 4000
    t = spectra.skewers_parallel_z(n, boxes["nx"], boxes["ny"], 1000, boxes["dx"], seed=1, dpix=0.2)
    pm = spectra.pmiss_gauss(0.05, 2.0)
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=2048, pmiss=pm, seed=5)
    r = spectra.SkewerRunner(t, cfg)
    out = boxes["out"]
    F, dtot, _, _ = r.run(out.delta_pad[0], out.eta_pad[0], nx=boxes["nx"], ny=boxes["ny"],
                          nz=boxes["nz"], pitch=out.pitch, dcell=boxes["dx"], want_fields=True)
    # delta_s = (delta_l + delta_s) - delta_l: rerun without small scales
    r0 = spectra.SkewerRunner(t, spectra.SpectraConfig())
    _, dl, _, _ = r0.run(out.delta_pad[0], out.eta_pad[0], nx=boxes["nx"], ny=boxes["ny"],
                         nz=boxes["nz"], pitch=out.pitch, dcell=boxes["dx"], want_fields=True)
    ds = (dtot - dl).double().cpu().numpy()
    expect = osk.sigma_p1d(pm, 0.2, 2048)
    assert ds.std() == pytest.approx(expect, rel=0.01)
    assert abs(ds.mean()) < 0.01 * expect


def test_abc_table_mode(env, boxes):
    _lib, _, spectra = env
    t = spectra.skewers_parallel_z(20, boxes["nx"], boxes["ny"], 80, boxes["dx"], seed=2)
    zt = np.linspace(1.8, 3.6, 101)
    tab = np.stack([zt, 0.05 + 0.1 * (zt - 1.8), 1.6 - 0.1 * (zt - 1.8), 0.5 + 0.05 * (zt - 1.8)], 1)
    cfg = spectra.SpectraConfig(abc_mode=_lib.SMK_ABC_TABLE, abc_table=tab)
    g = _run(env, boxes, t, cfg)
    ref = _oracle(boxes, t, dict(kind="const", a=0, b=0, c=0))
    for s in range(t.n):
        z = ref["z"][s]
        a = np.interp(z, zt, tab[:, 1])
        b = np.interp(z, zt, tab[:, 2])
        c = np.interp(z, zt, tab[:, 3])
        ref["F"][s] = osk.fgpa(ref["delta"][s], ref["eta"][s], 1.0, a, b, c)
    _cmp(g, ref, np.std(boxes["d"]))


@pytest.mark.parametrize("tag", ["fitp1d"])
def test_pixel_mode_matches_merge_spectra_golden(env, golden, tag):
    """SMK_INTERP_PIXELS is the merge_spectra step: per-pixel delta_l, eta_par, z in, the
    reference's own white noise (RandomState(seed+islice), ID order), FLUX out."""
    _lib, _, spectra = env
    f = golden(f"merge_{tag}.npz")
    order = f["order"]
    n_sp, npx = f["delta_l_in"].shape
    z = f["redshift"].astype(np.float32)
    table = spectra.SkewerTable(np.zeros((n_sp, 3)), np.tile([0, 0, 1.0], (n_sp, 1)),
                                np.full(n_sp, npx), dpix=0.2)
    dl = torch.from_numpy(np.ascontiguousarray(f["delta_l_in"][order]).reshape(-1)).cuda()
    et = torch.from_numpy(np.ascontiguousarray(f["eta_par_in"][order]).reshape(-1)).cuda()
    zz = torch.from_numpy(np.tile(z, n_sp)).cuda()
    from scipy.interpolate import InterpolatedUnivariateSpline
    kt = np.linspace(0.0, float(f["pm_kmax"]), int(f["pm_n"]))
    spl = InterpolatedUnivariateSpline(kt, float(f["pm_amp"]) * np.exp(-(kt / float(f["pm_kscale"])) ** 2)
                                       + float(f["pm_floor"]))
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_HOST, ss_nz=0, pmiss=spl, a=0.1, b=1.6, c=0.5,
                                growth=_lib.SMK_G_MERGE)
    rs = np.random.RandomState(int(f["seed"]))
    nz = osk.nz_rule(npx)
    noise = np.concatenate([rs.normal(size=nz) for _ in range(n_sp)]).astype(np.float32)
    offs = np.arange(n_sp, dtype=np.int64) * nz
    r = spectra.SkewerRunner(table, cfg, pixels=(dl, et, zz))
    F, dtot, _, _ = r.run(noise=(torch.from_numpy(noise).cuda(), torch.from_numpy(offs).cuda()),
                          want_fields=True)
    torch.cuda.synchronize()
    F = F.cpu().numpy().reshape(n_sp, npx)
    ds = dtot.cpu().numpy().reshape(n_sp, npx) - f["delta_l_in"][order]
    np.testing.assert_allclose(ds, f["delta_s"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(F, f["flux"], rtol=0, atol=F_ATOL)


# ----------------------------------------------------------------------------- Gaussian 7^3 read
ETA6 = ("xx", "yy", "zz", "xy", "xz", "yz")


def _padded(box, pitch):
    nx, ny, nz = box.shape
    t = torch.zeros((nx, ny, pitch), dtype=torch.float32)
    t[:, :, :nz] = torch.from_numpy(np.ascontiguousarray(box, np.float32))
    return t.cuda()


def _readspec_table(spectra, r):
    pos = r["pos"]                                            # (n, 60, 3), corner frame
    d = pos[:, 1] - pos[:, 0]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return spectra.SkewerTable(pos[:, 0].copy(), d, np.full(len(pos), pos.shape[1], np.int32), dpix=0.2)


def _gauss_run(env, table, cfg, delta_box, eta6, nxyz, pitch, dx):
    _, _, spectra = env
    run = spectra.SkewerRunner(table, cfg)
    F, dl, et, z = run.run(delta_box, None, nx=nxyz[0], ny=nxyz[1], nz=nxyz[2], pitch=pitch, dcell=dx,
                           want_fields=True, eta6=eta6)
    torch.cuda.synchronize()
    return spectra.split(dl, table), spectra.split(et, table)


def test_gauss343_read_of_reference_boxes_matches_readspec(env, golden):
    """SMK_INTERP_GAUSS343 on the reference's own delta and eta_ij boxes against ReadSpec
    (bin/make_spectra.py:39-139) run by the reference: delta_l and eta_par per pixel."""
    _lib, grf, spectra = env
    g, r = golden("grf_cube16.npz"), golden("readspec.npz")
    n, dx, R0 = int(g["NX"]), float(g["DX"]), float(r["R0"])
    L = n * dx
    pitch = grf.pitch_of(n)
    cfg = spectra.SpectraConfig(read="gauss343", observer=(L / 2, L / 2, L / 2 - R0))
    t = _readspec_table(spectra, r)
    dl, et = _gauss_run(env, t, cfg, _padded(g["delta"], pitch), [_padded(g["eta_" + c], pitch) for c in ETA6],
                        (n, n, n), pitch, dx)
    sig = float(np.std(g["delta"]))
    for s in range(len(dl)):
        np.testing.assert_allclose(dl[s], r["delta_l"][s], rtol=0, atol=5e-6 * sig)
        np.testing.assert_allclose(et[s], r["eta_par"][s], rtol=0, atol=5e-6 * sig)


def test_gauss343_on_gpu_boxes_matches_readspec(env, golden):
    """The full chain: delta and the six eta_ij boxes made on the GPU from the reference's
    noise (eta_comp per component), then the Gaussian read, against ReadSpec's output."""
    _lib, grf, spectra = env
    g, r = golden("grf_cube16.npz"), golden("readspec.npz")
    n, dx, R0 = int(g["NX"]), float(g["DX"]), float(r["R0"])
    L = n * dx
    noise = torch.from_numpy(ograf.draw_noise(n, n, n, int(g["seed"]))).cuda()
    outs = [grf.make_boxes(n, n, n, dx, noise=noise, k0=float(g["k0"]), eta_comp=c) for c in ETA6]
    torch.cuda.synchronize()
    for c, o in zip(ETA6, outs):
        e = o.eta[0].cpu().numpy()
        assert np.abs(e - g["eta_" + c]).max() < 1e-5 * np.std(g["delta"]), c
    cfg = spectra.SpectraConfig(read="gauss343", observer=(L / 2, L / 2, L / 2 - R0))
    t = _readspec_table(spectra, r)
    dl, et = _gauss_run(env, t, cfg, outs[0].delta_pad[0], [o.eta_pad[0] for o in outs], (n, n, n),
                        outs[0].pitch, dx)
    sig = float(np.std(g["delta"]))
    for s in range(len(dl)):
        np.testing.assert_allclose(dl[s], r["delta_l"][s], rtol=0, atol=1e-5 * sig)
        np.testing.assert_allclose(et[s], r["eta_par"][s], rtol=0, atol=1e-5 * sig)


def test_gauss343_periodic_wrap_vs_oracle(env, boxes):
    """Tilted skewers leaving the box: the 7^3 neighbourhoods wrap periodically; eta_par
    projected on the unwrapped observer->pixel vector; no RSD boxes gives eta_par = 0."""
    _lib, grf, spectra = env
    nx, ny, nz, dx = boxes["nx"], boxes["ny"], boxes["nz"], boxes["dx"]
    t = spectra.skewers_cone(12, (nx * dx, ny * dx, nz * dx), seed=4, max_angle_deg=35.0)
    t = spectra.SkewerTable(t.start, t.direction, np.minimum(t.npix, 500).astype(np.int32), dpix=t.dpix)
    rs = np.random.RandomState(9)
    eta6 = [rs.normal(size=(nx, ny, nz)).astype(np.float32) for _ in ETA6]
    pitch = boxes["out"].pitch
    obs = (0.3 * nx * dx, 0.6 * ny * dx, -120.0)
    cfg = spectra.SpectraConfig(read="gauss343", observer=obs)
    dl, et = _gauss_run(env, t, cfg, boxes["out"].delta_pad[0], [_padded(e, pitch) for e in eta6],
                        (nx, ny, nz), pitch, dx)
    dl0, et0 = _gauss_run(env, t, cfg, boxes["out"].delta_pad[0], None, (nx, ny, nz), pitch, dx)
    sig = float(np.std(boxes["d"]))
    for s in range(t.n):
        i = np.arange(t.npix[s])
        pos = t.start[s].astype(np.float64) + (i * t.dpix)[:, None] * t.direction[s].astype(np.float64)
        vals = osk.gauss343([boxes["d"]] + [e.astype(np.float64) for e in eta6], pos, dx)
        ep = osk.eta_par_projection(dict(zip(ETA6, vals[1:])), pos - np.asarray(obs))
        np.testing.assert_allclose(dl[s], vals[0], rtol=0, atol=1e-5 * sig)
        np.testing.assert_allclose(et[s], ep, rtol=0, atol=1e-5)
        np.testing.assert_array_equal(dl0[s], dl[s])
        assert not np.any(et0[s])


def test_one_skewer_per_item_schedule_matches_paired(env, boxes):
    """The one-skewer-per-work-item schedule (the baseline of the paired one) gives the same
    flux up to float32 rounding of the packed complex FFT."""
    _lib, _, spectra = env
    L = np.array([boxes["nx"], boxes["ny"], boxes["nz"]]) * boxes["dx"]
    t = spectra.skewers_cone(33, L, seed=5, npix_range=(60, 700), log_uniform=True)
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=0, seed=3)
    out = boxes["out"]
    kw = dict(nx=boxes["nx"], ny=boxes["ny"], nz=boxes["nz"], pitch=out.pitch, dcell=boxes["dx"])
    fp = spectra.SkewerRunner(t, cfg).run(out.delta_pad[0], out.eta_pad[0], **kw)
    fs = spectra.SkewerRunner(t, cfg, pair=False).run(out.delta_pad[0], out.eta_pad[0], **kw)
    torch.cuda.synchronize()
    assert float((fp - fs).abs().max()) <= F_ATOL


def test_skewer_launch_replayed_from_a_cuda_graph_equals_eager(env, boxes):
    _lib, _, spectra = env
    L = np.array([boxes["nx"], boxes["ny"], boxes["nz"]]) * boxes["dx"]
    t = spectra.skewers_cone(40, L, seed=6, npix_range=(100, 500))
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=1024, seed=4)
    out = boxes["out"]
    kw = dict(nx=boxes["nx"], ny=boxes["ny"], nz=boxes["nz"], pitch=out.pitch, dcell=boxes["dx"])
    run = spectra.SkewerRunner(t, cfg)
    eager = run.run(out.delta_pad[0], out.eta_pad[0], **kw).clone()
    flux = torch.zeros_like(eager)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        run.run(out.delta_pad[0], out.eta_pad[0], flux=flux, **kw)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(flux, eager)


def test_empty_table_and_zero_or_one_pixel_skewers(env, boxes):
    """Edge cases: an empty skewer table is a no-op; skewers of 0 and 1 pixels mixed with long
    ones (ragged, odd counts per FFT length) match the oracle."""
    _lib, _, spectra = env
    out = boxes["out"]
    kw = dict(nx=boxes["nx"], ny=boxes["ny"], nz=boxes["nz"], pitch=out.pitch, dcell=boxes["dx"])
    empty = spectra.SkewerTable(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0, np.int32))
    f = spectra.SkewerRunner(empty, spectra.SpectraConfig()).run(out.delta_pad[0], out.eta_pad[0], **kw)
    torch.cuda.synchronize()
    assert f.numel() == 0
    L = np.array([boxes["nx"], boxes["ny"], boxes["nz"]]) * boxes["dx"]
    t = spectra.skewers_cone(9, L, seed=12, npix_range=(40, 90))
    npix = t.npix.copy()
    npix[[1, 4]] = 0
    npix[[2, 7]] = 1
    t = spectra.SkewerTable(t.start, t.direction, npix, dpix=t.dpix)
    cfg = spectra.SpectraConfig(a=0.1, b=1.6, c=0.5)
    g = _run(env, boxes, t, cfg)
    ref = _oracle(boxes, t, dict(kind="const", a=0.1, b=1.6, c=0.5))
    for s in range(t.n):
        assert len(g[0][s]) == npix[s]
    _cmp(g, ref, np.std(boxes["d"]))


def test_longest_skewer_of_the_fft_rule(env, boxes):
    """The largest small-scale FFT (4096 points, skewers up to 4046 pixels under the rule
    256*2^n >= npix + 50) against the oracle with host noise."""
    _lib, _, spectra = env
    L = np.array([boxes["nx"], boxes["ny"], boxes["nz"]]) * boxes["dx"]
    t = spectra.skewers_cone(3, L, seed=13, npix_range=(4046, 4046))
    rs = np.random.RandomState(2)
    noise1d = [rs.normal(size=osk.nz_rule(int(n))).astype(np.float32) for n in t.npix]
    packed = torch.from_numpy(np.concatenate(noise1d)).cuda()
    offs = torch.from_numpy(np.concatenate([[0], np.cumsum([len(x) for x in noise1d])[:-1]]).astype(np.int64)).cuda()
    pm = lambda k: osk.pmiss_analytic(k)  # noqa: E731
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_HOST, ss_nz=0, pmiss=pm, a=0.1, b=1.6, c=0.5)
    g = _run(env, boxes, t, cfg, noise=(packed, offs))
    ref = _oracle(boxes, t, dict(kind="const", a=0.1, b=1.6, c=0.5),
                  small=dict(pixsize=0.2, nz="rule", pmiss=pm), noise1d=[x.astype(np.float64) for x in noise1d])
    _cmp(g, ref, np.std(boxes["d"]))


def test_skewer_tuner_choice_and_block_cap(env, boxes):
    """The skewer autotuner times the paired and one-per-item schedules at several resident-block
    caps and applies its choice; a block cap changes only how many blocks share the work
    (flux identical bit for bit), the schedule only the packing of the small-scale FFTs (flux
    within float32 rounding)."""
    _lib, _, spectra = env
    from saclaymocks_gb300 import tune
    L = np.array([boxes["nx"], boxes["ny"], boxes["nz"]]) * boxes["dx"]
    t = spectra.skewers_cone(60, L, seed=7, npix_range=(100, 600))
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=2048, seed=5, a=0.1, b=1.6, c=0.5)
    out = boxes["out"]
    kw = dict(nx=boxes["nx"], ny=boxes["ny"], nz=boxes["nz"], pitch=out.pitch, dcell=boxes["dx"])
    try:
        _lib.tune_flag(_lib.SMK_TUNE_SKEWER_BLOCKS, 0)
        f0 = spectra.SkewerRunner(t, cfg).run(out.delta_pad[0], out.eta_pad[0], **kw).clone()
        _lib.tune_flag(_lib.SMK_TUNE_SKEWER_BLOCKS, 1)
        f1 = spectra.SkewerRunner(t, cfg).run(out.delta_pad[0], out.eta_pad[0], **kw).clone()
        torch.cuda.synchronize()
        assert torch.equal(f0, f1)
        res = tune.tune_skewers(t, cfg, (out.delta_pad[0], out.eta_pad[0]), reps=1, use_cache=False, **kw)
        ch = res["choice"]
        assert ch["blocks"] in (0, 1, 2, 3) and isinstance(ch["pair"], bool)
        assert len(res["ms"]) == 8 and all(v > 0 for v in res["ms"].values())
        assert _lib.tune_flag(_lib.SMK_TUNE_SKEWER_BLOCKS, ch["blocks"]) == ch["blocks"]
        fc = spectra.SkewerRunner(t, cfg, pair=ch["pair"]).run(out.delta_pad[0], out.eta_pad[0], **kw)
        torch.cuda.synchronize()
        assert float((fc - f0).abs().max()) <= F_ATOL
    finally:
        _lib.tune_flag(_lib.SMK_TUNE_SKEWER_BLOCKS, 0)
