"""merge_spectra's small-scale step on the GPU (SMK_INTERP_PIXELS) against the reference's own
output and the oracle: the default branch (per-skewer z_eff over the Lya-forest pixels,
nearest-redshift P1D_miss table, clip, sigma_s(z)/sigma_s(z_eff) rescale) and the forest rule
(no forest pixel: no draw, no delta_s), bin/merge_spectra.py:116-118, 303-331.

Tolerances (FP32 kernel vs FP64 reference/oracle): |dF| <= 2e-6, |d delta_s| <= 2e-6.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import skewers as osk        # noqa: E402

F_ATOL = 2e-6
DS_ATOL = 2e-6


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from saclaymocks_gb300 import _lib, spectra
    return _lib, spectra


def _gpu_merge(env, spectra_list, *, ptab=None, pmiss=None, mode="host", seed=0, abc=(0.1, 1.6, 0.5)):
    """spectra_list in the loop's order; host mode draws RandomState(seed).normal(nz) for the
    spectra with forest pixels, in that order, as merge_spectra does."""
    _lib, spectra = env
    wav = [np.asarray(s["wav"]) for s in spectra_list]
    npix = np.array([len(w) for w in wav], np.int32)
    forest = spectra.forest_ranges(wav, [s["zq"] for s in spectra_list])
    n = len(npix)
    table = spectra.SkewerTable(np.zeros((n, 3)), np.tile([0, 0, 1.0], (n, 1)), npix, forest=forest)
    cat = lambda k: torch.from_numpy(np.concatenate([np.asarray(s[k], np.float32) for s in spectra_list])).cuda()  # noqa: E731
    pm = spectra.P1DMissTable(ptab["z"], ptab["k"], ptab["pk"], ptab.get("sigma")) if ptab is not None else pmiss
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_HOST if mode == "host" else _lib.SMK_SS_PHILOX,
                                ss_nz=0, pmiss=pm, seed=seed, growth=_lib.SMK_G_MERGE,
                                a=abc[0], b=abc[1], c=abc[2])
    noise = None
    if mode == "host":
        rs = np.random.RandomState(seed)
        draws, offs, o = [], np.zeros(n, np.int64), 0
        for s in range(n):
            offs[s] = o
            if forest[s, 1] > forest[s, 0]:
                d = rs.normal(size=spectra.nz_rule(int(npix[s])))
                draws.append(d)
                o += len(d)
        buf = np.concatenate(draws) if draws else np.zeros(1)
        noise = (torch.from_numpy(buf.astype(np.float32)).cuda(), torch.from_numpy(offs).cuda())
    r = spectra.SkewerRunner(table, cfg, pixels=(cat("delta_l"), cat("eta_par"), cat("z")))
    F, dtot, _, _ = r.run(noise=noise, want_fields=True)
    torch.cuda.synchronize()
    F = spectra.split(F, table)
    ds = [d - np.asarray(s["delta_l"], np.float32) for d, s in zip(spectra.split(dtot, table), spectra_list)]
    return F, ds


def test_default_branch_matches_merge_spectra_golden(env, golden):
    """FLUX and DELTA_S of the reference's merge_spectra main() (default branch) are reproduced."""
    f = golden("merge_table.npz")
    sl = [dict(wav=f["wav"], delta_l=f["delta_l_in"][s], eta_par=f["eta_par_in"][s], z=f["redshift"],
               zq=float(f["zq"][s])) for s in f["order"]]
    ptab = dict(z=f["pm_z"], k=f["pm_k"], pk=f["pm_pk"], sigma=f["pm_sigma"])
    F, ds = _gpu_merge(env, sl, ptab=ptab, seed=int(f["seed"]))
    np.testing.assert_allclose(np.array(ds), f["delta_s"], rtol=0, atol=DS_ATOL)
    np.testing.assert_allclose(np.array(F), f["flux"], rtol=0, atol=F_ATOL)


def _synthetic(seed=5, n=48):
    """Ragged spectra on different wavelength windows, quasars placed so that some spectra are
    all forest, some partly and some not at all; pairs of equal FFT length with different z_eff."""
    rs = np.random.RandomState(seed)
    out = []
    for s in range(n):
        npx = int(rs.choice([150, 199, 206, 300, 460, 461, 700, 973]))
        w0 = rs.uniform(3500.0, 5200.0)
        wav = (w0 + 0.8 * np.arange(npx)).astype(np.float32)
        z = (wav / 1215.67 - 1).astype(np.float32)
        kind = s % 4
        if kind == 0:
            zq = float(z[-1]) + 0.3          # all forest
        elif kind == 1:
            zq = float(z[npx // 3])          # forest = the first third
        elif kind == 2:
            zq = float(z[0]) - 0.05          # no forest pixel
        else:
            zq = float(z[rs.randint(1, npx - 1)])
        out.append(dict(wav=wav, delta_l=rs.normal(0, 0.8, npx).astype(np.float32),
                        eta_par=rs.normal(0, 0.3, npx).astype(np.float32), z=z, zq=zq))
    return out


PTAB = dict(z=np.array([1.8, 2.2, 2.6, 3.0, 3.6]), k=np.linspace(0.0, 20.0, 2001),
            sigma=np.array([0.31, 0.28, 0.26, 0.24, 0.20]))
PTAB["pk"] = np.stack([a * 0.05 * np.exp(-(PTAB["k"] / 2.0) ** 2) - 2e-4 for a in (1.4, 1.2, 1.0, 0.9, 0.7)])


def test_default_branch_matches_oracle_on_ragged_spectra(env):
    """Ragged lengths, partial and empty forests, five redshift tables (negative P1D_miss tails
    clipped), sigma rescale, a(z)/c(z) as constants: GPU (host noise in the loop's draw order)
    against the oracle restatement of the loop."""
    sl = _synthetic()
    F, ds = _gpu_merge(env, sl, ptab=PTAB, seed=11)
    fo, dso = osk.merge_spectra_loop(sl, np.random.RandomState(11), ptab=PTAB, abc=(0.1, 1.6, 0.5))
    for s in range(len(sl)):
        np.testing.assert_allclose(ds[s], dso[s], rtol=0, atol=DS_ATOL, err_msg=f"delta_s {s}")
        np.testing.assert_allclose(F[s], fo[s], rtol=0, atol=F_ATOL, err_msg=f"flux {s}")
    empty = [s for s in range(len(sl)) if s % 4 == 2]
    assert all(np.all(ds[s] == 0) for s in empty)


def test_fit_branch_forest_rule_matches_oracle(env):
    """--fit-p1d branch (one P1D_miss function, no rescale) with the same forest rule."""
    sl = _synthetic(seed=8, n=24)

    def pm(k):
        return 0.05 * np.exp(-(np.asarray(k) / 2.0) ** 2) + 1e-4
    F, ds = _gpu_merge(env, sl, pmiss=pm, seed=3)
    fo, dso = osk.merge_spectra_loop(sl, np.random.RandomState(3), pmiss_fit=pm, abc=(0.1, 1.6, 0.5))
    for s in range(len(sl)):
        np.testing.assert_allclose(ds[s], dso[s], rtol=0, atol=DS_ATOL, err_msg=f"delta_s {s}")
        np.testing.assert_allclose(F[s], fo[s], rtol=0, atol=F_ATOL, err_msg=f"flux {s}")


def test_philox_mode_table_choice_and_sigma_rescale(env):
    """GPU-drawn small scales: a spectrum with no forest pixel gets none; with sigma the field
    is the unscaled one times sigma(z)/sigma(z_eff) pixel by pixel; the table set of each
    spectrum is the one nearest its z_eff (same field as a run given only that table)."""
    sl = _synthetic(seed=21, n=32)
    F1, ds1 = _gpu_merge(env, sl, ptab=PTAB, mode="philox", seed=99)
    nos = dict(PTAB)
    nos["sigma"] = None
    F0, ds0 = _gpu_merge(env, sl, ptab=nos, mode="philox", seed=99)
    for s, sp in enumerate(sl):
        fr = osk.merge_forest(sp)
        if len(fr) == 0:
            assert np.all(ds1[s] == 0) and np.all(ds0[s] == 0)
            continue
        zeff = np.asarray(sp["z"], np.float64)[fr].mean()
        ratio = np.interp(sp["z"], PTAB["z"], PTAB["sigma"]) / np.interp(zeff, PTAB["z"], PTAB["sigma"])
        np.testing.assert_allclose(ds1[s], ds0[s] * ratio, rtol=0, atol=2e-6 * max(1.0, np.abs(ds0[s]).max()))
    # table choice: with only table j given, every spectrum whose z_eff is nearest to z_j gets
    # the same field (the draw depends on the seed and the skewer index only)
    nearest = []
    for sp in sl:
        fr = osk.merge_forest(sp)
        nearest.append(int(np.argsort(np.abs(PTAB["z"] - np.asarray(sp["z"], np.float64)[fr].mean()))[0])
                       if len(fr) else -1)
    for j in range(len(PTAB["z"])):
        one = dict(z=PTAB["z"][j:j + 1], k=PTAB["k"], pk=PTAB["pk"][j:j + 1], sigma=None)
        _, dsj = _gpu_merge(env, sl, ptab=one, mode="philox", seed=99)
        for s in range(len(sl)):
            if nearest[s] == j:
                np.testing.assert_allclose(dsj[s], ds0[s], rtol=0, atol=2e-6, err_msg=f"spectrum {s}, table {j}")
