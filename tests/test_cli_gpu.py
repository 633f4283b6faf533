"""The drop-in command lines: make_boxes -> make_spectra -> merge_spectra through files in the
reference's formats, checked against the oracle on the same noise."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import grf as ograf       # noqa: E402
from oracle import skewers as osk     # noqa: E402


@pytest.fixture(scope="module")
def ok():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _fixture_files(tmp_path, f):
    """The P-grid file of interpolate_pk (P0, Pln1..3) and a growth-rate table whose first row
    is the golden dD/dz(0), as the reference's make_boxes reads them."""
    from saclaymocks_gb300 import fits
    pkdir = tmp_path / "pk"
    pkdir.mkdir()
    n = int(f["NX"])
    w = fits.FitsWriter(str(pkdir / f"P{n}.fits")).image(f["P0"])
    for i in (1, 2, 3):
        w.image(f[f"Pln{i}"], extname=f"Pln{i}")
    w.image(f["P0"], extname="P0").close()
    dg = tmp_path / "dgrowth.fits"
    fits.FitsWriter(str(dg)).table({"dD/dz": np.array([float(f["dgrowth0"]), 0.0])}).close()
    return pkdir, dg


def test_make_boxes_files_match_reference_golden(ok, tmp_path, golden):
    """Every file the reference's make_boxes writes: box, boxln_1..3, eta_ij, vx/vy/vz."""
    from saclaymocks_gb300 import fits
    from saclaymocks_gb300.bin import make_boxes
    f = golden("grf_cube16.npz")
    pkdir, dg = _fixture_files(tmp_path, f)
    out = tmp_path / "out"
    make_boxes.main(["-NX", "16", "-pixel", "2.19", "-seed", "0", "-outDir", str(out), "--noise", "numpy",
                     "-PkDir", str(pkdir), "-dgrowthfile", str(dg)])

    def stack(prefix, nfiles):
        return np.concatenate([fits.read(str(out / f"{prefix}-{i}.fits")) for i in range(nfiles)])
    box = stack("box", 16)
    assert box.shape == (16, 16, 16)
    d = box - f["delta"]
    assert np.sqrt((d ** 2).mean() / (f["delta"] ** 2).mean()) < 1e-6
    for name, nfiles in [("eta_xx", 16), ("eta_yy", 16), ("eta_zz", 16), ("eta_xy", 16), ("eta_xz", 16),
                         ("eta_yz", 16), ("boxln_1", 1), ("boxln_2", 1), ("boxln_3", 1), ("vx", 1), ("vy", 1),
                         ("vz", 1)]:
        got = stack(name, nfiles)
        ref = f[name]
        assert got.shape == ref.shape, name
        assert np.abs(got - ref).max() < 1e-5 * ref.std(), name
    h = fits.read_header(str(out / "box-0.fits"))
    assert h["NX"] == 16 and h["DX"] == pytest.approx(2.19)
    assert h["SIGMA"] == pytest.approx(float(f["sigma"]), rel=1e-5) and h["SEED"] == 0


def test_make_boxes_checkpoint_and_resume(ok, tmp_path):
    """seed_boxk.npy / boxk.npy checkpoint: a rerun in the same directory takes the saved seed
    (not -seed) and skips the families whose files all exist, regenerating a removed family
    bit for bit; a directory holding only boxk.npy gives the same boxes from the saved modes."""
    from saclaymocks_gb300 import fits
    from saclaymocks_gb300.bin import make_boxes
    out = tmp_path / "out"
    args = ["-NX", "12", "-NY", "10", "-NZ", "16", "-seed", "5", "-outDir", str(out), "-rsd", "True",
            "--eta-only-zz", "--write-boxk", "True"]
    make_boxes.main(args)
    box = np.concatenate([fits.read(str(out / f"box-{i}.fits")) for i in range(12)])
    eta = np.concatenate([fits.read(str(out / f"eta_zz-{i}.fits")) for i in range(12)])
    assert int(np.load(out / "seed_boxk.npy")) == 5
    boxk = np.load(out / "boxk.npy")
    assert boxk.shape == (12, 10, 9) and boxk.dtype == np.complex64
    os.remove(out / "eta_zz-3.fits")
    make_boxes.main(args[:7] + ["99"] + args[8:])               # another -seed: the saved one wins
    eta2 = np.concatenate([fits.read(str(out / f"eta_zz-{i}.fits")) for i in range(12)])
    np.testing.assert_array_equal(eta2, eta)
    # only boxk.npy: noise = irfftn(boxk), the same boxes to float32 rounding of the round trip
    other = tmp_path / "other"
    other.mkdir()
    np.save(other / "boxk.npy", boxk)
    make_boxes.main(["-NX", "12", "-NY", "10", "-NZ", "16", "-outDir", str(other), "-rsd", "True", "--eta-only-zz"])
    box3 = np.concatenate([fits.read(str(other / f"box-{i}.fits")) for i in range(12)])
    assert np.abs(box3 - box).max() < 1e-5 * box.std()


ETA6 = ("xx", "yy", "zz", "xy", "xz", "yz")


def _write_qso_inputs(tmp_path, g):
    """The boxes and QSO catalogue of spectra_qso.npz as files (box-{x}.fits, eta_ij-{x}.fits,
    QSO-0-1.fits), as the reference's make_spectra read them."""
    from saclaymocks_gb300 import fits
    bdir = tmp_path / "boxes"
    bdir.mkdir()
    NX, NY, NZ = g["box_delta"].shape
    dx = float(g["dx"])
    hdr = {"DX": dx, "DY": dx, "DZ": dx, "NX": NX, "NY": NY, "NZ": NZ}
    for nm in ["delta"] + ["eta_" + c for c in ETA6]:
        prefix = "box" if nm == "delta" else nm
        for i in range(NX):
            fits.write_image(str(bdir / f"{prefix}-{i}.fits"), g["box_" + nm][i:i + 1], hdr)
    n = len(g["cat_RA"])
    cat = {k: g["cat_" + k] for k in ("RA", "DEC", "Z_QSO_NO_RSD", "Z_QSO_RSD", "THING_ID", "HDU", "PLATE",
                                       "MJD", "FIBERID")}
    cat["PMF"] = np.array([f"7-55000-{i}" for i in range(n)])
    qdir = tmp_path / "qso"
    qdir.mkdir()
    fits.FitsWriter(str(qdir / "QSO-0-1.fits")).table(cat, {"RA0": 180.0, "DEC0": 0.0}).close()
    return bdir, str(qdir / "QSO-")


def test_make_spectra_matches_reference_golden(ok, tmp_path, golden):
    """The make_spectra drop-in on a QSO catalogue writes what the reference's make_spectra
    main() wrote: files per HDU, METADATA rows and header, LAMBDA and REDSHIFT (bit for bit),
    DELTA_L and ETA_PAR of the Gaussian 7^3 read (FP32 kernel: 5e-6 sigma), -1e6 / 0 beyond
    the forest and the -1 / -2e6 padding."""
    from saclaymocks_gb300 import fits
    from saclaymocks_gb300.bin import make_spectra
    g = golden("spectra_qso.npz")
    bdir, qso = _write_qso_inputs(tmp_path, g)
    sdir = tmp_path / "spec"
    make_spectra.main(["-QSOfile", qso, "-boxdir", str(bdir), "-outDir", str(sdir), "-i", "0", "-N", "1",
                       "-zmin", repr(float(g["zmin"])), "-zmax", repr(float(g["zmax"])), "-pixel", "0.2",
                       "-dmax", "3", "-rsd", "True"])
    sig_d, sig_e = float(g["box_delta"].std()), float(g["box_eta_zz"].std())
    for hdu in (0, 1):
        hd = {h.name: h for h in fits.read_fits(str(sdir / f"spectra-0-{hdu}.fits.gz"))}
        meta = hd["METADATA"]
        np.testing.assert_array_equal(meta.data["THING_ID"], g[f"h{hdu}_THING_ID"])
        np.testing.assert_array_equal(meta.data["Z"], g[f"h{hdu}_Z"])
        np.testing.assert_array_equal(meta.data["RA"], g[f"h{hdu}_RA"])
        h = meta.header
        np.testing.assert_allclose([h["Z0"], h["PIXEL"], h["NPIXEL"], h["NX"], h["DMAX"], h["RA0"], h["DEC0"]],
                                   g[f"h{hdu}_header"], rtol=1e-12)
        np.testing.assert_array_equal(hd["LAMBDA"].data, g[f"h{hdu}_LAMBDA"])
        np.testing.assert_array_equal(hd["REDSHIFT"].data, g[f"h{hdu}_REDSHIFT"])
        for name, sig in (("DELTA_L", sig_d), ("ETA_PAR", sig_e)):
            got, ref = hd[name].data, g[f"h{hdu}_{name}"]
            assert got.shape == ref.shape
            inner = np.abs(ref) < 1e5
            np.testing.assert_array_equal(got[~inner], ref[~inner])
            np.testing.assert_allclose(got[inner], ref[inner], rtol=0, atol=5e-6 * sig, err_msg=name)


def _write_merge_inputs(tmp_path, f, ids):
    """The spectra file and P1D_miss inputs make_golden served to merge_spectra main()."""
    from saclaymocks_gb300 import fits
    n, npix = f["delta_l_in"].shape
    sdir = tmp_path / "spec"
    sdir.mkdir()
    meta = {"RA": np.linspace(10, 11, n).astype(np.float32), "DEC": np.linspace(-1, 1, n).astype(np.float32),
            "Z_noRSD": (f["zq"] - 0.001).astype(np.float32), "Z": f["zq"].astype(np.float32),
            "HDU": np.zeros(n, np.int64), "THING_ID": ids, "PLATE": np.zeros(n, np.int64),
            "MJD": np.zeros(n, np.int32), "FIBERID": np.zeros(n, np.int32), "PMF": np.array(["0"] * n)}
    hdr = {"z0": 1.70975268202, "pixel": 0.2, "NX": 1, "dmax": 3, "ra0": 0.0, "dec0": 0.0, "Npixel": npix}
    w = fits.FitsWriter(str(sdir / "spectra-0-0.fits.gz"))
    w.table(meta, hdr, extname="METADATA")
    w.image(np.tile(f["wav"], (n, 1)), extname="LAMBDA")
    w.image(f["delta_l_in"], extname="DELTA_L")
    w.image(f["eta_par_in"], extname="ETA_PAR")
    w.image(np.zeros((n, npix), np.float32), extname="VELO_PAR")
    w.image(np.tile(f["redshift"], (n, 1)), extname="REDSHIFT")
    w.close()
    return sdir


GOLDEN_IDS = np.array([901, 17, 5003, 42, 77, 313], np.int64)   # THING_ID of the served spectra


@pytest.mark.parametrize("tag", ["table", "fitp1d"])
def test_merge_spectra_matches_reference_golden(ok, tmp_path, golden, tag):
    """The merge_spectra drop-in, run with the flags make_golden gave the reference's main(),
    reproduces its FLUX and DELTA_S: the default branch (nearest-z P1D_miss table, clip,
    sigma_s rescale) and the --fit-p1d spline branch.  -nside 1 puts the six quasars in one
    healpix pixel, as the golden's stand-in for healpy did."""
    from saclaymocks_gb300 import fits
    from saclaymocks_gb300.bin import merge_spectra
    f = golden(f"merge_{tag}.npz")
    np.testing.assert_array_equal(np.argsort(GOLDEN_IDS), f["order"])
    sdir = _write_merge_inputs(tmp_path, f, GOLDEN_IDS)
    pdir = tmp_path / "p1d"
    pdir.mkdir()
    if tag == "table":
        p1d = str(pdir / "pkmiss_test.fits")
        (fits.FitsWriter(p1d).image(f["pm_z"], extname="z").image(f["pm_k"], extname="k")
         .image(f["pm_pk"], extname="pk").image(f["pm_sigma"], extname="sigma").close())
        extra = ["--fit-p1d", "False"]
    else:
        p1d = str(pdir / "p1dmiss_test.fits")
        kt = np.linspace(0.0, float(f["pm_kmax"]), int(f["pm_n"]))
        pt = float(f["pm_amp"]) * np.exp(-(kt / float(f["pm_kscale"])) ** 2) + float(f["pm_floor"])
        fits.FitsWriter(p1d).table({"k": kt, "P1DmissRSD": pt}).close()
        extra = ["--fit-p1d", "True"]
    mdir = tmp_path / "merged"
    paths = merge_spectra.main(["-inDir", str(sdir), "-outDir", str(mdir), "-i", "0", "-aa", "0.1", "-bb", "1.6",
                                "-cc", "0.5", "-pixsize", "0.2", "-nside", "1", "-rsd", "True", "-addnoise", "True",
                                "-dla", "True", "--check-id", "False", "-seed", str(int(f["seed"])),
                                "--store-g", "True", "-p1dfile", p1d] + extra)
    assert len(paths) == 1
    hd = {h.name: h.data for h in fits.read_fits(paths[0])}
    np.testing.assert_array_equal(hd["METADATA"]["THING_ID"], np.sort(GOLDEN_IDS))
    np.testing.assert_allclose(hd["DELTA_S"], f["delta_s"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(hd["FLUX"], f["flux"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(hd["GROWTHF"], f["growthf"], rtol=1e-6)
    np.testing.assert_array_equal(hd["LAMBDA"], f["wav"])


def test_boxes_spectra_merge_chain(ok, tmp_path, golden):
    """make_boxes -> make_spectra (QSO catalogue, Gaussian read of the six eta_ij boxes) ->
    merge_spectra (default branch) through files: every merged spectrum equals the oracle's
    merge loop on the spectra file make_spectra wrote."""
    from saclaymocks_gb300 import fits
    from saclaymocks_gb300.bin import make_boxes, make_spectra, merge_spectra
    g = golden("spectra_qso.npz")
    _, qso = _write_qso_inputs(tmp_path, g)
    bdir, sdir, mdir = tmp_path / "gb", tmp_path / "spec", tmp_path / "merged"
    dg = tmp_path / "dgrowth.fits"
    fits.FitsWriter(str(dg)).table({"dD/dz": np.array([-0.52, -0.5])}).close()
    make_boxes.main(["-NX", "12", "-NY", "12", "-NZ", "40", "-pixel", "12", "-seed", "4", "-outDir", str(bdir),
                     "-dgrowthfile", str(dg)])
    make_spectra.main(["-QSOfile", qso, "-boxdir", str(bdir), "-outDir", str(sdir), "-i", "0", "-N", "1",
                       "-zmin", repr(float(g["zmin"])), "-zmax", repr(float(g["zmax"]))])
    ptab = dict(z=np.array([1.8, 1.9, 2.0]), k=np.linspace(0, 20, 2001), sigma=np.array([0.3, 0.27, 0.25]))
    ptab["pk"] = np.stack([a * 0.05 * np.exp(-(ptab["k"] / 2) ** 2) for a in (1.2, 1.0, 0.8)])
    p1d = str(tmp_path / "pk.fits")
    (fits.FitsWriter(p1d).image(ptab["z"], extname="z").image(ptab["k"], extname="k")
     .image(ptab["pk"], extname="pk").image(ptab["sigma"], extname="sigma").close())
    # merge_spectra -i k takes the files whose last number is k: the spectra of QSO-file HDU k
    for hdu in (0, 1):
        paths = merge_spectra.main(["-inDir", str(sdir), "-outDir", str(mdir), "-i", str(hdu), "-aa", "0.1",
                                    "-bb", "1.6", "-cc", "0.5", "-seed", "7", "--store-g", "True", "-p1dfile", p1d,
                                    "-nside", "1"])
        hd = {h.name: h.data for h in fits.read_fits(str(sdir / f"spectra-0-{hdu}.fits.gz"))}
        spec = []
        for r in range(len(hd["METADATA"])):
            ok_ = hd["LAMBDA"][r] > 0
            spec.append(dict(tid=int(hd["METADATA"]["THING_ID"][r]), wav=hd["LAMBDA"][r][ok_],
                             delta_l=hd["DELTA_L"][r][ok_], eta_par=hd["ETA_PAR"][r][ok_],
                             z=hd["REDSHIFT"][r][ok_], zq=float(hd["METADATA"]["Z"][r])))
        spec.sort(key=lambda d: d["tid"])
        fo, dso = osk.merge_spectra_loop(spec, np.random.RandomState(7 + hdu), ptab=ptab, abc=(0.1, 1.6, 0.5))
        md = {h.name: h.data for h in fits.read_fits(paths[0])}
        np.testing.assert_array_equal(md["METADATA"]["THING_ID"], [d["tid"] for d in spec])
        np.testing.assert_allclose(md["FLUX"], np.array(fo), rtol=0, atol=2e-6)
        np.testing.assert_allclose(md["DELTA_S"], np.array(dso), rtol=0, atol=2e-6)
