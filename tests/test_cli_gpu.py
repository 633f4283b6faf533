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


def test_spectra_then_merge(ok, tmp_path):
    from saclaymocks_gb300 import fits
    from saclaymocks_gb300.bin import make_boxes, make_spectra, merge_spectra
    bdir, sdir, mdir = tmp_path / "boxes", tmp_path / "spec", tmp_path / "merged"
    make_boxes.main(["-NX", "24", "-NY", "20", "-NZ", "30", "-seed", "4", "-outDir", str(bdir),
                     "--noise", "numpy", "--eta-only-zz"])
    make_spectra.main(["-boxdir", str(bdir), "-outDir", str(sdir), "--synthetic", "12", "-i", "0", "-N", "1"])
    path = merge_spectra.main(["-inDir", str(sdir), "-outDir", str(mdir), "-i", "0", "-aa", "0.1",
                               "-bb", "1.6", "-cc", "0.5", "-seed", "7", "--store-g", "True"])
    hd = {h.name: h.data for h in fits.read_fits(path)}
    sp = {h.name: h.data for h in fits.read_fits(str(sdir / "spectra-0-0.fits.gz"))}
    ids = sp["METADATA"]["THING_ID"]
    order = np.argsort(ids, kind="stable")
    rs = np.random.RandomState(7)
    for row, s in enumerate(order):
        ok_ = sp["LAMBDA"][s] > 0
        dl = sp["DELTA_L"][s][ok_].astype(np.float64)
        et = sp["ETA_PAR"][s][ok_].astype(np.float64)
        z = sp["REDSHIFT"][s][ok_]
        nz = osk.nz_rule(len(dl))
        noise = rs.normal(size=nz).astype(np.float32).astype(np.float64)
        ds = osk.small_scales(noise, len(dl), osk.small_scale_scale(nz, 0.2, osk.pmiss_analytic))
        F = osk.fgpa(dl + ds, et, osk.growth_merge(z), 0.1, 1.6, 0.5)
        got = hd["FLUX"][row][:len(dl)]
        np.testing.assert_allclose(got, F, rtol=0, atol=2e-6)
        np.testing.assert_allclose(hd["DELTA_S"][row][:len(dl)], ds, rtol=0, atol=2e-6)
