"""Lines of sight from a QSO catalogue (saclaymocks_gb300.los) against the reference's own
make_spectra main() (tests/golden/spectra_qso.npz): the pixel grid, wavelengths, redshifts,
which quasars are kept and in what order, and, through the oracle's Gaussian read at the
positions los.py builds, DELTA_L and ETA_PAR.  CPU only."""
import numpy as np
import pytest

from oracle import skewers as osk
from saclaymocks_gb300 import los


@pytest.fixture(scope="module")
def g(golden):
    return golden("spectra_qso.npz")


def _lines(g):
    dx = float(g["dx"])
    NX, NY, NZ = g["box_delta"].shape
    cat = np.zeros(len(g["cat_RA"]), dtype=[("RA", "f8"), ("DEC", "f8"), ("Z_QSO_RSD", "f4"),
                                            ("Z_QSO_NO_RSD", "f4")])
    cat["RA"], cat["DEC"] = g["cat_RA"], g["cat_DEC"]
    cat["Z_QSO_RSD"], cat["Z_QSO_NO_RSD"] = g["cat_Z_QSO_RSD"], g["cat_Z_QSO_NO_RSD"]
    cosmo = los.Cosmo()
    grid = los.pixel_grid(cosmo, float(g["zmin"]), float(g["zmax"]), 0.2)
    L = los.qso_lines(cosmo, grid, cat, 180.0, 0.0, (dx * NX, dx * NY, dx * NZ), dx, NX, 0, 1,
                      float(g["zmin"]), float(g["zmax"]))
    return cosmo, grid, L, dx, (NX, NY, NZ)


def test_pixel_grid_and_kept_quasars(g):
    cosmo, grid, L, _, _ = _lines(g)
    ids = np.concatenate([g["h0_THING_ID"], g["h1_THING_ID"]])
    kept = np.asarray(g["cat_THING_ID"])[L.qso_index]
    assert sorted(kept.tolist()) == sorted(ids.tolist())
    assert int(g["h0_header"][2]) == len(grid.R)                    # Npixel
    for h in (0, 1):
        for r, tid in enumerate(g[f"h{h}_THING_ID"]):
            q = int(np.nonzero(kept == tid)[0][0])
            sl = slice(L.r0[q], L.r0[q] + L.npix[q])
            lam = g[f"h{h}_LAMBDA"][r]
            n = int((lam > 0).sum())
            assert n == L.npix[q]
            np.testing.assert_array_equal(grid.lam[sl].astype(np.float32), lam[:n])
            np.testing.assert_array_equal(cosmo.r_2_z(grid.R[sl] / los.H).astype(np.float32),
                                          g[f"h{h}_REDSHIFT"][r][:n])
            # beyond the forest ReadSpec leaves -1e6
            dl = g[f"h{h}_DELTA_L"][r][:n]
            assert np.all(dl[L.imax[q]:] == -1e6) and np.all(dl[L.imin[q]:L.imax[q]] > -1e5)


def test_gaussian_read_at_los_positions(g):
    cosmo, grid, L, dx, (NX, NY, NZ) = _lines(g)
    kept = np.asarray(g["cat_THING_ID"])[L.qso_index]
    boxes = [g["box_delta"]] + [g["box_eta_" + c] for c in ("xx", "yy", "zz", "xy", "xz", "yz")]
    corner = np.array([dx * NX / 2, dx * NY / 2, dx * NZ / 2 - grid.R0])
    for h in (0, 1):
        for r, tid in enumerate(g[f"h{h}_THING_ID"]):
            q = int(np.nonzero(kept == tid)[0][0])
            a, b = int(L.r0[q] + L.imin[q]), int(L.r0[q] + L.imax[q])
            obsf = grid.R[a:b, None] * L.unit[q][None, :]           # observer frame X, Y, Z
            vals = osk.gauss343(boxes, obsf + corner[None, :], dx)
            np.testing.assert_allclose(vals[0], g[f"h{h}_DELTA_L"][r][L.imin[q]:L.imax[q]], rtol=0, atol=2e-7)
            eta = osk.eta_par_projection(dict(zip(("xx", "yy", "zz", "xy", "xz", "yz"), vals[1:])), obsf)
            np.testing.assert_allclose(eta, g[f"h{h}_ETA_PAR"][r][L.imin[q]:L.imax[q]], rtol=0, atol=2e-7)
