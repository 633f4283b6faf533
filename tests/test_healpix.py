"""HEALPix pixel indices of merge_spectra's healpix grouping (saclaymocks_gb300.healpix): every
pixel centre maps back to its pixel in both schemes, the nested and ring numberings are
permutations of each other, pixels are equal-area, and the poles and first ring sit where the
HEALPix scheme puts them.  CPU only."""
import numpy as np
import pytest

from saclaymocks_gb300 import healpix as hp


@pytest.mark.parametrize("nside", [1, 2, 4, 16, 64])
@pytest.mark.parametrize("nest", [False, True])
def test_pixel_centres_round_trip(nside, nest):
    p = np.arange(12 * nside * nside)
    th, ph = hp.pix2ang(nside, p, nest=nest)
    np.testing.assert_array_equal(hp.ang2pix(nside, th, ph, nest=nest), p)


@pytest.mark.parametrize("nside", [1, 8, 32])
def test_nested_and_ring_are_permutations(nside):
    p = np.arange(12 * nside * nside)
    th, ph = hp.pix2ang(nside, p, nest=True)
    r = hp.ang2pix(nside, th, ph, nest=False)
    assert len(np.unique(r)) == len(p)
    np.testing.assert_allclose(np.array(hp.pix2ang(nside, r, nest=False)), np.array([th, ph]), atol=1e-12)


def test_equal_area():
    rs = np.random.RandomState(0)
    n = 1_200_000
    th = np.arccos(rs.uniform(-1, 1, n))
    ph = rs.uniform(0, 2 * np.pi, n)
    for nest in (False, True):
        c = np.bincount(hp.ang2pix(4, th, ph, nest=nest), minlength=192)
        assert np.all(np.abs(c - n / 192) < 5 * np.sqrt(n / 192))


def test_known_pixels():
    ns = 16
    # north pole: ring pixel 0, nested pixel nside^2 - 1 (top corner of base face 0)
    assert hp.ang2pix(ns, 0.0, 0.0, nest=False) == 0
    assert hp.ang2pix(ns, 0.0, 0.0, nest=True) == ns * ns - 1
    # south pole: last ring's first pixel / bottom corner of face 8
    assert hp.ang2pix(ns, np.pi, 0.0, nest=False) == 12 * ns * ns - 4
    assert hp.ang2pix(ns, np.pi, 0.0, nest=True) == 8 * ns * ns
    # radec2pix is ang2pix at theta = pi/2 - dec, phi = ra (degrees in)
    assert hp.radec2pix(ns, 45.0, 30.0) == hp.ang2pix(ns, np.pi / 2 - np.radians(30.0), np.radians(45.0))
