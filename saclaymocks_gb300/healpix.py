"""HEALPix pixel indices (ring and nested schemes) of sky positions, host side.

merge_spectra groups the spectra of a slice by the healpix pixel of their quasar
(util.radec2pix, py/SaclayMocks/util.py:101-105, which calls healpy.ang2pix); the pixel decides
the output file name and the order in which the small-scale noise is drawn.  healpy is not a
dependency here, so this module restates the published HEALPix scheme (Gorski et al. 2005,
ApJ 622, 759): 12 nside^2 equal-area pixels, an equatorial belt |z| <= 2/3 and two polar caps,
pixels indexed along iso-latitude rings (RING) or along the hierarchical quadtree of the twelve
base faces (NESTED).
"""
from __future__ import annotations

import numpy as np

_TWO_THIRDS = 2.0 / 3.0


def _spread_bits(v: np.ndarray) -> np.ndarray:
    """Interleave zeros between the bits of v (bit i -> bit 2i), v < 2^30."""
    v = v.astype(np.int64)
    out = np.zeros_like(v)
    for i in range(30):
        out |= ((v >> i) & 1) << (2 * i)
    return out


def _compress_bits(v: np.ndarray) -> np.ndarray:
    """Inverse of _spread_bits on the even bits."""
    v = v.astype(np.int64)
    out = np.zeros_like(v)
    for i in range(30):
        out |= ((v >> (2 * i)) & 1) << i
    return out


def ang2pix(nside: int, theta, phi, nest: bool = True) -> np.ndarray:
    """Pixel of colatitude theta and longitude phi (radians)."""
    ns = int(nside)
    if ns < 1 or (nest and ns & (ns - 1)):
        raise ValueError("nside must be >= 1 (a power of two for the nested scheme)")
    z = np.cos(np.asarray(theta, np.float64))
    za = np.abs(z)
    tt = np.mod(np.asarray(phi, np.float64), 2 * np.pi) / (np.pi / 2)      # in [0, 4)
    z, za, tt = np.broadcast_arrays(z, za, tt)
    pix = np.zeros(z.shape, np.int64)
    eq = za <= _TWO_THIRDS
    # equatorial belt: indices of the ascending and descending edge lines through the point
    t1 = ns * (0.5 + tt[eq])
    t2 = ns * z[eq] * 0.75
    jp = (t1 - t2).astype(np.int64)
    jm = (t1 + t2).astype(np.int64)
    # polar caps
    cap = ~eq
    tp = tt[cap] - np.floor(tt[cap])
    tmp = ns * np.sqrt(3.0 * (1.0 - za[cap]))
    kp = (tp * tmp).astype(np.int64)
    km = ((1.0 - tp) * tmp).astype(np.int64)
    if not nest:
        ir = ns + 1 + jp - jm                        # ring counted from z = 2/3, 1..2 nside + 1
        kshift = 1 - (ir & 1)
        ip = np.mod((jp + jm - ns + kshift + 1) // 2, 4 * ns)
        pix[eq] = 2 * ns * (ns - 1) + (ir - 1) * 4 * ns + ip
        irc = kp + km + 1                            # ring counted from the nearer pole
        ipc = np.mod((tt[cap] * irc).astype(np.int64), 4 * irc)
        north = z[cap] > 0
        pix[cap] = np.where(north, 2 * irc * (irc - 1) + ipc, 12 * ns * ns - 2 * irc * (irc + 1) + ipc)
        return pix
    # nested: base face and (x, y) inside it
    face = np.zeros(z.shape, np.int64)
    ix = np.zeros(z.shape, np.int64)
    iy = np.zeros(z.shape, np.int64)
    ifp, ifm = jp // ns, jm // ns
    face[eq] = np.where(ifp == ifm, ifp | 4, np.where(ifp < ifm, ifp, ifm + 8))
    ix[eq] = jm & (ns - 1)
    iy[eq] = ns - (jp & (ns - 1)) - 1
    ntt = np.minimum(tt[cap].astype(np.int64), 3)
    tp = tt[cap] - ntt
    kp = np.minimum((tp * tmp).astype(np.int64), ns - 1)
    km = np.minimum(((1.0 - tp) * tmp).astype(np.int64), ns - 1)
    north = z[cap] >= 0
    face[cap] = np.where(north, ntt, ntt + 8)
    ix[cap] = np.where(north, ns - km - 1, kp)
    iy[cap] = np.where(north, ns - kp - 1, km)
    return face * ns * ns + _spread_bits(ix) + (_spread_bits(iy) << 1)


# ring index of the lowest corner of each base face, and its longitude offset (units of pi/4)
_JRLL = np.array([2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4])
_JPLL = np.array([1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7])


def pix2ang(nside: int, pix, nest: bool = True):
    """Colatitude and longitude (radians) of pixel centres."""
    ns = int(nside)
    p = np.asarray(pix, np.int64)
    npix = 12 * ns * ns
    if nest:
        face = p // (ns * ns)
        ipf = p - face * ns * ns
        ix, iy = _compress_bits(ipf), _compress_bits(ipf >> 1)
        jr = _JRLL[face] * ns - ix - iy - 1          # ring index counted from the north pole
        nr = np.where(jr < ns, jr, np.where(jr > 3 * ns, 4 * ns - jr, ns))
        z = np.where(jr < ns, 1.0 - nr * nr / (3.0 * ns * ns),
                     np.where(jr > 3 * ns, nr * nr / (3.0 * ns * ns) - 1.0, (2 * ns - jr) * 2.0 / (3.0 * ns)))
        kshift = np.where((jr < ns) | (jr > 3 * ns), 0, (jr - ns) & 1)
        jp = (_JPLL[face] * nr + ix - iy + 1 + kshift) // 2
        jp = np.where(jp > 4 * nr, jp - 4 * nr, np.where(jp < 1, jp + 4 * nr, jp))
        phi = (jp - (kshift + 1) * 0.5) * (np.pi / 2 / nr)
        return np.arccos(np.clip(z, -1, 1)), phi
    ncap = 2 * ns * (ns - 1)
    theta = np.zeros(p.shape)
    phi = np.zeros(p.shape)
    north = p < ncap
    south = p >= npix - ncap
    belt = ~north & ~south
    # north cap
    q = p[north]
    ir = (1 + np.floor(np.sqrt(1 + 2 * q))).astype(np.int64) // 2
    ip = q + 1 - 2 * ir * (ir - 1)
    theta[north] = np.arccos(1.0 - ir * ir / (3.0 * ns * ns))
    phi[north] = (ip - 0.5) * (np.pi / 2 / ir)
    # belt
    q = p[belt] - ncap
    ir = q // (4 * ns) + ns
    ip = q % (4 * ns) + 1
    fodd = np.where((ir + ns) & 1, 1.0, 0.5)
    theta[belt] = np.arccos((2 * ns - ir) * 2.0 / (3.0 * ns))
    phi[belt] = (ip - fodd) * (np.pi / 2 / ns)
    # south cap
    q = npix - p[south]
    ir = (1 + np.floor(np.sqrt(2 * q - 1))).astype(np.int64) // 2
    ip = 4 * ir + 1 - (q - 2 * ir * (ir - 1))
    theta[south] = np.arccos(ir * ir / (3.0 * ns * ns) - 1.0)
    phi[south] = (ip - 0.5) * (np.pi / 2 / ir)
    return theta, phi


def radec2pix(nside: int, ra, dec, nest: bool = True) -> np.ndarray:
    """util.radec2pix: pixel of (RA, DEC) in degrees."""
    ra = np.asarray(ra, np.float64)
    dec = np.asarray(dec, np.float64)
    return ang2pix(nside, np.pi / 2 - dec * np.pi / 180, ra * np.pi / 180, nest=nest)
