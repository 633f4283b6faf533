"""Numpy restatement of the GPU noise generator (Philox4x32-10 + Box-Muller), used to check
the kernels' GPU-noise modes against the oracle on identical white noise.

Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror & Shaw, "Parallel
random numbers: as easy as 1, 2, 3" (SC'11).  The counter/key layout and the uniform ->
Gaussian mapping follow saclaymocks_gb300/csrc/smk_common.cuh: block (q, row, tag) keyed
by the 64-bit seed gives four uint32 x0..x3; u = ((x >> 8) + 1) 2^-24 in (0,1],
t = (x >> 8) 2^-23 in [0,2); (g0, g1) = sqrt(-2 ln u(x0)) (cos, sin)(pi t(x1)), same for
(x2, x3).  TEST INFRASTRUCTURE ONLY (float64 arithmetic; the GPU computes in float32).
"""
from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)
STREAM_BOX, STREAM_SKEWER = 0x42, 0x53


def philox4x32_10(c0, c1, c2, c3, seed: int):
    c = [np.asarray(x, np.uint64) & MASK for x in np.broadcast_arrays(c0, c1, c2, c3)]
    k0 = np.uint64(seed & 0xFFFFFFFF)
    k1 = np.uint64((seed >> 32) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c


def gauss4(x):
    out = []
    for h in range(2):
        u1 = ((x[2 * h] >> np.uint64(8)) + np.uint64(1)).astype(np.float64) * 2.0 ** -24
        t = (x[2 * h + 1] >> np.uint64(8)).astype(np.float64) * 2.0 ** -23
        rad = np.sqrt(-2.0 * np.log(u1))
        out += [rad * np.cos(np.pi * t), rad * np.sin(np.pi * t)]
    return out


def box_noise(nx: int, ny: int, nz: int, seed: int) -> np.ndarray:
    """White-noise box of the GPU Philox mode ([nx, ny, nz], float64)."""
    rows = nx * ny
    ng = (nz + 3) // 4
    row = np.repeat(np.arange(rows, dtype=np.uint64), ng)
    q = np.tile(np.arange(ng, dtype=np.uint64), rows)
    x = philox4x32_10(q, row & MASK, row >> np.uint64(32), STREAM_BOX, seed)
    g = np.stack(gauss4(x), 1).reshape(rows, ng * 4)[:, :nz]
    return g.reshape(nx, ny, nz)


def skewer_modes(skewer_id: int, nz: int, seed: int):
    """(re, im) standard normals for k = 0..nz/2 of one skewer's small-scale field."""
    half = nz // 2
    nj = half // 2 + 1
    j = np.arange(nj, dtype=np.uint64)
    sid = np.uint64(skewer_id)
    x = philox4x32_10(j, sid & MASK, sid >> np.uint64(32), STREAM_SKEWER, seed)
    g = gauss4(x)
    re = np.stack([g[0], g[2]], 1).reshape(-1)[:half + 1]
    im = np.stack([g[1], g[3]], 1).reshape(-1)[:half + 1]
    return re, im


def skewer_small_scales(skewer_id: int, nz: int, seed: int, scale: np.ndarray, length: int):
    """delta_s of the GPU Philox mode: Fourier modes of white noise drawn directly
    (X_k = sqrt(nz/2)(g_re + i g_im), X_0 and X_{nz/2} = sqrt(nz) g_re), times the
    sqrt(P1Dmiss/pix) scale, irfft (1/nz), first `length` values."""
    re, im = skewer_modes(skewer_id, nz, seed)
    X = np.sqrt(nz / 2.0) * (re + 1j * im)
    X[0] = np.sqrt(nz) * re[0]
    X[-1] = np.sqrt(nz) * re[-1]
    return np.fft.irfft(X * scale, n=nz)[:length]
