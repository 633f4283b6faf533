"""Numpy restatement of the GPU noise generator (Philox4x32-10 + Box-Muller), used to check
the kernels' GPU-noise modes against the oracle on identical white noise.

Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror & Shaw, "Parallel
random numbers: as easy as 1, 2, 3" (SC'11).  The counter/key layout and the uniform ->
Gaussian mapping follow saclaymocks_gb300/csrc/smk_common.cuh: block (q, row, tag) keyed
by the 64-bit seed gives four uint32 x0..x3; with m = x >> 9 (23 bits), u = 1 - m 2^-23 in
(0,1], t = m 2^-22 in [0,2); (g0, g1) = sqrt(-2 ln u(x0)) (cos, sin)(pi t(x1)), same for
(x2, x3).  TEST INFRASTRUCTURE ONLY (float64 arithmetic; the GPU computes in float32).
"""
from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)
STREAM_KMODE, STREAM_SKEWER = 0x4B, 0x53


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
        u1 = 1.0 - (x[2 * h] >> np.uint64(9)).astype(np.float64) * 2.0 ** -23
        t = (x[2 * h + 1] >> np.uint64(9)).astype(np.float64) * 2.0 ** -22
        rad = np.sqrt(-2.0 * np.log(u1))
        out += [rad * np.cos(np.pi * t), rad * np.sin(np.pi * t)]
    return out


def kspace_noise(nx: int, ny: int, nz: int, seed: int) -> np.ndarray:
    """Fourier modes of white noise as the GPU noise mode draws them ([nx, ny, nz//2+1]
    complex128): mode (ix, iy, kz) takes Gaussians (2h, 2h+1), h = kz % 2, of the Philox block
    (kz // 2, ix, iy, STREAM_KMODE) keyed by seed; Re/Im scaled by sqrt(N/2).  On the kz = 0
    and kz = nz/2 planes, (ix, iy) and (-ix, -iy) are conjugate: the pair's lower flat index
    (ix*ny + iy) owns the draw, self-conjugate modes are real with scale sqrt(N)."""
    nzh = nz // 2 + 1
    N = nx * ny * nz
    ix = np.arange(nx, dtype=np.uint64)[:, None, None]
    iy = np.arange(ny, dtype=np.uint64)[None, :, None]
    kz = np.arange(nzh, dtype=np.uint64)[None, None, :]
    x = philox4x32_10(kz >> np.uint64(1), ix, iy, STREAM_KMODE, seed)
    g = gauss4(x)
    odd = (np.arange(nzh) % 2 == 1)[None, None, :]
    re = np.where(odd, g[2], g[0])
    im = np.where(odd, g[3], g[1])
    X = np.sqrt(N / 2.0) * (re + 1j * im)
    ixm = (-np.arange(nx)) % nx
    iym = (-np.arange(ny)) % ny
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    IM, JM = ixm[I], iym[J]
    selfc = (IM == I) & (JM == J)
    canon = I * ny + J < IM * ny + JM
    for p in sorted({0, nz // 2}):
        plane = X[:, :, p]
        mirrored = np.conj(plane[IM, JM])
        X[:, :, p] = np.where(selfc, np.sqrt(float(N)) * re[:, :, p],
                              np.where(canon, plane, mirrored))
    return X


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
