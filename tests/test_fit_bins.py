"""The fit kernels bin the modes of a length-N spectrum through integer thresholds on m computed
once per length (csrc/smk_fit.cu, kbin_thresholds / kbin_thr).  The same rule restated here in
FP64 numpy gives exactly the bins of numpy's rfftfreq(N)*2*k_ny + searchsorted(edges, k,
'right') - 1 with the last edge inclusive (util.MakeProfileHisto's binning of
py/SaclayMocks/powerspectrum.py:231-238), including modes that sit exactly on an edge."""
import numpy as np


def kfreq(m, N, kfac):
    return (np.float64(m) * (1.0 / np.float64(N))) * kfac


def thresholds(N, kfac, edges):
    half = N // 2
    nkb = len(edges) - 1
    thr = np.zeros(nkb + 1, np.int64)
    for b in range(nkb + 1):
        e = edges[b]
        m = int(min(max(np.floor(e * N / kfac), 0.0), half + 1))
        if b < nkb:
            while m > 0 and kfreq(m - 1, N, kfac) >= e:
                m -= 1
            while m <= half and kfreq(m, N, kfac) < e:
                m += 1
        else:
            while m > 0 and kfreq(m - 1, N, kfac) > e:
                m -= 1
            while m <= half and kfreq(m, N, kfac) <= e:
                m += 1
        thr[b] = m
    return thr


def bin_thr(m, thr):
    nkb = len(thr) - 1
    if m < thr[0] or m >= thr[nkb]:
        return -1
    lo, hi = 0, nkb
    while hi - lo > 1:
        mid = (lo + hi) >> 1
        if thr[mid] <= m:
            lo = mid
        else:
            hi = mid
    return lo


def bin_numpy(k, edges):
    b = np.searchsorted(edges, k, side="right") - 1
    b[k == edges[-1]] = len(edges) - 2
    b[(k < edges[0]) | (k > edges[-1])] = -1
    return b


def test_thresholds_give_the_searchsorted_bins():
    dx = 0.2
    kfac = 2.0 * (np.pi / dx)
    rng = np.random.RandomState(4)
    for edges in (np.logspace(np.log10(0.05), np.log10(15.0), 33), np.linspace(0.0, 10.0, 11)):
        for N in list(rng.randint(1, 2049, 120)) + [1, 2, 3, 2048]:
            k = np.fft.rfftfreq(N) * 2 * (np.pi / dx)
            ref = bin_numpy(k, edges)
            thr = thresholds(N, kfac, edges)
            got = np.array([bin_thr(m, thr) for m in range(N // 2 + 1)])
            np.testing.assert_array_equal(got, ref, err_msg=f"N={N}")


def test_modes_on_the_edges():
    """Edges placed exactly on mode frequencies (first, inner and the inclusive last edge), and
    repeated edges (an empty bin)."""
    dx = 0.2
    kfac = 2.0 * (np.pi / dx)
    for N in (100, 257, 1024, 1199):
        k = kfreq(np.arange(N // 2 + 1), N, kfac)
        edges = np.array([k[3], k[10], k[10], k[17], k[N // 4], k[N // 2 - 1]])
        ref = bin_numpy(k, edges)
        thr = thresholds(N, kfac, edges)
        got = np.array([bin_thr(m, thr) for m in range(N // 2 + 1)])
        np.testing.assert_array_equal(got, ref, err_msg=f"N={N}")
