"""Regenerate the golden fixtures in this directory by running the REFERENCE's own code.

    python tests/golden/make_golden.py --ref <checkout of igmhub/SaclayMocks> [name ...]
    (or SACLAYMOCKS_REF=<checkout> python tests/golden/make_golden.py); names pick fixtures
    (grf, readspec, spectra, iterate, merge, util), default all.

Every fixture is produced by calling igmhub/SaclayMocks functions (or running a
pipeline script's ``main()``) under the import shims of ``ref_shims.py``:

* ``grf_*.npz``      bin/make_boxes.py ``main()`` (DrawGRF_boxk :40-72, P0 multiply
                     :288-292, FFTandStore :77-125, eta_ij :315-391) fed a served
                     sqrt(P/Vcell) grid of the analytic spectrum A*k/(1+(k/k0)^2)^2;
* ``readspec.npz``   ``ReadSpec``/``ComputeWeight``/``computeRho`` compiled out of
                     bin/make_spectra.py:39-139 (Gaussian 7^3-cell read + eta_par projection);
* ``spectra_qso.npz`` bin/make_spectra.py ``main()`` on box files and a QSO catalogue written
                     to disk (lines of sight :286-472, Gaussian read, METADATA/LAMBDA/DELTA_L/
                     ETA_PAR/REDSHIFT of spectra-{i}-{hdu});
* ``merge_*.npz``    bin/merge_spectra.py ``main()`` on a served spectra file
                     (small-scale loop :303-331 and FGPA :336-339);
* ``util.npz``       util.fgpa :421-433, util.fgrowth :123-134, util.sigma_p1d :372-398,
                     util.MakeProfileHisto :46-75, powerspectrum.P1D_1spectrum/ComputeP1D
                     :204-238, FGPApdf.Fmean/sig2F :39-58, fit_az.Fitter.chi2 :194-264.

The FFT inside the shimmed pyfftw is numpy's pocketfft in float64 rounded to the
reference's float32/complex64 arrays, so FFTW itself is not pinned (it is absent here).
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
if "--ref" in sys.argv:
    _k = sys.argv.index("--ref")
    os.environ["SACLAYMOCKS_REF"] = sys.argv[_k + 1]
    del sys.argv[_k:_k + 2]
import ref_shims  # noqa: E402

ref_shims.install()

K0 = 0.02          # h/Mpc, break scale of the analytic spectrum of the configs
DX = 2.19          # Mpc/h, box cell


def sqrt_pk_grid(NX, NY, NZ, dcell, k0):
    """sqrt(P/Vcell) grid laid out like bin/interpolate_pk.py:63-77 and :23-26, with
    P(k) = A*k/(1+(k/k0)^2)^2 and A such that the expected variance of delta is 1."""
    k_ny = np.pi / dcell
    kx = np.float32(np.fft.fftfreq(NX) * 2 * k_ny).reshape(-1, 1, 1)
    ky = np.float32(np.fft.fftfreq(NY) * 2 * k_ny).reshape(-1, 1)
    kz = np.float32(np.fft.rfftfreq(NZ) * 2 * k_ny)
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    kd = k.astype(np.float64)
    pt = kd / (1.0 + (kd / k0) ** 2) ** 2
    w = np.full(kz.shape, 2.0)
    w[0] = 1.0
    if NZ % 2 == 0:
        w[-1] = 1.0
    vcell = np.float32(dcell ** 3)
    ncell = NX * NY * NZ
    A = ncell * float(vcell) / float((pt * w).sum())
    P = np.float32(A * pt)
    return np.float32(np.sqrt(P / vcell)), A


def gen_grf(NX, NY, NZ, seed, tag):
    P0, A = sqrt_pk_grid(NX, NY, NZ, DX, K0)
    ref_shims.FITS_CAPTURE.clear()
    tmp = tempfile.mkdtemp()
    pname = f"P{NX}.fits" if NX == NY == NZ else f"P{NX}-{NY}-{NZ}.fits"
    # distinct grids for the three lognormal boxes (any float32 grid: the step is a multiply)
    kx = np.fft.fftfreq(NX).reshape(-1, 1, 1)
    ky = np.fft.fftfreq(NY).reshape(-1, 1)
    kz = np.fft.rfftfreq(NZ)
    kq = np.sqrt(kx * kx + ky * ky + kz * kz)
    pln = [np.float32(P0 * f) for f in (0.5, 1.0 + 2.0 * kq, np.exp(-4.0 * kq))]
    ref_shims.FITS_SERVE[pname] = {"P0": P0, "Pln1": pln[0], "Pln2": pln[1], "Pln3": pln[2], 0: P0}
    mb = ref_shims.load_script("make_boxes")
    argv = sys.argv
    sys.argv = ["make_boxes.py", "-NX", str(NX), "-NY", str(NY), "-NZ", str(NZ),
                "-pixel", str(DX), "-seed", str(seed), "-PkDir", tmp, "-outDir", tmp,
                "-ncpu", "1", "-rsd", "True"]
    try:
        mb.main()
    finally:
        sys.argv = argv
    cap = ref_shims.FITS_CAPTURE

    def stack(prefix):
        return np.concatenate([cap[f"{prefix}-{i}.fits"]["hdus"][0]["data"] for i in range(NX)])
    out = dict(NX=NX, NY=NY, NZ=NZ, DX=DX, seed=seed, A=A, k0=K0, P0=P0,
               delta=stack("box"),
               sigma=np.float32(cap["box-0.fits"]["hdus"][0]["header"]["sigma"]),
               boxk_scaled=np.load(os.path.join(tmp, "boxk.npy")))
    for f in ("eta_xx", "eta_yy", "eta_zz", "eta_xy", "eta_xz", "eta_yz"):
        out[f] = stack(f)
    # nHDU = 1 outputs: lognormal boxes (bin/make_boxes.py:241-275) and velocities (:393-431)
    for f in ("boxln_1", "boxln_2", "boxln_3", "vx", "vy", "vz"):
        out[f] = cap[f"{f}-0.fits"]["hdus"][0]["data"]
    for i, g in enumerate(pln):
        out[f"Pln{i + 1}"] = g
    from saclaymocks_gb300 import fits as _f
    dg = _f.read(os.path.join(ref_shims.REF, "etc", "dgrowth.fits"), 1)
    out["dgrowth0"] = np.float64(dg["dD/dz"][0])
    out["H0"] = np.float64(100.0)       # py/SaclayMocks/constant.py:36
    np.savez_compressed(os.path.join(HERE, f"grf_{tag}.npz"), **out)
    print("grf", tag, out["delta"].shape, "sigma", out["sigma"])
    return out


def gen_readspec(g):
    ns = ref_shims.load_nested("make_spectra", "main",
                               ("ComputeWeight", "computeRho", "ReadSpec"))
    NX, NY, NZ = int(g["NX"]), int(g["NY"]), int(g["NZ"])
    LX, LY, LZ = DX * NX, DX * NY, DX * NZ
    R0 = 100.0
    dmax = 3
    xx = 2 * dmax + 1
    cells = np.indices((xx, xx, xx)).reshape(3, -1) - dmax
    grid = np.array([DX * cells[0], DX * cells[1], DX * cells[2]]).T.copy()
    cells = cells.T.copy().astype(np.int64)
    rng = np.random.RandomState(11)
    npix = 60
    skewers = []
    for s in range(6):
        # start well inside [dmax, N-dmax-1] cells so every 7^3 neighbourhood is in the box
        p0 = np.array([rng.uniform(4, NX - 6), rng.uniform(4, NY - 6), rng.uniform(4, 5)]) * DX
        d = np.array([rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1), 1.0])
        d /= np.linalg.norm(d)
        t = np.arange(npix) * 0.2
        P = p0[None, :] + t[:, None] * d[None, :]
        X = P[:, 0] - LX / 2
        Y = P[:, 1] - LY / 2
        Z = P[:, 2] - LZ / 2 + R0
        empty = np.array([], dtype=np.float32)
        spec, eta, _ = ns["ReadSpec"](
            g["delta"].ravel(), NX, NY, NZ, X, X.copy(), Y, Z, grid, cells,
            LX, LY, LZ, DX, DX, DX, R0, 1, 0,
            g["eta_xx"].ravel(), g["eta_yy"].ravel(), g["eta_zz"].ravel(),
            g["eta_xy"].ravel(), g["eta_xz"].ravel(), g["eta_yz"].ravel(),
            empty, empty, empty, 0, npix)
        skewers.append(dict(pos=P, X=X, Y=Y, Z=Z, delta=spec, eta=eta))
    np.savez_compressed(os.path.join(HERE, "readspec.npz"),
                        pos=np.stack([s["pos"] for s in skewers]),
                        XYZ=np.stack([np.stack([s["X"], s["Y"], s["Z"]], 1) for s in skewers]),
                        delta_l=np.stack([s["delta"] for s in skewers]),
                        eta_par=np.stack([s["eta"] for s in skewers]),
                        R0=R0, grf="grf_cube16.npz")
    print("readspec", len(skewers), "skewers")


def _spectra_file(nspec, npix, rng):
    lya = 1215.67
    wav = np.linspace(3600.0, 3700.0, npix).astype(np.float32)
    ids = np.array([901, 17, 5003, 42, 77, 313][:nspec], dtype=np.int64)
    zq = np.full(nspec, 2.5)
    meta = np.zeros(nspec, dtype=[("RA", "f4"), ("DEC", "f4"), ("Z_noRSD", "f4"),
                                  ("Z", "f4"), ("HDU", "i8"), ("THING_ID", "i8"),
                                  ("PLATE", "i8"), ("MJD", "i4"), ("FIBERID", "i4"),
                                  ("PMF", "U22")])
    meta["THING_ID"] = ids
    meta["Z"] = zq
    meta["Z_noRSD"] = zq - 0.001
    meta["RA"] = np.linspace(10, 11, nspec)
    meta["DEC"] = np.linspace(-1, 1, nspec)
    hdr = {"z0": 1.70975268202, "pixel": 0.2, "NX": 1, "dmax": 3, "ra0": 0.0,
           "dec0": 0.0, "Npixel": npix}
    delta = rng.normal(0.0, 0.8, (nspec, npix)).astype(np.float32)
    eta = rng.normal(0.0, 0.3, (nspec, npix)).astype(np.float32)
    velo = rng.normal(0.0, 1.0, (nspec, npix)).astype(np.float32)
    red = np.tile((wav / lya - 1).astype(np.float32), (nspec, 1))
    served = {1: {"data": meta, "header": hdr},
              "LAMBDA": {"data": np.tile(wav, (nspec, 1))},
              "DELTA_L": {"data": delta}, "ETA_PAR": {"data": eta},
              "VELO_PAR": {"data": velo}, "REDSHIFT": {"data": red}}
    return served, dict(ids=ids, wav=wav, delta_l=delta, eta_par=eta, redshift=red[0], zq=zq)


def gen_merge(tag, fit_p1d, seed):
    rng = np.random.RandomState(3)
    npix = 300
    served, inputs = _spectra_file(6, npix, rng)
    tmp_in, tmp_out = tempfile.mkdtemp(), tempfile.mkdtemp()
    open(os.path.join(tmp_in, "spectra-0-0.fits.gz"), "wb").close()
    ref_shims.FITS_SERVE["spectra-0-0.fits.gz"] = served
    args = ["merge_spectra.py", "-inDir", tmp_in, "-outDir", tmp_out, "-i", "0",
            "-aa", "0.1", "-bb", "1.6", "-cc", "0.5", "-pixsize", "0.2", "-nside", "16",
            "-rsd", "True", "-addnoise", "True", "-dla", "True", "--check-id", "False",
            "-seed", str(seed), "-ncpu", "1"]
    extra = {}
    if fit_p1d:
        # The P1Dmiss tables in etc/ go negative below k_Nyquist=pi/0.2, where the fit
        # path of merge_spectra takes sqrt() without clipping and returns NaN; a smooth
        # positive table (analytic P1Dmiss plus a floor) keeps the spline path finite.
        kt = np.linspace(0.0, 19.999, 20000)
        tab = np.zeros(kt.size, dtype=[("k", ">f8"), ("P1DmissRSD", ">f8")])
        tab["k"] = kt
        tab["P1DmissRSD"] = 0.05 * np.exp(-(kt / 2.0) ** 2) + 1e-4
        ref_shims.FITS_SERVE["p1dmiss_test.fits"] = {1: {"data": tab}}
        args += ["--fit-p1d", "True", "--store-g", "True", "-p1dfile", "p1dmiss_test.fits"]
        extra = dict(pm_amp=0.05, pm_kscale=2.0, pm_floor=1e-4, pm_kmax=19.999, pm_n=20000)
    else:
        # served P1D-missing table in the layout util.InterpP1Dmissing reads (z, k, pk)
        zt = np.array([1.8, 2.4, 3.6])
        kt = np.linspace(0.0, 20.0, 4001)
        pk = np.stack([amp * 0.05 * np.exp(-(kt / 2.0) ** 2) for amp in (0.8, 1.0, 1.3)])
        sig = np.array([0.20, 0.22, 0.25])
        ref_shims.FITS_SERVE["pkmiss_test.fits"] = {
            "z": {"data": zt}, "k": {"data": kt}, "pk": {"data": pk}, "sigma": {"data": sig}}
        args += ["--fit-p1d", "False", "--store-g", "True", "-p1dfile", "pkmiss_test.fits"]
        extra = dict(pm_z=zt, pm_k=kt, pm_pk=pk, pm_sigma=sig)
    ref_shims.FITS_CAPTURE.clear()
    ms = ref_shims.load_script("merge_spectra")
    argv = sys.argv
    sys.argv = args
    try:
        ms.main()
    finally:
        sys.argv = argv
    rec = ref_shims.FITS_CAPTURE["spectra_merged-0-0.fits.gz"]["hdus"]
    hd = {h["extname"]: h["data"] for h in rec}
    order = np.argsort(inputs["ids"])          # merge_spectra walks np.unique(IDs)
    np.savez_compressed(os.path.join(HERE, f"merge_{tag}.npz"),
                        seed=seed, fit_p1d=fit_p1d, order=order,
                        wav=inputs["wav"], delta_l_in=inputs["delta_l"],
                        eta_par_in=inputs["eta_par"], redshift=inputs["redshift"],
                        zq=inputs["zq"], flux=hd["FLUX"], delta_s=hd["DELTA_S"],
                        growthf=hd["GROWTHF"], **extra)
    print("merge", tag, hd["FLUX"].shape, "delta_s std", hd["DELTA_S"].std())


def gen_util():
    from SaclayMocks import util, powerspectrum, FGPApdf, fit_az
    import numpy.ma as ma
    rng = np.random.RandomState(21)
    n = 2000
    delta = rng.normal(0, 1.2, n)
    eta = rng.normal(0, 0.5, n)
    G = rng.uniform(0.6, 1.0, n)
    a_arr = rng.uniform(0.05, 0.3, n)
    b_arr = rng.uniform(1.3, 1.8, n)
    c_arr = rng.uniform(0.4, 0.8, n)
    F_scalar = util.fgpa(delta, eta, G, 0.1, 1.6, 0.5)
    F_array = util.fgpa(delta, eta, G, a_arr, b_arr, c_arr)
    zg = np.linspace(0.0, 4.0, 41)
    fg = util.fgrowth(zg, 0.31457)
    pm = lambda k: 0.05 * np.exp(-(k / 2.0) ** 2)   # noqa: E731
    sig_s = util.sigma_p1d(p1dmiss=pm, pixel=0.2, N=10000)
    # P1D estimator on a few spectra of different lengths, binned like ComputeP1D.P1D
    specs = [rng.normal(0, 0.3, L) for L in (64, 100, 257, 300)]
    p1d = powerspectrum.ComputeP1D(0.2)
    for s in specs:
        p1d.add_spectrum(s)
    # MakeProfileHisto (util.py:63-73) only defines its bin mask when some bin is
    # empty, so the bin edges run past k_Nyquist = pi/0.2 to leave the last bins empty
    p1d_bins = np.linspace(0.0, 20.0, 13)
    k_b, p_b, e_b = p1d.P1D(bins=p1d_bins)
    one = powerspectrum.P1D_1spectrum(specs[1], 0.2)
    xh = rng.uniform(0, 10, 500)
    yh = rng.normal(0, 1, 500) + xh
    mx, my, me = util.MakeProfileHisto(xh, yh, bins=np.linspace(0, 12, 13))
    ln_a, b = -5.3199529, 5.71883103
    fm = FGPApdf.Fmean(ln_a, b)
    s2 = FGPApdf.sig2F(ln_a, b)
    # fit_az chi2 on stored fields (masked float64 arrays, as read_mock builds them)
    nsp, npx = 8, 200
    dl = rng.normal(0, 1.0, (nsp, npx))
    ds = rng.normal(0, 0.3, (nsp, npx))
    et = rng.normal(0, 0.4, (nsp, npx))
    mask = np.zeros((nsp, npx), bool)
    mask[:, 180:] = True
    gf = np.linspace(0.75, 0.85, npx)
    fitter = fit_az.Fitter("unused", 2.4, 0.5, bb=1.6)
    fitter.mock["delta_l"] = ma.array(dl, mask=mask)
    fitter.mock["delta_s"] = ma.array(ds, mask=mask)
    fitter.mock["eta_par"] = ma.array(et, mask=mask)
    fitter.mock["growthf"] = gf
    fitter.mock["mask_size"] = mask.size
    # 12 bins of 0.5 h/Mpc, one bin up to just past k_Nyquist, then an empty bin
    # (MakeProfileHisto needs one, util.py:63-73)
    edges = np.concatenate([np.arange(0.0, 6.01, 0.5), [15.8, 16.5]])
    kc = 0.5 * (edges[1:-1] + edges[:-2])
    fitter.data["bins"] = edges
    fitter.data["Pk"] = 0.1 * np.exp(-kc / 3.0)
    fitter.data["Pkerr"] = 0.01 + 0.0 * kc
    chi = [fitter.chi2(a) for a in (0.05, 0.1, 0.2)]
    np.savez_compressed(os.path.join(HERE, "util.npz"),
                        delta=delta, eta=eta, G=G, a_arr=a_arr, b_arr=b_arr, c_arr=c_arr,
                        F_scalar=F_scalar, F_array=F_array, zg=zg, fg=fg, sig_s=sig_s,
                        spec_lens=np.array([len(s) for s in specs]),
                        specs=np.concatenate(specs), p1d_bins=p1d_bins, k_b=k_b, p_b=p_b, e_b=e_b, one=one,
                        xh=xh, yh=yh, mx=mx, my=my, me=me, fm_ln_a=ln_a, fm_b=b,
                        fmean=fm, sig2F=s2, fit_dl=dl, fit_ds=ds, fit_eta=et,
                        fit_mask=mask, fit_gf=gf, fit_bins=fitter.data["bins"],
                        fit_pk=fitter.data["Pk"], fit_pkerr=fitter.data["Pkerr"],
                        fit_a=np.array([0.05, 0.1, 0.2]), fit_chi2=np.array(chi))
    print("util: Fmean", fm, "sigF", np.sqrt(s2), "chi2", chi)


def gen_iterate():
    """One step of fit_az.Fitter.iterate (py/SaclayMocks/fit_az.py:281-332) on synthetic
    mock / model / P1Dmiss arrays: the P1D-missing update (ratio spline, multiplicative
    update, smoothing spline).  The I/O and regeneration steps it ends with are stubbed."""
    import types

    import scipy.interpolate as si
    from SaclayMocks import fit_az
    rng = np.random.RandomState(21)
    k = np.linspace(0.12, 9.5, 40)
    model_k = np.linspace(0.05, 12.0, 200)
    model_p = 0.12 * np.exp(-model_k / 2.5) + 0.01
    p1d = (0.12 * np.exp(-k / 2.2) + 0.008) * (1 + 0.05 * rng.normal(size=k.size))
    err = 0.04 * p1d * (1 + 0.2 * rng.uniform(size=k.size))
    kmiss = np.arange(0.0, 20.0, 0.05)
    pmiss = 0.05 * np.exp(-(kmiss / 2.0) ** 2) + 1e-4
    outs = {}
    for cf, crit in ((1.0, None), (0.6, None), (1.0, 1e3)):
        obj = types.SimpleNamespace()
        obj.data = {"bins": None, "p1d_model_interp": si.interp1d(model_k, model_p)}
        obj.mock = {"k": k, "p1d": p1d, "err_p1d": err, "kmiss": kmiss, "p1dmiss": pmiss,
                    "p1dmiss_interp": si.InterpolatedUnivariateSpline(kmiss, pmiss)}
        obj.fit = {"a": 0.1}
        obj.convergence_factor = cf
        obj.convergence_criterium = crit
        obj.converged = False
        obj.niter = 0
        for name in ("export_p1dmiss", "gen_small_scales", "export_p1d"):
            setattr(obj, name, lambda *a, **kw: None)
        obj.compute_p1d = lambda *a, **kw: None
        fit_az.Fitter.iterate(obj)
        tag = f"cf{cf:g}" + ("_conv" if crit else "")
        outs[tag + "_converged"] = np.bool_(obj.converged)
        outs[tag + "_niter"] = np.int64(obj.niter)
        outs[tag + "_p1dmiss"] = np.asarray(obj.mock["p1dmiss"], np.float64)
        outs[tag + "_interp_on_kmiss"] = np.asarray(obj.mock["p1dmiss_interp"](kmiss), np.float64)
    np.savez_compressed(os.path.join(HERE, "iterate.npz"), k=k, p1d=p1d, err=err, model_k=model_k,
                        model_p=model_p, kmiss=kmiss, pmiss=pmiss, **outs)
    print("iterate: p1dmiss[0..3]", outs["cf1_p1dmiss"][:3])


def gen_spectra():
    """make_spectra main() on seeded 12 x 12 x 40 boxes of 12 Mpc/h cells (deep enough along z to
    reach lambda > 3476 A behind the box centre at z0) and a QSO catalogue, both written to disk:
    the lines of sight of bin/make_spectra.py:286-472 (cosmology, pixel grid, slice and forest
    cuts) and the Gaussian read, with the redshift range set so every line stays in the box."""
    from saclaymocks_gb300 import fits as _f
    NX, NY, NZ, dx = 12, 12, 40, 12.0
    rng = np.random.RandomState(23)
    names = ["delta"] + ["eta_" + c for c in ("xx", "yy", "zz", "xy", "xz", "yz")]
    boxes = {nm: rng.normal(0.0, 1.0 if nm == "delta" else 0.4, (NX, NY, NZ)).astype(np.float32) for nm in names}
    tmp = tempfile.mkdtemp()
    boxdir, outdir = os.path.join(tmp, "boxes"), os.path.join(tmp, "spec")
    os.makedirs(boxdir)
    os.makedirs(outdir)
    hdr = {"DX": dx, "DY": dx, "DZ": dx, "NX": NX, "NY": NY, "NZ": NZ}
    for nm in names:
        prefix = "box" if nm == "delta" else nm
        for i in range(NX):
            _f.write_image(os.path.join(boxdir, f"{prefix}-{i}.fits"), boxes[nm][i:i + 1], hdr)
    util = __import__("SaclayMocks.util", fromlist=["cosmo"])
    const = __import__("SaclayMocks.constant", fromlist=["h"])
    cos = util.cosmo(const.omega_M_0, Ok=const.omega_k_0, H0=100 * const.h)
    R0 = const.h * cos.r_comoving(const.z0)
    LX, LZ = dx * NX, dx * NZ
    margin = 3 * dx + 1.0
    zmin = max(float(cos.r_2_z((R0 - LZ / 2 + margin) / const.h)), 3480.0 / const.lya - 1)
    zmax = float(cos.r_2_z((R0 + LZ / 2 - margin) / const.h))
    n = 9
    ang = 0.8 * (LX / 2 - margin) / (R0 + LZ / 2) * 180 / np.pi     # degrees: lines stay inside
    ra = 180.0 + rng.uniform(-ang, ang, n)
    dec = rng.uniform(-ang, ang, n)
    zq = np.concatenate([[zmax, zmax - 1e-3], rng.uniform(zmin + 0.005, zmax, n - 4), [zmax + 0.01, zmin - 0.01]])
    ra[3] = 180.0 + 40 * ang                                  # outside the slice cone: skipped
    cat = {"RA": ra, "DEC": dec, "Z_QSO_NO_RSD": (zq - 1e-4).astype(np.float32),
           "Z_QSO_RSD": zq.astype(np.float32), "THING_ID": np.arange(100, 100 + n, dtype=np.int64),
           "HDU": np.array([0, 1, 0, 1, 0, 1, 0, 1, 0], np.int64),
           "PLATE": np.full(n, 7, np.int64), "MJD": np.full(n, 55000, np.int32),
           "FIBERID": np.arange(n, dtype=np.int32), "PMF": np.array([f"7-55000-{i}" for i in range(n)])}
    qso = os.path.join(tmp, "QSO-")
    _f.FitsWriter(qso + "0-1.fits").table(cat, {"RA0": 180.0, "DEC0": 0.0}).close()
    ref_shims.FITS_CAPTURE.clear()
    ms = ref_shims.load_script("make_spectra")
    argv = sys.argv
    sys.argv = ["make_spectra.py", "-QSOfile", qso, "-boxdir", boxdir, "-outDir", outdir, "-i", "0", "-N", "1",
                "-zmin", repr(zmin), "-zmax", repr(zmax), "-pixel", "0.2", "-dmax", "3", "-rsd", "True"]
    try:
        ms.main()
    finally:
        sys.argv = argv
    out = dict(zmin=zmin, zmax=zmax, dx=dx, **{f"box_{k}": v for k, v in boxes.items()},
               **{f"cat_{k}": v for k, v in cat.items() if k != "PMF"})
    for hdu in (0, 1):
        rec = ref_shims.FITS_CAPTURE[f"spectra-0-{hdu}.fits.gz"]["hdus"]
        hd = {h["extname"]: h for h in rec}
        for k in ("LAMBDA", "DELTA_L", "ETA_PAR", "REDSHIFT"):
            out[f"h{hdu}_{k}"] = np.asarray(hd[k]["data"])
        meta = hd["METADATA"]["data"]
        for k in ("THING_ID", "Z", "Z_noRSD", "RA", "DEC", "HDU"):
            out[f"h{hdu}_{k}"] = np.asarray(meta[k])
        hh = hd["METADATA"]["header"]
        out[f"h{hdu}_header"] = np.array([hh["z0"], hh["pixel"], hh["Npixel"], hh["NX"], hh["dmax"],
                                          hh["ra0"], hh["dec0"]], np.float64)
    np.savez_compressed(os.path.join(HERE, "spectra_qso.npz"), **out)
    print("spectra", {k: v.shape for k, v in out.items() if k.startswith("h")})


def main(names=()):
    want = lambda n: not names or n in names  # noqa: E731
    if want("grf"):
        g = gen_grf(16, 16, 16, 0, "cube16")
        gen_grf(20, 12, 18, 5, "rect")
    else:
        g = dict(np.load(os.path.join(HERE, "grf_cube16.npz")))
    if want("readspec"):
        gen_readspec(g)
    if want("spectra"):
        gen_spectra()
    if want("iterate"):
        gen_iterate()
    if want("merge"):
        gen_merge("fitp1d", True, 7)
        gen_merge("table", False, 9)
    if want("util"):
        gen_util()


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
