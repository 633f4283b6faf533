"""Drop-in for bin/merge_spectra.py: small-scale power and FGPA for the spectra of
make_spectra, written as spectra_merged-{pix}-{i}.fits.gz (bin/merge_spectra.py:385-406:
METADATA, LAMBDA, FLUX, + DELTA_L, GROWTHF, ETA_PAR, Z, DELTA_S with --store-g).

    python -m saclaymocks_gb300.bin.merge_spectra -inDir spec -outDir merged -i 0 -aa 0.1 -bb 1.6 -cc 0.5

Per spectrum (one GPU launch for all of them, SMK_INTERP_PIXELS): nz = 256*2^n >= len+50,
white noise (--noise numpy: RandomState(seed+i).normal(nz) in THING_ID order, the reference's
draws; gpu: Fourier modes drawn on the GPU), x sqrt(P1Dmiss(k)/pixsize) (--fit-p1d True: spline
of the p1dfile's P1Dmiss[RSD] column, else the first table of the file interpolated
linearly), delta = delta_l + delta_s, F = exp(-a exp(b G (delta + c eta_par))) with
G = fgrowth(2.4) * 3.4/(1+z), a, b, c fixed (-aa/-bb/-cc > 0) or from -paramfile.
Differences: spectra of different lengths are kept (FLUX rows padded with -1); one output per
input slice (no healpix split); the sigma_s(z)/sigma_s(zeff) rescaling of the default p1d
path is not applied.
"""
from __future__ import annotations

import argparse
import glob
import os
import sys

import numpy as np
import torch

from .make_boxes import str2bool
from .make_spectra import LYA


def parser():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("-inDir", required=True)
    p.add_argument("-outDir", default=".")
    p.add_argument("-i", type=int, default=0)
    p.add_argument("-aa", type=float, default=-1)
    p.add_argument("-bb", type=float, default=1.58)
    p.add_argument("-cc", type=float, default=-1)
    p.add_argument("-paramfile", default=None)
    p.add_argument("-p1dfile", default=None)
    p.add_argument("-pixsize", type=float, default=0.2)
    p.add_argument("-nside", type=int, default=16)
    p.add_argument("-nest", default="True")
    p.add_argument("-rsd", default="True")
    p.add_argument("-addnoise", default="True")
    p.add_argument("-dla", default="False")
    p.add_argument("-zfix", type=float, default=None)
    p.add_argument("--fit-p1d", default="False")
    p.add_argument("--store-g", default="False")
    p.add_argument("-seed", type=int, default=None)
    p.add_argument("--check-id", default="False")
    p.add_argument("-ncpu", type=int, default=2)
    p.add_argument("--noise", choices=["numpy", "gpu"], default="numpy")
    return p


def read_inputs(indir, islice):
    """All spectra of slice i (files whose last number is i, as merge_spectra :124-132)."""
    from saclaymocks_gb300 import fits
    meta, wav, dl, et, zz = [], [], [], [], []
    for f in sorted(glob.glob(os.path.join(indir, "spectra-*.fits*"))):
        base = os.path.basename(f)
        if base[base.rfind("-") + 1:base.find(".")] != str(islice):
            continue
        hd = {h.name: h for h in fits.read_fits(f)}
        m = hd["METADATA"].data
        lam = hd["LAMBDA"].data
        for r in range(len(m)):
            ok = lam[r] > 0
            meta.append(m[r])
            wav.append(lam[r][ok])
            dl.append(hd["DELTA_L"].data[r][ok])
            et.append(hd["ETA_PAR"].data[r][ok] if "ETA_PAR" in hd else np.zeros(ok.sum(), np.float32))
            zz.append(hd["REDSHIFT"].data[r][ok])
    return meta, wav, dl, et, zz


def main(argv=None):
    from saclaymocks_gb300 import _lib, fits, spectra
    from saclaymocks_gb300.util import fgrowth
    args = parser().parse_args(argv)
    rsd, addnoise, store_g = str2bool(args.rsd), str2bool(args.addnoise), str2bool(args.store_g)
    fit_p1d = str2bool(args.fit_p1d)
    meta, wav, dl, et, zz = read_inputs(args.inDir, args.i)
    if not meta:
        raise SystemExit("No fits file opened. Exit.")
    ids = np.array([int(m["THING_ID"]) for m in meta])
    order = np.argsort(ids, kind="stable")                   # merge_spectra walks np.unique(IDs)
    wav, dl, et, zz = ([x[k] for k in order] for x in (wav, dl, et, zz))
    meta = [meta[k] for k in order]
    if args.zfix is not None:
        zz = [np.full_like(z, args.zfix) for z in zz]
    npix = np.array([len(x) for x in dl], np.int32)
    table = spectra.SkewerTable(np.zeros((len(npix), 3)), np.tile([0, 0, 1.0], (len(npix), 1)), npix,
                                dpix=args.pixsize)
    cat = lambda rows: torch.from_numpy(np.concatenate(rows).astype(np.float32)).cuda()  # noqa: E731
    pix = (cat(dl), cat(et) if rsd else None, cat(zz))
    # P1D missing: spline of the fit-p1d column, or the first redshift table of the file
    pmiss = spectra.pmiss_gauss()
    if args.p1dfile:
        if fit_p1d:
            from scipy.interpolate import InterpolatedUnivariateSpline
            t = fits.read_table_columns(args.p1dfile, 1)
            col = "P1DmissRSD" if rsd and "P1DmissRSD" in t else "P1Dmiss"
            pmiss = InterpolatedUnivariateSpline(t["k"], t[col])
        else:
            kt = np.asarray(fits.read(args.p1dfile, "k"), np.float64)
            pk = np.asarray(fits.read(args.p1dfile, "pk"), np.float64)
            pmiss = lambda k: np.interp(k, kt, pk[0])  # noqa: E731
    abc = dict(abc_mode=_lib.SMK_ABC_CONST, a=args.aa, b=args.bb, c=args.cc)
    if args.aa <= 0 or args.cc <= 0 or args.bb <= 0:
        pf = args.paramfile or os.path.join(os.path.dirname(args.inDir), "params.fits")
        t = fits.read_table_columns(pf, 1)
        tab = np.stack([t["z"], t["a"], t["b"], t["c"]], 1)
        if args.aa > 0:
            tab[:, 1] = args.aa
        if args.bb > 0:
            tab[:, 2] = args.bb
        if args.cc > 0:
            tab[:, 3] = args.cc
        abc = dict(abc_mode=_lib.SMK_ABC_TABLE, abc_table=tab)
    seed = (args.seed if args.seed is not None else int(np.random.randint(2 ** 31 - 1))) + args.i
    cfg = spectra.SpectraConfig(ss_mode=(_lib.SMK_SS_NONE if not addnoise else
                                         _lib.SMK_SS_HOST if args.noise == "numpy" else _lib.SMK_SS_PHILOX),
                                ss_nz=0, pmiss=pmiss, pixsize=args.pixsize, seed=seed,
                                growth=_lib.SMK_G_MERGE, **abc)
    noise = None
    if addnoise and args.noise == "numpy":
        rs = np.random.RandomState(seed)
        draws = [rs.normal(size=spectra.nz_rule(int(n))) for n in npix]
        offs = np.concatenate([[0], np.cumsum([len(x) for x in draws])[:-1]]).astype(np.int64)
        noise = (torch.from_numpy(np.concatenate(draws).astype(np.float32)).cuda(), torch.from_numpy(offs).cuda())
    r = spectra.SkewerRunner(table, cfg, pixels=pix)
    F, dtot, _, _ = r.run(noise=noise, want_fields=True)
    F, dtot = spectra.split(F, table), spectra.split(dtot, table)
    n = len(meta)
    maxsize = int(npix.max())

    def padded(rows, fill=-1.0):
        out = np.full((n, maxsize), fill, np.float32)
        for k, x in enumerate(rows):
            out[k, :len(x)] = x
        return out
    names = meta[0].dtype.names
    cols = {nm: np.array([m[nm] for m in meta]) for nm in names}
    os.makedirs(args.outDir, exist_ok=True)
    path = os.path.join(args.outDir, f"spectra_merged-0-{args.i}.fits.gz")
    w = fits.FitsWriter(path)
    w.table(cols, {"NX": 1}, extname="METADATA")
    w.image(padded(wav), extname="LAMBDA")
    w.image(padded(F), extname="FLUX")
    if store_g:
        g24 = float(fgrowth(2.4))
        w.image(padded(dl), extname="DELTA_L")
        w.image(padded([g24 * 3.4 / (1 + z) for z in zz]), extname="GROWTHF")
        w.image(padded(et), extname="ETA_PAR")
        w.image(padded(zz), extname="Z")
        w.image(padded([d - l for d, l in zip(dtot, dl)]), extname="DELTA_S")
    w.close()
    print(f"{n} spectra merged -> {path}")
    return path


if __name__ == "__main__":
    main(sys.argv[1:])
