"""Drop-in for bin/merge_spectra.py: the spectra of one slice merged per quasar, missing
small-scale power added and the FGPA applied, written per healpix pixel as
spectra_merged-{pix}-{i}.fits.gz (bin/merge_spectra.py:385-406: METADATA, LAMBDA, FLUX, + DELTA_L,
GROWTHF, VELO_PAR with -dla True, + ETA_PAR, Z, DELTA_S with --store-g True).

    python -m saclaymocks_gb300.bin.merge_spectra -inDir spec -outDir merged -i 0 -aa 0.1 -bb 1.6 -cc 0.5

Same flags and files as the reference, and the same loop (:124-339):
  * the spectra files whose last number is i; rows grouped by healpix pixel of (RA, DEC)
    (-nside, -nest) and, inside a pixel, by THING_ID in ascending order; rows of one quasar
    concatenated and sorted by wavelength; with --check-id True (default) quasars absent from
    the catalogues in {inDir}/../qso are skipped;
  * np.random.seed(seed + i); per quasar with Lya-forest pixels (lambda/(1+Z) < lya), white
    noise of 256*2^n >= len+50 points (--noise numpy, the reference's draws, default) or
    Fourier modes drawn on the GPU (--noise gpu);
  * default branch: the P1D_miss table of -p1dfile (extensions z, k, pk, sigma) nearest to
    zeff = mean z of the forest pixels, clipped at 0, and delta_s rescaled by sigma(z)/sigma(zeff);
    --fit-p1d True: the spline of the P1Dmiss[RSD] column, no rescale;
  * F = exp(-a exp(b G (delta_l + delta_s + c eta_par))), G = fgrowth(2.4) 3.4/(1+z), a, b, c
    fixed (-aa/-bb/-cc > 0) or linear in z from -paramfile; spectra of another length than
    the header's Npixel are dropped after their draw, as in the reference.
All spectra of the slice go through the GPU in one launch (SMK_INTERP_PIXELS).
Differences: a P1D_miss negative in the --fit-p1d spline is clipped at 0 (the reference takes
its square root and gets NaN); a, b, c and sigma_s clamp outside their redshift tables (the
reference raises).  Extra flags: --noise numpy|gpu, --p1d-analytic AMP,KSCALE (P1D_miss =
AMP exp(-(k/KSCALE)^2) for every redshift, when no P1D_miss file is at hand).
"""
from __future__ import annotations

import argparse
import glob
import os
import sys

import numpy as np
import torch

from .make_boxes import str2bool

LYA = 1215.67      # py/SaclayMocks/constant.py:12
LYLIMIT = 0.0      # py/SaclayMocks/constant.py:14


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
    p.add_argument("--check-id", default="True")
    p.add_argument("-ncpu", type=int, default=2)
    p.add_argument("--noise", choices=["numpy", "gpu"], default="numpy")
    p.add_argument("--p1d-analytic", default=None)
    return p


def read_inputs(indir, islice, rsd, dla):
    """Rows of every spectra file of slice i (bin/merge_spectra.py:124-212)."""
    from saclaymocks_gb300 import fits
    rows, header = [], None
    for f in sorted(os.listdir(indir)):
        if f[f.rfind("-") + 1:f.find(".")] != str(islice):
            continue
        hd = {h.name: h for h in fits.read_fits(os.path.join(indir, f))}
        m = hd["METADATA"].data
        if len(m) == 0:
            print(f"*WARNING* fits table empty: {f}")
            continue
        if header is None:
            header = hd["METADATA"].header
        lam = hd["LAMBDA"].data
        for r in range(len(m)):
            ok = lam[r] > 0
            row = dict(meta=m[r], wav=lam[r][ok], delta_l=hd["DELTA_L"].data[r][ok],
                       z=hd["REDSHIFT"].data[r][ok])
            if rsd:
                row["eta"] = hd["ETA_PAR"].data[r][ok]
                if dla:
                    row["velo"] = hd["VELO_PAR"].data[r][ok]
            rows.append(row)
    return rows, header


def qso_ids(indir):
    """THING_ID of every readable catalogue in {inDir}/../qso (--check-id, :96-106)."""
    from saclaymocks_gb300 import fits
    ids = []
    for f in glob.glob(os.path.join(indir, "..", "qso", "*")):
        try:
            ids.append(np.asarray(fits.read(f, 1)["THING_ID"]))
        except Exception:
            print(f"Can't read file: {f}")
    if not ids:
        raise SystemExit(f"merge_spectra: --check-id True needs the QSO catalogues in {os.path.join(indir, '..', 'qso')}")
    return np.concatenate(ids)


def main(argv=None):
    from saclaymocks_gb300 import _lib, fits, healpix, spectra
    from saclaymocks_gb300.util import fgrowth
    args = parser().parse_args(argv)
    rsd, addnoise, dla = str2bool(args.rsd), str2bool(args.addnoise), str2bool(args.dla)
    fit_p1d, store_g, check_id = str2bool(args.fit_p1d), str2bool(args.store_g), str2bool(args.check_id)
    nest = str2bool(args.nest)
    if fit_p1d:
        store_g = True
    # P1D missing (:108-118)
    pmiss = None
    if args.p1d_analytic:
        amp, ks = (float(v) for v in args.p1d_analytic.split(","))
        pmiss = spectra.pmiss_gauss(amp, ks)
    else:
        path = args.p1dfile or os.path.expandvars("$SACLAYMOCKS_BASE/etc/pkmiss_interp.fits.gz")
        if not os.path.exists(path):
            raise SystemExit(f"merge_spectra: P1D missing file {path} not found (give -p1dfile, or "
                             "--p1d-analytic AMP,KSCALE)")
        print(f"Reading P1D file {path}")
        if fit_p1d:
            from scipy.interpolate import InterpolatedUnivariateSpline
            t = fits.read_table_columns(path, 1)
            pmiss = InterpolatedUnivariateSpline(t["k"], t["P1DmissRSD" if rsd else "P1Dmiss"])
        else:
            pmiss = spectra.P1DMissTable.from_fits(path)
    # FGPA parameters (:58-75)
    abc = dict(abc_mode=_lib.SMK_ABC_CONST, a=args.aa, b=args.bb, c=args.cc)
    if args.aa <= 0 or args.bb <= 0 or args.cc <= 0:
        pf = args.paramfile or os.path.expandvars("$SACLAYMOCKS_BASE/etc/params.fits")
        if not os.path.exists(pf):
            raise SystemExit(f"merge_spectra: parameter file {pf} not found (give -paramfile or -aa/-bb/-cc)")
        t = fits.read_table_columns(pf, 1)
        tab = np.stack([t["z"], t["a"], t["b"], t["c"]], 1).astype(np.float64)
        for col, v in ((1, args.aa), (2, args.bb), (3, args.cc)):
            if v > 0:
                tab[:, col] = v
        abc = dict(abc_mode=_lib.SMK_ABC_TABLE, abc_table=tab)
    if args.seed is None:
        seed = int(np.random.randint(2 ** 31 - 1))
        print(f"Seed has not been specified. Seed is set to {seed}")
    else:
        seed = args.seed + args.i
        print(f"Specified seed is {seed}")
    known = qso_ids(args.inDir) if check_id else None

    rows, header = read_inputs(args.inDir, args.i, rsd, dla)
    if not rows:
        print("No fits file opened. Exit.")
        raise SystemExit(0)
    npixeltot = int(header["NPIXEL"])
    ids = np.array([int(r["meta"]["THING_ID"]) for r in rows])
    ra = np.array([float(r["meta"]["RA"]) for r in rows])
    dec = np.array([float(r["meta"]["DEC"]) for r in rows])
    hpix = healpix.radec2pix(args.nside, ra, dec, nest=nest)
    # merged spectra in the loop's order: healpix pixel, then THING_ID (:225-268)
    spectra_list = []
    for pix in np.unique(hpix):
        cut = np.nonzero(hpix == pix)[0]
        for tid in np.unique(ids[cut]):
            msk = cut[ids[cut] == tid]
            if known is not None and not np.isin(tid, known):
                print(f"WARNING ID: {tid} didn't match any QSO ID")
                continue
            wav = np.concatenate([rows[k]["wav"] for k in msk])
            o = np.argsort(wav)
            cat = lambda key: np.concatenate([rows[k][key] for k in msk])[o]  # noqa: E731
            z = cat("z") if args.zfix is None else np.full(len(wav), args.zfix, np.float32)
            m0 = rows[msk[0]]["meta"]
            sp = dict(pix=int(pix), tid=int(tid), wav=wav[o], z=z, delta_l=cat("delta_l"), zq=float(m0["Z"]),
                      meta=m0, nmerged=len(msk))
            if rsd:
                sp["eta"] = cat("eta")
                if dla:
                    sp["velo"] = cat("velo")
            spectra_list.append(sp)
    n = len(spectra_list)
    if n == 0:
        print("No spectrum left. Exit.")
        return []
    npix = np.array([len(s["wav"]) for s in spectra_list], np.int32)
    forest = spectra.forest_ranges([s["wav"] for s in spectra_list], [s["zq"] for s in spectra_list],
                                   lya=LYA, lylimit=LYLIMIT)
    table = spectra.SkewerTable(np.zeros((n, 3)), np.tile([0, 0, 1.0], (n, 1)), npix, dpix=args.pixsize,
                                forest=forest)
    dev = lambda rows_: torch.from_numpy(np.concatenate(rows_).astype(np.float32)).cuda()  # noqa: E731
    pix_in = (dev([s["delta_l"] for s in spectra_list]),
              dev([s["eta"] for s in spectra_list]) if rsd else None,
              dev([s["z"] for s in spectra_list]))
    ss_mode = (_lib.SMK_SS_NONE if not addnoise else
               _lib.SMK_SS_HOST if args.noise == "numpy" else _lib.SMK_SS_PHILOX)
    cfg = spectra.SpectraConfig(ss_mode=ss_mode, ss_nz=0, pmiss=pmiss, pixsize=args.pixsize, seed=seed,
                                growth=_lib.SMK_G_MERGE, **abc)
    noise = None
    if ss_mode == _lib.SMK_SS_HOST:
        # np.random.seed(seed) then one normal(nz) per quasar with forest pixels, in loop order
        rs = np.random.RandomState(seed)
        offs, draws, o = np.zeros(n, np.int64), [], 0
        for s in range(n):
            offs[s] = o
            if forest[s, 1] > forest[s, 0]:
                d = rs.normal(size=spectra.nz_rule(int(npix[s])))
                draws.append(d)
                o += len(d)
        buf = np.concatenate(draws) if draws else np.zeros(1)
        noise = (torch.from_numpy(buf.astype(np.float32)).cuda(), torch.from_numpy(offs).cuda())
    r = spectra.SkewerRunner(table, cfg, pixels=pix_in)
    F = spectra.split(r.run(noise=noise), table)
    dsm = None
    if store_g:
        # delta_s itself: the same launch on delta_l = 0 (same noise, the same small-scale field),
        # since (delta_l + delta_s) - delta_l loses delta_s where delta_l = -1e6 beyond the forest
        r.pixels = (torch.zeros_like(pix_in[0]), pix_in[1], pix_in[2])
        _, ds_dev, _, _ = r.run(noise=noise, want_fields=True)
        dsm = spectra.split(ds_dev, table)

    g24 = float(fgrowth(2.4))
    names = ["RA", "DEC", "Z_noRSD", "Z", "HDU", "THING_ID", "PLATE", "MJD", "FIBERID", "PMF"]
    hlist = {"z0": header.get("Z0", 0.0), "NX": header.get("NX", 1), "dmax": header.get("DMAX", 3),
             "ra0": header.get("RA0", 0.0), "dec0": header.get("DEC0", 0.0)}
    os.makedirs(args.outDir, exist_ok=True)
    paths, written = [], 0
    for pix in np.unique([s["pix"] for s in spectra_list]):
        keep = [k for k, s in enumerate(spectra_list) if s["pix"] == pix]
        good = []
        for k in keep:
            if npix[k] != npixeltot:
                sp = spectra_list[k]
                print(f"/!\\ WARNING Spectrum hasn't the nominal lenght /!\\ ID: {sp['tid']} in healpix: {pix} "
                      f"and z: {sp['zq']}  Lenght {npix[k]} != {npixeltot}")
                continue
            good.append(k)
        if not good:
            continue
        last = spectra_list[good[-1]]
        meta = {nm: np.array([spectra_list[k]["meta"][nm] for k in good]) for nm in names if nm != "HDU"}
        meta["HDU"] = np.full(len(good), args.i, np.int64)
        meta = {nm: meta[nm] for nm in names}
        growth = (g24 * 3.4 / (1 + last["z"].astype(np.float64))).astype(np.float32)
        path = os.path.join(args.outDir, f"spectra_merged-{pix}-{args.i}.fits.gz")
        w = fits.FitsWriter(path)
        w.table(meta, hlist, extname="METADATA")
        w.image(last["wav"].astype(np.float32), extname="LAMBDA")
        w.image(np.array([F[k] for k in good], np.float32), extname="FLUX")
        if dla or store_g:
            w.image(np.array([spectra_list[k]["delta_l"] for k in good], np.float32), extname="DELTA_L")
            w.image(growth, extname="GROWTHF")
            w.image(np.array([spectra_list[k]["velo"] if (rsd and dla) else np.zeros(npixeltot)
                              for k in good], np.float32), extname="VELO_PAR")
        if store_g:
            w.image(np.array([spectra_list[k]["eta"] if rsd else np.zeros(npixeltot) for k in good], np.float32),
                    extname="ETA_PAR")
            w.image(last["z"].astype(np.float32), extname="Z")
            w.image(np.array([dsm[k] for k in good], np.float32), extname="DELTA_S")
        w.close()
        paths.append(path)
        written += len(good)
    print(f"{len(rows)} initial forests, {sum(s['nmerged'] > 1 for s in spectra_list)} forest mergers, "
          f"{written} total forest written.")
    return paths


if __name__ == "__main__":
    main(sys.argv[1:])
