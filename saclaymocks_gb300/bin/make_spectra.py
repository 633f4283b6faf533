"""Drop-in for bin/make_spectra.py: delta_l and eta_par read along the lines of sight of a QSO
catalogue through the boxes of make_boxes, written as spectra-{i}-{hdu}.fits.gz
(bin/make_spectra.py:525-597: METADATA, LAMBDA, DELTA_L, ETA_PAR, REDSHIFT, rows padded with
-1 / -2e6).

    python -m saclaymocks_gb300.bin.make_spectra -QSOfile qso/QSO- -boxdir boxes -outDir spec -i 0 -N 1

Same flags and files as the reference:
  * the boxes of slice i (x planes [i nHDU/N - dmax, (i+1) nHDU/N + dmax), clipped to the box)
    are read from -boxdir: box-{x}.fits and, with -rsd True, eta_{xx,yy,zz,xy,xz,yz}-{x}.fits;
  * the quasars come from {QSOfile}{f}-{NQSOfile}.fits (f over the files the slice needs, RA0
    and DEC0 from the first file's header); their lines of sight are built on the host
    exactly as the reference builds them (los.py: pixel grid in comoving distance between
    -zmin and -zmax with -pixel spacing, lambda > 3476 A, slice cut, forest limits);
  * every pixel of the forest is read on the GPU with the reference's Gaussian (2 dmax + 1)^3
    weights and eta_par = r_i r_j eta_ij / r^2 (one launch for all quasars); the pixels beyond
    the forest keep delta_l = -1e6, eta_par = 0 as ReadSpec leaves them.
Differences: indices wrap periodically inside the slab read (the reference's flat index runs
into the neighbouring row within dmax cells of a y or z face); -dla True (velocity skewers)
is refused with an error.  Extra flag: --synthetic N (N skewers within 10 deg of +z through
the whole box, trilinear read of delta and eta_zz, redshift linear along x between -zmin and
-zmax), a benchmark input with no QSO catalogue.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np
import torch

from .make_boxes import str2bool

LYA = 1215.67  # py/SaclayMocks/constant.py:12
ETA6 = ("xx", "yy", "zz", "xy", "xz", "yz")


def parser():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("-dmax", type=int, default=3)
    p.add_argument("-pixel", type=float, default=0.2)
    p.add_argument("-zmin", type=float, default=1.3)
    p.add_argument("-zmax", type=float, default=3.6)
    p.add_argument("-QSOfile", default=None)
    p.add_argument("-boxdir", required=True)
    p.add_argument("-outDir", default=".")
    p.add_argument("-i", type=int, default=0)
    p.add_argument("-N", type=int, default=1)
    p.add_argument("-NQSOfile", type=int, default=-1)
    p.add_argument("-NQSO", type=int, default=-1)
    p.add_argument("-rsd", default="True")
    p.add_argument("-dla", default="False")
    p.add_argument("-dgrowthfile", default=None)
    p.add_argument("--synthetic", type=int, default=0)
    p.add_argument("--seed", type=int, default=1)
    return p


def load_planes(boxdir, prefix, i0, i1, pitch=None):
    """Stack the one-plane files {prefix}-{i}.fits, i in [i0, i1), into a padded CUDA box."""
    from saclaymocks_gb300 import fits, grf
    h = fits.read_header(os.path.join(boxdir, f"{prefix}-{i0}.fits"))
    NY, NZ = int(h["NAXIS2"]), int(h["NAXIS1"])
    pad = torch.zeros((i1 - i0, NY, pitch or grf.pitch_of(NZ)), dtype=torch.float32)
    for k, i in enumerate(range(i0, i1)):
        path = os.path.join(boxdir, f"{prefix}-{i}.fits")
        if not os.path.exists(path):
            raise SystemExit(f"missing box file {path}")
        pad[k, :, :NZ] = torch.from_numpy(np.ascontiguousarray(fits.read(path)[0]))
    return pad.cuda()


def read_qsos(args, n_slice):
    """The QSO files of the slice, as bin/make_spectra.py:323-381 selects and reads them."""
    from saclaymocks_gb300 import fits
    nqf = n_slice if args.NQSOfile < 0 else args.NQSOfile
    if args.i >= n_slice // 2:
        f0, f1 = n_slice // 2, nqf
    else:
        f0, f1 = 0, n_slice // 2
    tabs, ra0, dec0 = [], None, None
    for f in range(f0, f1):
        path = f"{args.QSOfile}{f}-{nqf}.fits"
        if not os.path.exists(path):
            print(f"*Warning* Fits file {path} cannot be read.")
            continue
        hd = fits.read_fits(path)
        if ra0 is None:
            ra0, dec0 = float(hd[1].header["RA0"]), float(hd[1].header["DEC0"])
        tabs.append(hd[1].data)
    if not tabs or sum(len(t) for t in tabs) == 0:
        print("No QSO read. ==> Exit.")
        raise SystemExit(0)
    return np.concatenate(tabs), ra0, dec0


def write_spectra(path, meta, lam, fields, header):
    """METADATA + padded float32 images (bin/make_spectra.py:566-597)."""
    from saclaymocks_gb300 import fits
    n = len(lam)
    maxsize = max((len(x) for x in lam), default=0) if "maxsize" not in header else header.pop("maxsize")

    def padded(rows, fill):
        out = np.full((n, maxsize), fill, np.float32)
        for r, x in enumerate(rows):
            out[r, :len(x)] = x
        return out
    w = fits.FitsWriter(path)
    w.table(meta, header, extname="METADATA")
    w.image(padded(lam, -1.0), extname="LAMBDA")
    for name, rows in fields.items():
        w.image(padded(rows, -1.0 if name == "REDSHIFT" else -2e6), extname=name)
    w.close()


def main_qso(args):
    from saclaymocks_gb300 import fits, los, spectra
    rsd = str2bool(args.rsd)
    if str2bool(args.dla):
        raise SystemExit("make_spectra: -dla True (velocity skewers) is not supported by this drop-in")
    if not 1 <= args.dmax <= 4:
        raise SystemExit("make_spectra: -dmax must be 1..4")
    h = fits.read_header(os.path.join(args.boxdir, "box-0.fits"))
    DX, DY, DZ = float(h["DX"]), float(h["DY"]), float(h["DZ"])
    NZ, NY, nplanes, nHDU = int(h["NAXIS1"]), int(h["NAXIS2"]), int(h["NAXIS3"]), int(h["NX"])
    if nplanes != 1:
        raise SystemExit(f"NX= {nplanes}  != 1  => abort !")
    if args.i >= args.N:
        raise SystemExit(f"iSlice= {args.i} >= NSlice = {args.N} => abort !")
    if nHDU % args.N != 0:
        raise SystemExit(f"{args.N}  slices not divider of nHDU: {nHDU} => abort !")
    LX, LY, LZ = DX * nHDU, DY * NY, DZ * NZ
    ix0 = max(args.i * nHDU // args.N - args.dmax, 0)
    ix1 = min((args.i + 1) * nHDU // args.N + args.dmax, nHDU)
    delta = load_planes(args.boxdir, "box", ix0, ix1)
    eta6 = [load_planes(args.boxdir, f"eta_{c}", ix0, ix1) for c in ETA6] if rsd else None

    cosmo = los.Cosmo()
    grid = los.pixel_grid(cosmo, args.zmin, args.zmax, args.pixel)
    qsos, ra0, dec0 = read_qsos(args, args.N)
    L = los.qso_lines(cosmo, grid, qsos, ra0, dec0, (LX, LY, LZ), DX, nHDU, args.i, args.N,
                      args.zmin, args.zmax, rsd=rsd, nqso_max=args.NQSO)
    n = len(L.npix)
    # the forest pixels [imin, imax) of every line: one Gaussian read for all quasars
    nread = np.maximum(L.imax - L.imin, 0).astype(np.int32)
    rd = np.nonzero(nread > 0)[0]
    corner = np.array([LX / 2 - ix0 * DX, LY / 2, LZ / 2 - grid.R0])   # observer, slab corner frame
    dl_rows = [np.full(int(m), -1e6) for m in L.npix]
    et_rows = [np.zeros(int(m)) for m in L.npix]
    if len(rd):
        R_first = grid.R[L.r0[rd] + L.imin[rd]]
        start = R_first[:, None] * L.unit[rd] + corner[None, :]
        table = spectra.SkewerTable(start, L.unit[rd], nread[rd], dpix=args.pixel, start64=start,
                                    dir64=L.unit[rd])
        cfg = spectra.SpectraConfig(read="gauss343", observer=tuple(corner), dmax=args.dmax)
        r = spectra.SkewerRunner(table, cfg)
        _, dl, et, _ = r.run(delta, None, nx=ix1 - ix0, ny=NY, nz=NZ,
                             pitch=delta.shape[-1], dcell=DX, want_fields=True, eta6=eta6)
        dl, et = spectra.split(dl, table), spectra.split(et, table)
        for k, q in enumerate(rd):
            a, b = int(L.imin[q]), int(L.imin[q]) + int(nread[q])
            dl_rows[q][a:b] = dl[k]
            et_rows[q][a:b] = et[k] if rsd else 0.0
    red = [cosmo.r_2_z(grid.R[L.r0[q]:L.r0[q] + L.npix[q]] / los.H).astype(np.float32) for q in range(n)]
    lam = [grid.lam[L.r0[q]:L.r0[q] + L.npix[q]].astype(np.float32) for q in range(n)]
    cat = qsos[L.qso_index] if n else qsos[:0]
    names = ["RA", "DEC", "Z_noRSD", "Z", "HDU", "THING_ID", "PLATE", "MJD", "FIBERID", "PMF"]
    src = ["RA", "DEC", "Z_QSO_NO_RSD", "Z_QSO_RSD", "HDU", "THING_ID", "PLATE", "MJD", "FIBERID", "PMF"]
    maxsize = max((len(x) for x in lam), default=0)
    header = {"z0": los.Z0, "pixel": args.pixel, "Npixel": len(grid.R), "NX": 1, "dmax": args.dmax,
              "ra0": ra0, "dec0": dec0}
    os.makedirs(args.outDir, exist_ok=True)
    paths = []
    for hdu in np.unique(cat["HDU"]) if n else []:
        m = np.nonzero(cat["HDU"] == hdu)[0]
        meta = {nm: np.asarray(cat[s][m]) for nm, s in zip(names, src)}
        fields = {"DELTA_L": [dl_rows[k].astype(np.float32) for k in m]}
        if rsd:
            fields["ETA_PAR"] = [et_rows[k].astype(np.float32) for k in m]
        fields["REDSHIFT"] = [red[k] for k in m]
        path = os.path.join(args.outDir, f"spectra-{args.i}-{hdu}.fits.gz")
        write_spectra(path, meta, [lam[k] for k in m], fields, dict(header, maxsize=maxsize))
        paths.append(path)
    print(f"{n} QSO written, {int(nread.sum())} forest pixels read")
    return paths


def main_synthetic(args):
    """--synthetic N: the benchmark input (no catalogue), trilinear read of delta and eta_zz."""
    from saclaymocks_gb300 import fits, spectra
    rsd = str2bool(args.rsd)
    h = fits.read_header(os.path.join(args.boxdir, "box-0.fits"))
    nHDU, NY, NZ, dx = int(h["NX"]), int(h["NAXIS2"]), int(h["NAXIS1"]), float(h["DX"])
    delta = load_planes(args.boxdir, "box", 0, nHDU)
    eta = load_planes(args.boxdir, "eta_zz", 0, nHDU) if rsd else None
    table = spectra.skewers_cone(args.synthetic, np.array([nHDU, NY, NZ]) * dx, seed=args.seed,
                                 dpix=args.pixel)
    keep = np.arange(table.n) % args.N == args.i
    table = spectra.SkewerTable(table.start[keep], table.direction[keep], table.npix[keep], dpix=args.pixel)
    ids = np.nonzero(keep)[0]
    cfg = spectra.SpectraConfig(z_lo=args.zmin, z_hi=args.zmax)
    r = spectra.SkewerRunner(table, cfg)
    _, dl, et, z = r.run(delta, eta, nx=nHDU, ny=NY, nz=NZ, pitch=delta.shape[-1], dcell=dx, want_fields=True)
    dl, et, z = (spectra.split(x, table) for x in (dl, et, z))
    n = table.n
    meta = {"RA": np.zeros(n, np.float32), "DEC": np.zeros(n, np.float32),
            "Z_noRSD": np.array([zz.max() for zz in z], np.float32), "Z": np.array([zz.max() for zz in z], np.float32),
            "HDU": np.zeros(n, np.int64), "THING_ID": ids.astype(np.int64), "PLATE": np.zeros(n, np.int64),
            "MJD": np.zeros(n, np.int32), "FIBERID": np.zeros(n, np.int32), "PMF": np.array(["0-0-0"] * n)}
    fields = {"DELTA_L": dl}
    if rsd:
        fields["ETA_PAR"] = et
    fields["REDSHIFT"] = z
    header = {"z0": 0.5 * (args.zmin + args.zmax), "pixel": args.pixel, "Npixel": int(table.npix.max()),
              "NX": 1, "dmax": args.dmax, "ra0": 0.0, "dec0": 0.0}
    os.makedirs(args.outDir, exist_ok=True)
    path = os.path.join(args.outDir, f"spectra-{args.i}-0.fits.gz")
    write_spectra(path, meta, [LYA * (1 + zz) for zz in z], fields, header)
    print(f"{table.n} skewers, {table.total_pixels} pixels -> {path}")
    return [path]


def main(argv=None):
    args = parser().parse_args(argv)
    if args.synthetic > 0:
        return main_synthetic(args)
    if not args.QSOfile:
        raise SystemExit("make_spectra: -QSOfile is required (or --synthetic N for a benchmark input)")
    return main_qso(args)


if __name__ == "__main__":
    main(sys.argv[1:])
