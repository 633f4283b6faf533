"""Drop-in for bin/make_spectra.py: delta_l and eta_par read along skewers through the boxes
of make_boxes, written as spectra-{i}-{hdu}.fits.gz (bin/make_spectra.py:566-597: METADATA,
LAMBDA, DELTA_L, ETA_PAR, REDSHIFT, rows padded with -1 / -2e6).

    python -m saclaymocks_gb300.bin.make_spectra -boxdir out -outDir spec --synthetic 1000 -i 0 -N 1

The reference's lines of sight come from a QSO catalogue and the cosmology (:300-321,
:429-472); here the skewer table is given (--skewers file.npz with start [n,3], dir [n,3],
npix [n], box-corner frame in Mpc/h) or drawn (--synthetic N: start uniform in the box, within
10 deg of +z, 400-1200 pixels).  The read is trilinear (periodic); redshift runs linearly from
-zmin to -zmax along x.  -i/-N keep skewers with index % N == i.  Reference flags -dmax,
-QSOfile, -NQSOfile, -NQSO, -rsd, -dla, -dgrowthfile are accepted; -rsd False drops eta_par.
"""
from __future__ import annotations

import argparse
import glob
import os
import sys

import numpy as np
import torch

from .make_boxes import str2bool

LYA = 1215.67  # py/SaclayMocks/constant.py:12


def parser():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("-dmax", type=int, default=3)
    p.add_argument("-pixel", type=float, default=0.2)
    p.add_argument("-zmin", type=float, default=1.8)
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
    p.add_argument("--skewers", default=None)
    p.add_argument("--synthetic", type=int, default=0)
    p.add_argument("--seed", type=int, default=1)
    return p


def load_box(boxdir, prefix):
    """Stack the one-plane files {prefix}-{i}.fits of make_boxes into a padded float32 box."""
    from saclaymocks_gb300 import fits, grf
    files = glob.glob(os.path.join(boxdir, f"{prefix}-*.fits"))
    n = len(files)
    if n == 0:
        raise SystemExit(f"no {prefix}-*.fits in {boxdir}")
    h = fits.read_header(os.path.join(boxdir, f"{prefix}-0.fits"))
    NY, NZ = int(h["NAXIS2"]), int(h["NAXIS1"])
    pad = torch.zeros((n, NY, grf.pitch_of(NZ)), dtype=torch.float32)
    for i in range(n):
        pad[i, :, :NZ] = torch.from_numpy(np.ascontiguousarray(fits.read(os.path.join(boxdir, f"{prefix}-{i}.fits"))[0]))
    return pad.cuda(), float(h["DX"]), (n, NY, NZ)


def write_spectra(path, ids, lam, fields, header):
    """METADATA + padded float32 images, as bin/make_spectra.py:566-597."""
    from saclaymocks_gb300 import fits
    n = len(ids)
    meta = {"RA": np.zeros(n, np.float32), "DEC": np.zeros(n, np.float32),
            "Z_noRSD": np.array([z.max() for z in fields["REDSHIFT"]], np.float32),
            "Z": np.array([z.max() for z in fields["REDSHIFT"]], np.float32),
            "HDU": np.zeros(n, np.int64), "THING_ID": np.asarray(ids, np.int64),
            "PLATE": np.zeros(n, np.int64), "MJD": np.zeros(n, np.int32),
            "FIBERID": np.zeros(n, np.int32), "PMF": np.array(["0-0-0"] * n)}
    maxsize = max(len(x) for x in lam) if n else 0

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


def main(argv=None):
    from saclaymocks_gb300 import _lib, spectra
    args = parser().parse_args(argv)
    rsd = str2bool(args.rsd)
    delta, dx, (NX, NY, NZ) = load_box(args.boxdir, "box")
    eta = load_box(args.boxdir, "eta_zz")[0] if rsd else None
    if args.skewers:
        d = np.load(args.skewers)
        table = spectra.SkewerTable(d["start"], d["dir"], d["npix"], dpix=args.pixel)
    else:
        table = spectra.skewers_cone(max(args.synthetic, 1), np.array([NX, NY, NZ]) * dx, seed=args.seed,
                                     dpix=args.pixel)
    keep = np.arange(table.n) % args.N == args.i
    table = spectra.SkewerTable(table.start[keep], table.direction[keep], table.npix[keep], dpix=args.pixel)
    ids = np.nonzero(keep)[0]
    cfg = spectra.SpectraConfig(z_lo=args.zmin, z_hi=args.zmax)
    r = spectra.SkewerRunner(table, cfg)
    _, dl, et, z = r.run(delta, eta, nx=NX, ny=NY, nz=NZ, pitch=delta.shape[-1], dcell=dx, want_fields=True)
    dl, et, z = (spectra.split(x, table) for x in (dl, et, z))
    lam = [LYA * (1 + zz) for zz in z]
    fields = {"DELTA_L": dl}
    if rsd:
        fields["ETA_PAR"] = et
    fields["REDSHIFT"] = z
    header = {"z0": 0.5 * (args.zmin + args.zmax), "pixel": args.pixel, "Npixel": int(table.npix.max()),
              "NX": 1, "dmax": args.dmax, "ra0": 0.0, "dec0": 0.0}
    os.makedirs(args.outDir, exist_ok=True)
    path = os.path.join(args.outDir, f"spectra-{args.i}-0.fits.gz")
    write_spectra(path, ids, lam, fields, header)
    print(f"{table.n} skewers, {table.total_pixels} pixels -> {path}")
    return path


if __name__ == "__main__":
    main(sys.argv[1:])
