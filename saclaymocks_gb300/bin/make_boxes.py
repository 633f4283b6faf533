"""Drop-in for bin/make_boxes.py: the GRF boxes on the GPU, written as the reference writes
them (bin/make_boxes.py:110-117, 241-431).

    python -m saclaymocks_gb300.bin.make_boxes -NX 256 -pixel 2.19 -seed 0 -outDir out

Reference flags (bin/make_boxes.py:137-148) keep their meaning: -pixel, -NX/-NY/-NZ, -seed,
-rsd, -outDir, -nHDU, -PkDir, -dgrowthfile.  Outputs: box-{i}.fits (one x plane per file);
with a P-grid file in -PkDir holding Pln1..3, boxln_{1,2,3}-{i}.fits (nHDU files); with -rsd
True, eta_{xx,yy,zz,xy,xz,yz}-{i}.fits (one x plane per file) and v{x,y,z}-{i}.fits (nHDU
files, velocity factor H0 * dD/dz(z=0) from the growth-rate table of -dgrowthfile or
$SACLAYMOCKS_BASE/etc/dgrowth.fits).  Without a P-grid file the analytic spectrum
A k/(1+(k/k0)^2)^2 with E[var delta] = 1 is used (no lognormal boxes).  -ncpu is accepted and
ignored.  Extra flags: --noise numpy|gpu (numpy, the default: the reference's MT19937
plane-order draws, bit-identical input; gpu: Fourier modes drawn on the GPU), -k0,
--eta-only-zz (write only the eta_zz box the trilinear skewer read uses), --no-write,
--write-boxk True|False.

Checkpoint (bin/make_boxes.py:206-245, 241-352): every run writes seed_boxk.npy, and with
--write-boxk True also boxk.npy (the unnormalised r2c of the noise, complex64 [NX][NY][NZ/2+1],
computed on the host; the default skips it because the GPU redraws the modes from the seed in
less time than reading them back takes).  A run in an outDir that holds seed_boxk.npy takes
that seed; one that holds only boxk.npy (e.g. from the reference, P0-scaled or not) recovers the
noise from it; either way a box family whose files all exist is skipped.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np
import torch


def str2bool(v: str) -> bool:
    """util.str2bool (py/SaclayMocks/util.py:91-98)."""
    if v.lower() in ("yes", "true", "t", "y", "1"):
        return True
    if v.lower() in ("no", "false", "f", "n", "0"):
        return False
    raise SystemExit("Error: boolean value expected.")


def parser():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("-pixel", type=float, default=2.19)
    p.add_argument("-NX", type=int, default=256)
    p.add_argument("-NY", type=int, default=-1)
    p.add_argument("-NZ", type=int, default=-1)
    p.add_argument("-nHDU", type=int, default=1)
    p.add_argument("-ncpu", type=int, default=2)
    p.add_argument("-PkDir", default=None)
    p.add_argument("-seed", type=int, default=None)
    p.add_argument("-rsd", type=str, default="True")
    p.add_argument("-dgrowthfile", default=None)
    p.add_argument("-outDir", default=".")
    p.add_argument("-k0", type=float, default=0.02)
    p.add_argument("--noise", choices=["numpy", "gpu"], default="numpy")
    p.add_argument("--eta-only-zz", action="store_true")
    p.add_argument("--no-write", action="store_true")
    p.add_argument("--write-boxk", default="False")
    return p


H0 = 100.0   # km/s/(Mpc/h), py/SaclayMocks/constant.py:36


def growth_rate_at_zero(path):
    """dD/dz at z = 0: first row of the growth-rate table (bin/make_boxes.py:310-318)."""
    from saclaymocks_gb300 import fits
    return float(fits.read(path, 1)["dD/dz"][0])


def pgrid_file(pkdir, NX, NY, NZ):
    """Name of the P-grid file the reference reads (bin/make_boxes.py:186-189)."""
    if NX == NY == NZ:
        return os.path.join(pkdir, f"P{NX}.fits")
    return os.path.join(pkdir, f"P{NX}-{NY}-{NZ}.fits")


def write_planes(prefix, box, dcell, sigma, seed, nhdu=None):
    """{prefix}-{i}.fits files, i < nhdu (default NX: one x plane per file), each holding
    planes [i NX/nhdu, (i+1) NX/nhdu) as float32 with keys DX..NZ; sigma and seed on file 0
    (bin/make_boxes.py:110-117)."""
    from saclaymocks_gb300 import fits
    NX, NY, NZ = box.shape
    nhdu = NX if nhdu is None else nhdu
    for i in range(nhdu):
        hdr = {"DX": dcell, "DY": dcell, "DZ": dcell, "NX": NX, "NY": NY, "NZ": NZ}
        if i == 0:
            hdr.update({"SIGMA": float(np.float32(sigma)), "SEED": int(seed)})
        part = box[i * NX // nhdu:(i + 1) * NX // nhdu]
        fits.write_image(f"{prefix}-{i}.fits", np.ascontiguousarray(part), hdr)


def family_done(outdir, prefix, nfiles):
    """True when every file {prefix}-{i}.fits, i < nfiles, exists (the file count the reference
    checks before it skips a box family on a resumed run, bin/make_boxes.py:241-352)."""
    return all(os.path.exists(os.path.join(outdir, f"{prefix}-{i}.fits")) for i in range(nfiles))


def main(argv=None):
    from saclaymocks_gb300 import fits, grf
    args = parser().parse_args(argv)
    NX = args.NX
    NY = NX if args.NY < 0 else args.NY
    NZ = NX if args.NZ < 0 else args.NZ
    rsd = str2bool(args.rsd)
    seed = args.seed if args.seed is not None else int(np.random.randint(2 ** 31 - 1))
    t0 = time.time()
    # checkpoint of a previous run in outDir (bin/make_boxes.py:206-245): the seed of its noise
    # (seed_boxk.npy) or, without it, the Fourier transform of its noise (boxk.npy)
    boxk_file = os.path.join(args.outDir, "boxk.npy")
    seed_file = os.path.join(args.outDir, "seed_boxk.npy")
    resumed = os.path.isfile(boxk_file) or os.path.isfile(seed_file)
    noise_box = None
    if os.path.isfile(seed_file):
        seed = int(np.load(seed_file))
        print(f"{seed_file} found: resuming with seed {seed}")
    elif os.path.isfile(boxk_file):
        if args.noise != "numpy":
            raise SystemExit("make_boxes: resuming from boxk.npy needs --noise numpy")
        boxk = np.load(boxk_file).astype(np.complex128)
        if boxk.shape != (NX, NY, NZ // 2 + 1):
            raise SystemExit(f"make_boxes: {boxk_file} has shape {boxk.shape}, not {(NX, NY, NZ // 2 + 1)}")
        if boxk.std() > 70 * NX:
            # saved after the P0 multiply (:284-287): undo it with the P-grid file
            fn = pgrid_file(args.PkDir, NX, NY, NZ) if args.PkDir else None
            if not fn or not os.path.exists(fn):
                raise SystemExit("make_boxes: boxk.npy holds the P0-scaled modes; the P-grid file of -PkDir "
                                 "is needed to undo the scaling")
            p0 = np.asarray(fits.read(fn, "P0"), np.float64)
            boxk = np.divide(boxk, p0, out=np.zeros_like(boxk), where=p0 != 0)
        noise_box = np.fft.irfftn(boxk, s=(NX, NY, NZ)).astype(np.float32)
        print(f"{boxk_file} found: noise recovered from the saved modes")
    noise = None
    if args.noise == "numpy":
        if noise_box is None:
            rs = np.random.RandomState(seed)        # the plane order of bin/make_boxes.py:46-48
            noise_box = np.zeros((NX, NY, NZ), dtype=np.float32)
            for iz in range(NZ):
                noise_box[:, :, iz] = np.float32(rs.normal(size=[NX, NY]))
        noise = torch.from_numpy(noise_box).cuda()
    if not args.no_write:
        os.makedirs(args.outDir, exist_ok=True)
        np.save(seed_file, np.int64(seed))
        if str2bool(args.write_boxk) and not os.path.isfile(boxk_file):
            if noise_box is None:
                raise SystemExit("make_boxes: --write-boxk True needs --noise numpy (the real-space noise)")
            np.save(boxk_file, np.fft.rfftn(noise_box.astype(np.float64)).astype(np.complex64))
    del noise_box
    grids = {}
    if args.PkDir:
        fn = pgrid_file(args.PkDir, NX, NY, NZ)
        if os.path.exists(fn):
            for ext in ("Pln1", "Pln2", "Pln3", "P0"):
                try:
                    g = fits.read(fn, ext)
                except Exception:
                    continue
                grids[ext] = torch.from_numpy(np.ascontiguousarray(g, dtype=np.float32)).cuda()
    vfac = None
    if rsd and not args.eta_only_zz:
        path = args.dgrowthfile or os.path.expandvars("$SACLAYMOCKS_BASE/etc/dgrowth.fits")
        if not os.path.exists(path):
            raise SystemExit(f"make_boxes: growth-rate table {path} not found (give -dgrowthfile, set "
                             "$SACLAYMOCKS_BASE, or use -rsd False / --eta-only-zz)")
        vfac = H0 * growth_rate_at_zero(path)
    common = dict(seed=seed, noise=noise, k0=args.k0)
    write = not args.no_write
    if write:
        os.makedirs(args.outDir, exist_ok=True)
    outdir = args.outDir

    def emit(prefix, field, nhdu=None):
        if write:
            write_planes(os.path.join(outdir, prefix), field[0], args.pixel, field[1], seed, nhdu)

    def skip(prefix, nfiles):
        if resumed and write and family_done(outdir, prefix, nfiles):
            print(f"{os.path.join(outdir, prefix)} files already exist ! Skiping this step.")
            return True
        return False

    # lognormal boxes: raw modes x Pln grids (bin/make_boxes.py:241-275)
    for i in (1, 2, 3):
        if f"Pln{i}" in grids and not skip(f"boxln_{i}", args.nHDU):
            o = grf.make_boxes(NX, NY, NZ, args.pixel, pk_grid=grids[f"Pln{i}"], want_eta=False, **common)
            o.check()
            emit(f"boxln_{i}", (o.delta[0].cpu().numpy(), o.sigma()[0]), args.nHDU)
    # density and the eta / velocity boxes, one GRF call per output component
    comps = []
    if rsd:
        comps = ["zz"] if args.eta_only_zz else ["xx", "yy", "zz", "xy", "xz", "yz", "vx", "vy", "vz"]
    pk = grids.get("P0")
    out = None
    names = {c: (c if c[0] == "v" else f"eta_{c}") for c in comps}
    box_done = skip("box", NX)
    comps = [c for c in comps if not skip(names[c], args.nHDU if c[0] == "v" else NX)]
    if box_done and not comps:
        print("every box family already exists")
        return None
    for j, c in enumerate(comps or [None]):
        o = grf.make_boxes(NX, NY, NZ, args.pixel, pk_grid=pk, want_eta=c is not None,
                           eta_comp=c or "zz", vel_factor=vfac if c and c[0] == "v" else None, **common)
        o.check()
        if j == 0:
            out = o
            if not box_done:
                emit("box", (o.delta[0].cpu().numpy(), o.sigma()[0]))
        if c is not None:
            emit(names[c], (o.eta[0].cpu().numpy(), o.sigma(1)[0]), args.nHDU if c[0] == "v" else None)
    torch.cuda.synchronize()
    print(f"boxes {NX}x{NY}x{NZ}: {1 + len(comps) + sum(f'Pln{i}' in grids for i in (1, 2, 3))} fields "
          f"in {time.time() - t0:.2f} s, sigma = {out.sigma()[0]:.6f}" + (f", written to {outdir}" if write else ""))
    return out


if __name__ == "__main__":
    main(sys.argv[1:])
