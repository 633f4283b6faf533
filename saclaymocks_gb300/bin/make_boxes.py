"""Drop-in for bin/make_boxes.py: GRF delta and eta_zz boxes on the GPU, written as the
reference writes them (one x-plane per FITS file, bin/make_boxes.py:110-117).

    python -m saclaymocks_gb300.bin.make_boxes -NX 256 -pixel 2.19 -seed 0 -outDir out

Reference flags (bin/make_boxes.py:137-148) keep their meaning: -pixel, -NX/-NY/-NZ, -seed,
-rsd (eta_zz box when True), -outDir, -PkDir (if it holds the P-grid file of interpolate_pk,
P0 = sqrt(P/Vcell) is read from it; otherwise the analytic spectrum A k/(1+(k/k0)^2)^2 with
E[var delta] = 1 is used); -nHDU, -ncpu and -dgrowthfile are accepted and ignored (no
lognormal or velocity boxes on this path).  Extra flags: --noise numpy|gpu (numpy: the
reference's MT19937 plane-order draws, bit-identical input; gpu: Fourier modes drawn on the
GPU), -k0, --no-write.
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
    p.add_argument("--noise", choices=["numpy", "gpu"], default="gpu")
    p.add_argument("--no-write", action="store_true")
    return p


def pgrid_file(pkdir, NX, NY, NZ):
    """Name of the P-grid file the reference reads (bin/make_boxes.py:186-189)."""
    if NX == NY == NZ:
        return os.path.join(pkdir, f"P{NX}.fits")
    return os.path.join(pkdir, f"P{NX}-{NY}-{NZ}.fits")


def write_planes(prefix, box, dcell, sigma, seed):
    """box-{i}.fits files: float32 [1, NY, NZ] per x plane, keys DX..NZ; sigma and seed on
    file 0 (bin/make_boxes.py:110-117)."""
    from saclaymocks_gb300 import fits
    NX, NY, NZ = box.shape
    for i in range(NX):
        hdr = {"DX": dcell, "DY": dcell, "DZ": dcell, "NX": NX, "NY": NY, "NZ": NZ}
        if i == 0:
            hdr.update({"SIGMA": float(np.float32(sigma)), "SEED": int(seed)})
        fits.write_image(f"{prefix}-{i}.fits", np.ascontiguousarray(box[i:i + 1]), hdr)


def main(argv=None):
    from saclaymocks_gb300 import fits, grf
    args = parser().parse_args(argv)
    NX = args.NX
    NY = NX if args.NY < 0 else args.NY
    NZ = NX if args.NZ < 0 else args.NZ
    rsd = str2bool(args.rsd)
    seed = args.seed if args.seed is not None else int(np.random.randint(2 ** 31 - 1))
    t0 = time.time()
    noise = None
    if args.noise == "numpy":
        rs = np.random.RandomState(seed)        # the plane order of bin/make_boxes.py:46-48
        box = np.zeros((NX, NY, NZ), dtype=np.float32)
        for iz in range(NZ):
            box[:, :, iz] = np.float32(rs.normal(size=[NX, NY]))
        noise = torch.from_numpy(box).cuda()
        del box
    pk = None
    if args.PkDir:
        fn = pgrid_file(args.PkDir, NX, NY, NZ)
        if os.path.exists(fn):
            pk = torch.from_numpy(np.ascontiguousarray(fits.read(fn, "P0"), dtype=np.float32)).cuda()
    out = grf.make_boxes(NX, NY, NZ, args.pixel, seed=seed, noise=noise, k0=args.k0, pk_grid=pk,
                         want_eta=rsd)
    out.check()
    sig = out.sigma()[0]
    torch.cuda.synchronize()
    print(f"boxes {NX}x{NY}x{NZ} drawn on the GPU in {time.time() - t0:.3f} s, sigma = {sig:.6f}")
    if not args.no_write:
        os.makedirs(args.outDir, exist_ok=True)
        write_planes(os.path.join(args.outDir, "box"), out.delta[0].cpu().numpy(), args.pixel, sig, seed)
        if rsd:
            write_planes(os.path.join(args.outDir, "eta_zz"), out.eta[0].cpu().numpy(), args.pixel,
                         out.sigma(1)[0], seed)
        print(f"written to {args.outDir} in {time.time() - t0:.1f} s")
    return out


if __name__ == "__main__":
    main(sys.argv[1:])
