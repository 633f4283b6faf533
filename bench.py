"""Benchmark of the SaclayMocks hot path on GB300: one production chunk per step.

Step = 2560 x 2560 x 1536 GRF delta + eta_par boxes (white noise -> sqrt(P/Vcell) -> c2r, five
HBM passes) + 2e5 skewer transmissions (start uniform in the box, direction within 10 deg of +z,
400-1200 pixels of 0.2 Mpc/h, trilinear read, P1D_miss = 0.05 exp(-(k/2)^2) on a 2048-point
grid, FGPA a(z) = 0.1((1+z)/3.2)^4.5, b = 1.58, c = 0.6, z = 1.8 -> 3.6 along x).  Noise is drawn
on the GPU (Philox).  Every step reads and writes ~560 GB (boxes of 40 GB >> 129 MB L2), so no
L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--small]

Prints one JSON line.  --impl reference times the CPU restatement of the reference's path on the
host cores (the reference itself does not run there).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GRF cells/s, flux pixels/s, (a,b,c) fit time: adjoint vs finite-diff, 1 GB300"

PRODUCTION = dict(nx=2560, ny=2560, nz=1536, dcell=2.19, n_skewers=200_000, npix=(400, 1200),
                  ss_nz=2048, seed=1)
SMALL = dict(nx=256, ny=256, nz=256, dcell=2.19, n_skewers=2_000, npix=(400, 1200), ss_nz=2048, seed=1)


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(backend="nccl"):
    """Replicas: one process per GPU under torchrun (RANK / WORLD_SIZE from the environment),
    each drawing its own chunk (seed + rank); no data is exchanged, only the timings."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend)
        return dist, rank, world
    return None, 0, 1


def spawn_replicas(n: int, argv: list, timeout: float | None = None) -> int:
    """`python bench.py --gpus N` without a launcher: start N copies of this script, one per
    GPU (LOCAL_RANK = RANK = i, WORLD_SIZE = N, rendezvous on 127.0.0.1), forward rank 0's
    output and return the first non-zero exit status (0 when all succeed)."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__), *argv], env=env,
                                      stdout=None if r == 0 else subprocess.DEVNULL))
    rc = 0
    for p in procs:
        code = p.wait(timeout=timeout)
        rc = rc or code
    return rc


def selftest_replicas(args):
    """Replica bookkeeping without a GPU (gloo): every rank reports a made-up step time, rank 0
    prints the job line (the N > 1 path's barrier / max-over-ranks / aggregate arithmetic)."""
    dist, rank, world = dist_setup("gloo")
    t = [0.5 + 0.25 * rank]
    mx = max_over_ranks(t, dist, device="cpu")[0]
    if rank == 0:
        print(json.dumps({"n_gpus": world, "seeds": [replica_seed(1, r) for r in range(world)], "max_s": mx,
                          "value": aggregate_value(100.0, world, mx), "parallelism": "replicas"}))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of the chunk replica `rank` draws (Philox boxes, skewer table, small scales)."""
    return base_seed + rank


def max_over_ranks(values, dist, device="cuda"):
    """Element-wise maximum of per-rank timings (the slowest replica sets the job's time)."""
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def aggregate_value(per_rank_units: float, world: int, max_seconds: float) -> float:
    """Whole-job throughput: the units all replicas processed over the slowest replica's time."""
    return world * per_rank_units / max_seconds


def cpu_baseline(cfg, sample_div, workers):
    """CPU restatement on a bounded sample: a box with 1/sample_div of the cells per axis
    product (same cell size) and the same number of skewers per cell."""
    import numpy as np
    from oracle import cpu_pipeline, skewers as osk
    from saclaymocks_gb300 import spectra
    f = round(sample_div ** (1 / 3))
    nx, ny, nz = cfg["nx"] // f, cfg["ny"] // f, cfg["nz"] // f
    nz -= nz % 2
    cells = nx * ny * nz
    nsk = max(1, int(cfg["n_skewers"] * cells / (cfg["nx"] * cfg["ny"] * cfg["nz"])))
    t0 = time.perf_counter()
    d, e, tg = cpu_pipeline.grf_cpu(nx, ny, nz, cfg["dcell"], cfg["seed"], workers=workers)
    t_grf = time.perf_counter() - t0
    tb = spectra.skewers_cone(nsk, np.array([nx, ny, nz]) * cfg["dcell"], seed=cfg["seed"],
                              npix_range=cfg["npix"])
    t0 = time.perf_counter()
    F, ts = cpu_pipeline.skewers_cpu(d, e, cfg["dcell"], tb.start, tb.direction, tb.npix, 0.2,
                                     cfg["ss_nz"], osk.pmiss_analytic, cfg["seed"], workers=workers)
    t_sk = time.perf_counter() - t0
    return dict(cells=cells, pixels=tb.total_pixels, t_grf=t_grf, t_sk=t_sk, stages={**tg, **ts},
                sample=f"{nx}x{ny}x{nz} box (1/{f ** 3} of the cells) + {nsk} skewers")


def extrapolate_cpu(rs, cfg):
    """CPU cells/s at the full workload from sample runs: the GRF time scaled by N log2 N (the
    FFT cost), the skewer time by the pixel count (2e5 skewers of the full chunk against the
    sample's), stated in the JSON beside the raw sample rate."""
    import math
    n_full = cfg["nx"] * cfg["ny"] * cfg["nz"]
    px_full = cfg["n_skewers"] * 0.5 * (cfg["npix"][0] + cfg["npix"][1])
    t = 0.0
    for r in rs:
        t += r["t_grf"] * (n_full * math.log2(n_full)) / (r["cells"] * math.log2(r["cells"]))
        t += r["t_sk"] * px_full / r["pixels"]
    t /= len(rs)
    return {"value": n_full / t, "unit": "cells/s", "s_per_step": t,
            "rule": "GRF time x (N log2 N)_full / (N log2 N)_sample + skewer time x pixels_full / pixels_sample"}


def skewer_sector_bytes(table, nx, ny, nz, pitch, dcell, chunk=20_000, device="cuda"):
    """Compulsory DRAM bytes of the trilinear skewer read of one box: 32 B for every distinct
    32-byte sector the 8 corners of the pixels touch, counted on the GPU from the geometry
    (the kernel's cell-centred rule, periodic wrap).  Bookkeeping of the roofline only."""
    import torch
    nsec = (nx * ny * pitch * 4 + 31) // 32
    mark = torch.zeros(nsec, dtype=torch.uint8, device=device)
    st = torch.from_numpy(table.start.astype("float64")).to(device)
    dr = torch.from_numpy(table.direction.astype("float64")).to(device)
    npx = torch.from_numpy(table.npix.astype("int64")).to(device)
    dims = torch.tensor([nx, ny, nz], device=device)
    for a in range(0, table.n, chunk):
        b = min(table.n, a + chunk)
        n = npx[a:b]
        sk = torch.repeat_interleave(torch.arange(b - a, device=device), n)
        first = torch.cumsum(n, 0) - n
        i = torch.arange(int(n.sum()), device=device) - torch.repeat_interleave(first, n)
        p = st[a:b][sk] + (i.double() * table.dpix)[:, None] * dr[a:b][sk]
        c0 = torch.floor(p / dcell - 0.5).long()
        for cx in (0, 1):
            ix = torch.remainder(c0[:, 0] + cx, dims[0])
            for cy in (0, 1):
                iy = torch.remainder(c0[:, 1] + cy, dims[1])
                row = (ix * ny + iy) * pitch
                for cz in (0, 1):
                    iz = torch.remainder(c0[:, 2] + cz, dims[2])
                    mark[((row + iz) * 4) // 32] = 1
    return 32.0 * float(mark.sum().item())


def workload_config(cfg, world):
    """The `config` of both arms' JSON lines (same workload, same keys)."""
    return {"workload": f"production chunk {cfg['nx']}x{cfg['ny']}x{cfg['nz']} delta+eta_par boxes + "
                        f"{cfg['n_skewers']} skewers of {cfg['npix'][0]}-{cfg['npix'][1]} pixels",
            "parallelism": "replicas" if world > 1 else "1 GPU",
            "l2": "inputs larger than L2 (40 GB boxes), no flush needed"}


def run_reference(args, cfg):
    dist, rank, world = dist_setup()
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    for _ in range(max(1, args.warmup)):
        cpu_baseline(cfg, 512, workers)        # warm-up: imports, FFT plans, C oracle build
    vals = []
    for _ in range(args.steps):
        r = cpu_baseline(cfg, 64 if not args.small else 8, workers)
        vals.append(r)
    cells = sum(r["cells"] for r in vals)
    t = sum(r["t_grf"] + r["t_sk"] for r in vals)
    v = cells / t
    out = {"metric": METRIC, "value": v, "unit": "cells/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic",
           "config": workload_config(cfg, args.gpus),
           "flux_pixels_per_s": sum(r["pixels"] for r in vals) / sum(r["t_sk"] for r in vals),
           "cpu_baseline": {"value": v, "unit": "cells/s", "cores": workers, "kind": "port",
                            "sample": vals[0]["sample"]},
           "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "stages_s": vals[0]["stages"], "extrapolated_full_size": extrapolate_cpu(vals, cfg)}
    print(json.dumps(out))


def run_ours(args, cfg):
    import numpy as np
    import torch

    from saclaymocks_gb300 import _lib, grf, pipeline, spectra

    dist, rank, world = dist_setup()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    L = np.array([cfg["nx"], cfg["ny"], cfg["nz"]]) * cfg["dcell"]
    seed = replica_seed(cfg["seed"], rank)
    table = spectra.skewers_cone(cfg["n_skewers"], L, seed=seed, npix_range=cfg["npix"])
    scfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=cfg["ss_nz"],
                                 pmiss=spectra.pmiss_gauss(0.05, 2.0), seed=seed,
                                 abc_mode=_lib.SMK_ABC_POWERLAW, a=0.1, a_zref1=3.2, a_power=4.5,
                                 b=1.58, c=0.6, z_lo=1.8, z_hi=3.6)
    xi = xi_chunk(args, cfg["nz"])
    chunk = pipeline.MockChunk(cfg["nx"], cfg["ny"], cfg["nz"], cfg["dcell"], seed=seed,
                               cfg=scfg, xi_chunk_kz=xi)
    runner = chunk._prepare(table.start, table.direction, table.npix)
    boxes, ws = chunk.boxes, chunk.ws
    tuned = None
    if args.variants:
        tuned = set_variants(args.variants, cfg["nx"], cfg["ny"], cfg["nz"])
    elif not args.no_tune:
        from saclaymocks_gb300 import tune
        tuned = tune.tune_grf(cfg["nx"], cfg["ny"], cfg["nz"], cfg["dcell"], out=boxes, workspace=ws,
                              xi_chunk_kz=xi, use_cache=xi == 0)
        # the skewer stage's schedule (paired or one per item) and blocks per SM, on the boxes
        # the GRF tuning left
        sk_tuned = tune.tune_skewers(table, scfg, (boxes[0][0], boxes[1][0]), cfg["nx"], cfg["ny"], cfg["nz"],
                                     grf.pitch_of(cfg["nz"]), cfg["dcell"], use_cache=False)
        if sk_tuned["choice"]["pair"] != chunk.pair:
            chunk.pair = sk_tuned["choice"]["pair"]
            chunk._runner = None
            runner = chunk._prepare(table.start, table.direction, table.npix)
        tuned = dict(tuned, skewers=sk_tuned)
    nx, ny, nz = cfg["nx"], cfg["ny"], cfg["nz"]
    cells = nx * ny * nz
    pixels = table.total_pixels

    def device_step(ev=None, sk_ev=None):
        out = grf.make_boxes(nx, ny, nz, cfg["dcell"], seed=seed, amp=chunk.amp,
                             out=boxes, workspace=ws, pass_events=ev, xi_chunk_kz=xi)
        if sk_ev:
            sk_ev[0].record()
        runner.run(out.delta_pad[0], out.eta_pad[0], nx=nx, ny=ny, nz=nz, pitch=out.pitch,
                   dcell=cfg["dcell"], flux=chunk._flux[0])
        if sk_ev:
            sk_ev[1].record()
        return out

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        device_step()
    barrier()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(args.steps)]
    skevs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    for e in [x for row in evs for x in row]:
        e.record()                              # materialise the raw event handles
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        barrier()
        t_start.record()
        for k in range(args.steps):
            out = device_step(evs[k], skevs[k])
        t_end.record()
        barrier()
    ms = t_start.elapsed_time(t_end)
    out.check()
    pass_ms = np.mean([[evs[k][i].elapsed_time(evs[k][i + 1]) for i in range(5)]
                       for k in range(args.steps)], axis=0)
    sk_ms = float(np.mean([skevs[k][0].elapsed_time(skevs[k][1]) for k in range(args.steps)]))
    ms = max_over_ranks([ms], dist)[0]

    # e2e: through MockChunk.run_async with host skewer arrays, H2D + D2H inside the timed
    # region; step k's flux copy overlaps step k+1's boxes, every step's flux is waited for
    chunk.run(table.start, table.direction, table.npix)
    barrier()
    t0 = time.perf_counter()
    pending = None
    for _ in range(args.steps):
        h = chunk.run_async(table.start, table.direction, table.npix)
        if pending is not None:
            pending.result()
        pending = h
    pending.result()
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks([e2e_s], dist)[0]

    # host-noise mode (the reference's own noise fed in: z r2c, y forward, x, y inverse, z c2r):
    # the same chunk with a dense device noise box, timed per pass
    host_res = None
    if not args.no_host_noise and rank == 0:
        noise = torch.randn(nx * ny * nz, dtype=torch.float32, device="cuda").view(nx, ny, nz)
        hev = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(3)]
        for e in [x for row in hev for x in row]:
            e.record()                          # materialise the raw event handles
        for k in range(3):
            hout = grf.make_boxes(nx, ny, nz, cfg["dcell"], noise=noise, amp=chunk.amp, out=boxes, workspace=ws,
                                  pass_events=hev[k], xi_chunk_kz=xi)
        torch.cuda.synchronize()
        hout.check()
        hp = np.mean([[hev[k][i].elapsed_time(hev[k][i + 1]) for i in range(5)] for k in (1, 2)], axis=0)
        del noise, hout
        torch.cuda.empty_cache()
        host_res = {"grf_ms": round(float(hp.sum()), 3),
                    "x_pass": "blocked intermediate" if xi else "in place",
                    "pass_ms": dict(zip(["zfwd_r2c", "y_fwd", "x_fwd_scale_inv(x2)", "y_inv(x2)", "zinv_c2r(x2)"],
                                        [round(float(x), 3) for x in hp])),
                    "ms_per_step": round(float(hp.sum()) + sk_ms, 3),
                    "noise": "dense device noise box (torch.randn), 2 timed calls after 1 warm-up"}

    fit_res = None
    if not args.no_fit and rank == 0:
        fit_res = fit_leg(args, runner, out, table, cfg)
    batch_res = None
    if not args.no_batching and rank == 0 and not args.small:
        del runner
        batch_res = batching_leg()
    if rank != 0:
        return
    pitch = boxes[0].shape[-1]
    h2d_bytes, d2h_bytes = chunk.h2d_bytes(), chunk.d2h_bytes()
    prec_res = None
    if not args.no_precision and not args.small:
        # the precision configuration (1536^3, FP32 path vs FP64 restatement) once the
        # production buffers are released
        sec_pre = skewer_sector_bytes(table, nx, ny, nz, pitch, cfg["dcell"])
        del chunk, boxes, ws, out
        torch.cuda.empty_cache()
        prec_res = precision_leg()
    else:
        sec_pre = None
    peak, peak_kind = hbm_peak()
    nzh = nz // 2 + 1
    modes = nx * ny * nzh
    cbytes = 8.0 * modes                   # one half-complex box
    rbytes = 4.0 * cells                   # one real box
    # GPU-noise passes (the two host-noise forward passes do not run): algorithmic bytes =
    # x: write delta_k, eta_k; y: read + write both; z: read both half spectra, write both boxes
    pass_names = ["x_gen", "y_inv(x2)", "zinv_c2r(x2)"]
    pass_ms = pass_ms[2:]
    pass_bytes = [2 * cbytes, 4 * cbytes, 2 * cbytes + 2 * rbytes]
    dom = int(np.argmax(pass_ms))
    achieved = pass_bytes[dom] / (pass_ms[dom] * 1e-3) / 1e9
    # DRAM bytes per unit from ncu captures of the same kernels on boxes with the production
    # line lengths (2560 x 128 x 1536 for the x pass, 128 x 2560 x 1536 for y and z), scaled by
    # the units of this launch: x (xgi_kernel, both fields) 15.84 B per mode, y (compile-time
    # plan variant) 16.92 and z (compile-time plan variant) 16.37 B per mode and field
    traffic = [15.84 * modes, 16.92 * modes * 2, 16.37 * modes * 2][dom] / 1e9
    grf_ms = float(np.sum(pass_ms))
    step_ms = ms / args.steps
    # The x pass is instruction-bound, so its issue-slot roofline is reported beside the HBM one:
    # warp instructions per mode from the same ncu capture (1.4248e9 for 2560x128x769 modes, both
    # fields), scaled by the modes of this launch; peak = SMs x 4 schedulers x the median SM clock
    # sampled during the timed region
    clk_sum = clk.summary()
    sm_hz = float(clk_sum.get("sm_mhz") or 2070.0) * 1e6
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    x_winst = 1.4248e9 / (2560 * 128 * 769) * modes
    issue = {"kernel": "x_gen", "warp_instructions": x_winst,
             "achieved_per_s": x_winst / (pass_ms[0] * 1e-3), "peak_per_s": nsm * 4 * sm_hz,
             "frac": x_winst / (pass_ms[0] * 1e-3) / (nsm * 4 * sm_hz),
             "basis": "ncu smsp__inst_executed.sum per mode and field, scaled; peak SMs x 4 x SM clock"}
    # skewer stage: 4 B of flux per pixel + the distinct 32-byte sectors of delta and eta the
    # trilinear corners touch (Philox small scales: no noise bytes)
    sec = sec_pre if sec_pre is not None else skewer_sector_bytes(table, nx, ny, nz, pitch, cfg["dcell"])
    sk_bytes = 4.0 * pixels + 2.0 * sec
    sk_roof = {"kernel": "skewer_kernel", "algorithmic_bytes": sk_bytes / 1e9,
               "achieved": sk_bytes / (sk_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
               "frac": sk_bytes / (sk_ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
               "box_sector_bytes": sec / 1e9, "naive_upper_bytes": 68.0 * pixels / 1e9,
               "basis": "4 B/pixel flux + distinct 32-B sectors of delta and eta touched by the 8 corners"}
    # the stage is bound by instruction issue, not HBM: its issue-slot roofline from the warp
    # instructions per pixel of an ncu capture of the same kernel (3.1197e9 for the 2e5-skewer
    # production set of 1.5995e8 pixels)
    sk_winst = 3.1197e9 / 1.5995e8 * pixels
    sk_roof["issue"] = {"warp_instructions": sk_winst, "achieved_per_s": sk_winst / (sk_ms * 1e-3),
                        "peak_per_s": nsm * 4 * sm_hz, "frac": sk_winst / (sk_ms * 1e-3) / (nsm * 4 * sm_hz),
                        "basis": "ncu smsp__inst_executed.sum per pixel, scaled; peak SMs x 4 x SM clock"}
    value = aggregate_value(cells, world, step_ms * 1e-3)
    res = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (Philox noise, synthetic skewers)",
           "config": workload_config(cfg, world),
           "pixels_per_step": world * pixels,
           "grf_cells_per_s": world * cells / (grf_ms * 1e-3),
           "flux_pixels_per_s": world * pixels / (sk_ms * 1e-3),
           "pass_ms": dict(zip(pass_names, [round(float(x), 3) for x in pass_ms])),
           "skewer_ms": round(sk_ms, 3),
           "roofline": {"bound": "hbm", "kernel": pass_names[dom], "achieved": achieved, "peak": peak,
                        "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                        "traffic": traffic, "traffic_unit": "GB per pass (ncu, scaled)",
                        "algorithmic_bytes": pass_bytes[dom] / 1e9,
                        "per_pass_frac": {n: round(b / (m * 1e-3) / 1e9 / peak, 3)
                                          for n, b, m in zip(pass_names, pass_bytes, pass_ms)},
                        "issue": issue, "skewer": sk_roof},
           "host_noise": host_res,
           "host_noise_ms_per_step": host_res["ms_per_step"] if host_res else None,
           "e2e": {"value": aggregate_value(cells, world, e2e_s), "unit": "cells/s",
                   "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes,
                   "ms_per_step": e2e_s * 1e3},
           "gpu_launches": args.steps * (grf.grf_launches(nx, ny, nz, xi_chunk_kz=xi) + 1),
           "tile_variants": tuned,
           "clocks": clk_sum,
           "fit": fit_res,
           "batching": batch_res,
           "precision": prec_res}
    if not args.no_cpu:
        workers = os.cpu_count() or 1
        r = cpu_baseline(cfg, 64 if not args.small else 8, workers)
        v = r["cells"] / (r["t_grf"] + r["t_sk"])
        res["cpu_baseline"] = {"value": v, "unit": "cells/s", "cores": workers, "kind": "port",
                               "sample": r["sample"], "stages_s": r["stages"],
                               "extrapolated_full_size": extrapolate_cpu([r], cfg)}
    print(json.dumps(res))


def fit_leg(args, runner, out, table, cfg):
    """The (a,b,c) fit on this chunk's skewers: 10 z bins (1.8-3.6) x (a, b, c), 32 log-k P1D
    bins; targets from theta* = (0.1, 1.58, 0.6); adjoint vs finite-difference gradients, and
    the same Adam fit (from (0.15, 1.3, 0.4)) with both."""
    import numpy as np
    import torch

    from saclaymocks_gb300 import fit
    nx, ny, nz = cfg["nx"], cfg["ny"], cfg["nz"]
    _, dtot, eta, z = runner.run(out.delta_pad[0], out.eta_pad[0], nx=nx, ny=ny, nz=nz, pitch=out.pitch,
                                 dcell=cfg["dcell"], want_fields=True)
    prob = fit.FitProblem(dtot, eta, None, z, table.npix, np.linspace(1.8, 3.6, 11),
                          np.logspace(np.log10(0.05), np.log10(15.0), 33), 0.2)
    del dtot, eta, z
    truth = np.tile([0.1, 1.58, 0.6], (10, 1))
    mz, pk, _ = prob.reductions(truth)
    th0 = np.tile([0.15, 1.3, 0.4], (10, 1))
    prob.loss_grad(th0, mz, pk)                       # warm-up (launch set-up)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        prob.loss_grad(th0, mz, pk)
    t_adj = (time.perf_counter() - t0) / 3
    _, g_adj = prob.loss_grad(th0, mz, pk)
    # the same adjoint with the chirp spectra transformed in the kernels (no table)
    import copy
    nt = copy.copy(prob)
    nt.fp = type(prob.fp).from_buffer_copy(prob.fp)
    nt.without_chirp_table()
    nt.loss_grad(th0, mz, pk)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        nt.loss_grad(th0, mz, pk)
    t_adj_nt = (time.perf_counter() - t0) / 3
    del nt
    # and with the backward transforming every pair again (no stored forward spectra)
    ns = copy.copy(prob)
    ns.fp = type(prob.fp).from_buffer_copy(prob.fp)
    ns.without_spectrum_store()
    ns.loss_grad(th0, mz, pk)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        ns.loss_grad(th0, mz, pk)
    t_adj_ns = (time.perf_counter() - t0) / 3
    del ns
    # finite-difference comparator: central differences, relative step 1e-4, 2 * 30 loss evaluations
    t0 = time.perf_counter()
    g_fd = prob.fd_grad(th0, mz, pk, h=1e-4, points=2)
    t_fd = time.perf_counter() - t0
    rel = np.abs(g_fd - g_adj) / np.abs(g_adj)
    scale = float(np.abs(g_adj).max())
    steps = args.fit_steps
    ta, la, sa, _ = fit.adam_fit(prob, th0, mz, pk, steps=steps, lr=0.02, grad="adjoint", eps_rel=1e-2)
    # algorithmic bytes of one gradient: delta + eta (4 B each) + z bin (2 B) per pixel read by the
    # mean-flux pass, the P1D pass and the adjoint pass (accumulation), plus the pair spectra
    # (N complex per pair of N-pixel skewers: 4 B per pixel) written by the P1D pass and read
    # back by the adjoint pass
    grad_bytes = (3 * 10.0 + 2 * 4.0) * prob.n_total
    res = {"params": "10 z bins x (a,b,c)", "pixels": prob.n_total, "adjoint_s_per_grad": t_adj,
           "adjoint_s_per_grad_without_chirp_table": t_adj_nt,
           "adjoint_s_per_grad_without_spectrum_store": t_adj_ns,
           "adjoint_gbs": grad_bytes / t_adj / 1e9,
           "adjoint_bytes_basis": "10 B/pixel (delta, eta, z bin) x 3 reads + 4 B/pixel spectra written and read",
           "fd": "central differences, relative step 1e-4 (60 loss evaluations per gradient)",
           "fd_s_per_grad": t_fd, "grad_speedup": t_fd / t_adj,
           "grad_rel_diff_median": float(np.median(rel)), "grad_rel_diff_max": float(rel.max()),
           "grad_abs_diff_max_over_max": float(np.abs(g_fd - g_adj).max() / scale),
           "adam_steps": steps, "adjoint_fit_s": sa, "loss_start": la[0], "loss_end": la[-1]}
    # P1D-missing tuning loop (fit_az.Fitter.iterate) on the same skewers: time per iteration
    from saclaymocks_gb300 import tune_p1d
    kmiss = np.arange(0.0, 20.0, 0.01)
    pm = 0.05 * np.exp(-(kmiss / 2.0) ** 2)
    kb = np.logspace(np.log10(0.05), np.log10(15.0), 33)
    k_c = 0.5 * (kb[1:] + kb[:-1])
    tuner = tune_p1d.P1DMissTuner(prob.delta, prob.eta, None, table.npix, 0.1, 1.58, 0.6, kmiss, pm,
                                  np.concatenate([[0.0], k_c, [20.0]]), 0.1 * np.exp(-np.concatenate([[0.0], k_c, [20.0]]) / 3),
                                  kb, ss_nz=2048, seed=3)
    tuner.compute_p1d()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tuner.run(3)
    torch.cuda.synchronize()
    res["p1dmiss_tuning"] = {"iterations": tuner.niter, "s_per_iteration": (time.perf_counter() - t0) / max(tuner.niter, 1),
                             "max_abs_ratio_minus_1": [round(x, 4) for x in tuner.history]}
    del tuner
    if steps * t_fd < 150:
        tf, lf, sf, _ = fit.adam_fit(prob, th0, mz, pk, steps=steps, lr=0.02, grad="fd", h=1e-4, points=2,
                                     eps_rel=1e-2)
        res.update({"fd_fit_s": sf, "fit_speedup": sf / sa,
                    "max_rel_param_diff": float(np.max(np.abs(ta - tf) / np.abs(tf)))})
    return res


def batching_leg(cfg_seed=2):
    """Batched and graph-captured launches: 64 boxes of 128^3 (seeds 100..163) in one batched
    call vs 64 single-box calls (plain and replayed from a CUDA graph); a 1024^3 box pair with
    5e4 skewers of log-uniform length 64..2048 pixels through the persistent paired-skewer
    kernel vs one skewer per work item, and the skewer launch replayed from a CUDA graph."""
    import numpy as np
    import torch

    from saclaymocks_gb300 import _lib, grf, spectra

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    res = {}
    n, B = 128, 64
    amp = grf.pk_normalisation(n, n, n)
    big = grf.alloc_boxes(n, n, n, batch=B)
    wsb = grf.GrfWorkspace(B)
    one = grf.alloc_boxes(n, n, n, batch=1)
    ws1 = grf.GrfWorkspace(1)
    t_batch = timed(lambda: grf.make_boxes(n, n, n, seed=100, batch=B, amp=amp, out=big, workspace=wsb))

    def singles():
        for b in range(B):
            grf.make_boxes(n, n, n, seed=100 + b, amp=amp, out=one, workspace=ws1)
    t_single = timed(singles)
    stream = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    singles()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=stream):
        singles()
    t_graph = timed(g.replay)
    o1 = grf.make_boxes(n, n, n, seed=100 + 37, amp=amp, out=one, workspace=ws1)
    ob = grf.make_boxes(n, n, n, seed=100, batch=B, amp=amp, out=big, workspace=wsb)
    torch.cuda.synchronize()
    same = bool(torch.equal(ob.delta[37], o1.delta[0]) and torch.equal(ob.eta[37], o1.eta[0]))
    cells = B * n ** 3
    res["grf_64x128^3"] = {"batched_ms": t_batch, "single_calls_ms": t_single, "graph_replay_ms": t_graph,
                           "batched_cells_per_s": cells / (t_batch * 1e-3),
                           "batched_member_equals_single_call": same}
    del big, wsb, one, ws1, g, o1, ob
    torch.cuda.empty_cache()

    n = 1024
    L = n * 2.19
    boxes = grf.alloc_boxes(n, n, n)
    ws = grf.GrfWorkspace(1)
    amp = grf.pk_normalisation(n, n, n)
    t_grf = timed(lambda: grf.make_boxes(n, n, n, seed=cfg_seed, amp=amp, out=boxes, workspace=ws), reps=3)
    out = grf.make_boxes(n, n, n, seed=cfg_seed, amp=amp, out=boxes, workspace=ws)
    table = spectra.skewers_cone(50_000, (L, L, L), seed=cfg_seed, npix_range=(64, 2048), log_uniform=True)
    scfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=0, pmiss=spectra.pmiss_gauss(0.05, 2.0),
                                 seed=cfg_seed, abc_mode=_lib.SMK_ABC_POWERLAW, a=0.1, a_zref1=3.2,
                                 a_power=4.5, b=1.58, c=0.6)
    kw = dict(nx=n, ny=n, nz=n, pitch=out.pitch, dcell=2.19)
    paired = spectra.SkewerRunner(table, scfg)
    single = spectra.SkewerRunner(table, scfg, pair=False)
    fp = torch.empty(table.total_pixels, device="cuda")
    fs = torch.empty(table.total_pixels, device="cuda")
    t_pair = timed(lambda: paired.run(out.delta_pad[0], out.eta_pad[0], flux=fp, **kw), reps=10)
    t_one = timed(lambda: single.run(out.delta_pad[0], out.eta_pad[0], flux=fs, **kw), reps=10)
    gs = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gs, stream=stream):
        paired.run(out.delta_pad[0], out.eta_pad[0], flux=fp, **kw)
    t_sgraph = timed(gs.replay, reps=10)
    paired.run(out.delta_pad[0], out.eta_pad[0], flux=fp, **kw)
    single.run(out.delta_pad[0], out.eta_pad[0], flux=fs, **kw)
    torch.cuda.synchronize()
    px = table.total_pixels
    res["grf_1024^3_ms"] = t_grf
    res["skewers_5e4_loguniform_64_2048"] = {
        "pixels": px, "paired_ms": t_pair, "one_per_item_ms": t_one, "graph_replay_ms": t_sgraph,
        "paired_pixels_per_s": px / (t_pair * 1e-3), "paired_speedup": t_one / t_pair,
        "max_abs_flux_diff_paired_vs_single": float((fp - fs).abs().max())}
    return res


def precision_leg(n=1536, seed=3, nsk=100_000, npix=1024, dcell=2.19, k0=0.02, nbins=64, slab=64):
    """FP32 GPU path against an FP64 restatement of the same arithmetic (cuFFT double through
    torch.fft) on the same white noise: delta / eta_zz boxes (relative RMS, max |err| / sigma),
    P(k) of delta in `nbins` linear |k| bins (P32/P64 - 1 per bin), and the flux of `nsk`
    skewers of `npix` pixels (trilinear read, FGPA with a(z) power law, no small scales):
    mean F and the binned P1D of F/<F> - 1.  Host-noise mode, i.e. all five HBM passes."""
    import math

    import numpy as np
    import torch

    from saclaymocks_gb300 import _lib, grf, spectra
    torch.cuda.empty_cache()
    dv = torch.device("cuda")
    f64 = torch.float64
    gen = torch.Generator(device=dv)
    gen.manual_seed(seed)
    noise = torch.randn((n, n, n), generator=gen, device=dv, dtype=torch.float32)
    amp = grf.pk_normalisation(n, n, n, dcell, k0)
    out = grf.make_boxes(n, n, n, dcell, noise=noise, amp=amp, k0=k0)
    torch.cuda.synchronize()
    spec = torch.fft.rfftn(noise.to(f64))
    del noise
    kf = 2.0 * math.pi / dcell
    kx = torch.fft.fftfreq(n, device=dv, dtype=f64).mul_(kf).view(n, 1, 1)
    ky = torch.fft.fftfreq(n, device=dv, dtype=f64).mul_(kf).view(1, n, 1)
    kz = torch.fft.rfftfreq(n, device=dv, dtype=f64).mul_(kf).view(1, 1, -1)
    nzh = n // 2 + 1
    kmax = math.sqrt(3.0) * math.pi / dcell
    wz = torch.full((1, 1, nzh), 2.0, device=dv, dtype=f64)
    wz[..., 0] = 1.0
    if n % 2 == 0:
        wz[..., -1] = 1.0

    def kgrid(i0, i1):
        return kx[i0:i1] ** 2 + ky ** 2 + kz ** 2

    def binned_power(sp):
        num = torch.zeros(nbins, device=dv, dtype=f64)
        cnt = torch.zeros(nbins, device=dv, dtype=f64)
        for i0 in range(0, n, slab):
            k = kgrid(i0, i0 + slab).sqrt_()
            b = (k / kmax * nbins).long().clamp_(0, nbins - 1)
            w = wz.expand_as(k)
            num.index_add_(0, b.flatten(), (sp[i0:i0 + slab].abs() ** 2 * w).flatten())
            cnt.index_add_(0, b.flatten(), w.flatten())
        return num / cnt.clamp(min=1), cnt
    for i0 in range(0, n, slab):
        k = kgrid(i0, i0 + slab).sqrt_()
        spec[i0:i0 + slab] *= (amp * k / (1.0 + (k / k0) ** 2) ** 2 / dcell ** 3).sqrt_()
    p64, cnt = binned_power(spec)
    d64 = torch.fft.irfftn(spec, s=(n, n, n))
    for i0 in range(0, n, slab):
        kk = kgrid(i0, i0 + slab)
        if i0 == 0:
            kk[0, 0, 0] = 1.0
        spec[i0:i0 + slab] *= kz ** 2 / kk
    e64 = torch.fft.irfftn(spec, s=(n, n, n))
    del spec
    torch.cuda.empty_cache()

    def box_err(a32, a64):
        se = sa = 0.0
        mx = 0.0
        for i0 in range(0, n, slab):
            d = a32[i0:i0 + slab].to(f64) - a64[i0:i0 + slab]
            se += float((d * d).sum())
            sa += float((a64[i0:i0 + slab] ** 2).sum())
            mx = max(mx, float(d.abs().max()))
        sig = math.sqrt(sa / n ** 3)
        return {"rel_rms": math.sqrt(se / sa), "max_abs_over_sigma": mx / sig}
    res = {"box": f"{n}^3", "delta": box_err(out.delta[0], d64), "eta_zz": box_err(out.eta[0], e64)}
    sp32 = torch.fft.rfftn(out.delta[0].to(f64))
    p32, _ = binned_power(sp32)
    del sp32
    torch.cuda.empty_cache()
    ok = cnt > 0
    ratio = (p32[ok] / p64[ok] - 1.0).abs()
    res["pk_bins"] = int(ok.sum())
    res["pk_max_rel_diff"] = float(ratio.max())
    res["pk_median_rel_diff"] = float(ratio.median())

    # skewers: GPU kernel on the FP32 boxes vs FP64 trilinear read + FGPA on the FP64 boxes
    L = n * dcell
    table = spectra.skewers_cone(nsk, (L, L, L), seed=seed, npix_range=(npix, npix))
    scfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_NONE, abc_mode=_lib.SMK_ABC_POWERLAW, a=0.1,
                                 a_zref1=3.2, a_power=4.5, b=1.58, c=0.6, z_lo=1.8, z_hi=3.6)
    run = spectra.SkewerRunner(table, scfg)
    F32 = run.run(out.delta_pad[0], out.eta_pad[0], nx=n, ny=n, nz=n, pitch=out.pitch, dcell=dcell)
    st = torch.from_numpy(table.start).to(dv).to(f64)
    di = torch.from_numpy(table.direction).to(dv).to(f64)
    F64 = torch.empty(table.total_pixels, device=dv, dtype=f64)
    # z(x) jumps from z_hi to z_lo where x wraps; pixels within 1e-3 cell of that plane can fall
    # on either side in float32 vs float64, so they are left out of the per-pixel maximum
    edge = torch.zeros(table.total_pixels, device=dv, dtype=torch.bool)
    i = torch.arange(npix, device=dv, dtype=f64) * table.dpix
    dflat, eflat = d64.view(-1), e64.view(-1)
    per = max(1, 20_000_000 // npix)
    for s0 in range(0, nsk, per):
        pos = st[s0:s0 + per, None, :] + i[None, :, None] * di[s0:s0 + per, None, :]
        u = pos / dcell - 0.5
        fl = torch.floor(u)
        fr = u - fl
        c0 = torch.remainder(fl.long(), n)
        c1 = torch.remainder(c0 + 1, n)
        val_d = torch.zeros(pos.shape[:2], device=dv, dtype=f64)
        val_e = torch.zeros_like(val_d)
        for cx in (0, 1):
            wx = fr[..., 0] if cx else 1 - fr[..., 0]
            ix = c1[..., 0] if cx else c0[..., 0]
            for cy in (0, 1):
                wy = fr[..., 1] if cy else 1 - fr[..., 1]
                iy = c1[..., 1] if cy else c0[..., 1]
                for cz in (0, 1):
                    wzz = fr[..., 2] if cz else 1 - fr[..., 2]
                    iz = c1[..., 2] if cz else c0[..., 2]
                    idx = (ix * n + iy) * n + iz
                    w = wx * wy * wzz
                    val_d += w * dflat[idx]
                    val_e += w * eflat[idx]
        xc = torch.remainder(pos[..., 0] / dcell, n)
        edge[s0 * npix:(s0 + per) * npix] = (torch.minimum(xc, n - xc) < 1e-3).flatten()
        z = 1.8 + 1.8 * xc / n
        a = 0.1 * ((1.0 + z) / 3.2) ** 4.5
        F = torch.exp(-a * torch.exp(1.58 * (val_d + 0.6 * val_e)))
        F64[s0 * npix:(s0 + per) * npix] = F.flatten()
    del d64, e64
    F32d = F32.to(f64)
    res["skewers"] = f"{nsk} x {npix} pixels"
    res["flux_max_abs_diff"] = float((F32d - F64).abs()[~edge].max())
    res["flux_pixels_at_x_wrap_excluded"] = int(edge.sum())
    m32, m64 = float(F32d.mean()), float(F64.mean())
    res["mean_flux_rel_diff"] = abs(m32 / m64 - 1.0)
    dF32 = (F32d / m32 - 1.0).view(nsk, npix)
    dF64 = (F64 / m64 - 1.0).view(nsk, npix)
    q32 = (torch.fft.rfft(dF32, dim=1).abs() ** 2).mean(0)
    q64 = (torch.fft.rfft(dF64, dim=1).abs() ** 2).mean(0)
    kk = np.fft.rfftfreq(npix) * 2 * np.pi / table.dpix
    edges = np.logspace(np.log10(kk[1]), np.log10(kk[-1] * 1.0001), 33)
    b = np.searchsorted(edges, kk, side="right") - 1
    rel = []
    q32n, q64n = q32.cpu().numpy(), q64.cpu().numpy()
    for j in range(32):
        sel = b == j
        if sel.any():
            rel.append(abs(q32n[sel].mean() / q64n[sel].mean() - 1.0))
    res["p1d_bins"] = len(rel)
    res["p1d_max_rel_diff"] = float(max(rel))
    return res


def xi_chunk(args, nz):
    """k_z columns per chunk of the x pass's blocked intermediate: --xi-chunk (0: x pass in
    place; -1: one chunk for the whole half spectrum)."""
    v = args.xi_chunk
    return (nz // 2 + 1) if v < 0 else v


def set_variants(spec, nx, ny, nz):
    """--variants xgen=5,line=5,zinv=4: fixed tile variants per GRF pass instead of tuning
    (so a profile replays the tile choice of an earlier tuned run)."""
    from saclaymocks_gb300 import _lib, tune
    ids = {"zfwd": (_lib.SMK_PASS_ZFWD, nz), "line": (_lib.SMK_PASS_LINE, ny), "xpass": (_lib.SMK_PASS_XPASS, nx),
           "xgen": (_lib.SMK_PASS_XGEN, nx), "zinv": (_lib.SMK_PASS_ZINV, nz)}
    choices = {}
    for item in spec.split(","):
        name, v = item.split("=")
        choices[ids[name.strip()]] = int(v)
    tune.apply(choices)
    return {"fixed": spec}


def run_grf_only(args, shape):
    """GRF boxes of one shape, Philox noise (or, --host-noise, a dense device noise box through
    the five-pass path), W + K calls (the ncu profiling case)."""
    import numpy as np
    import torch

    from saclaymocks_gb300 import grf
    nx, ny, nz = shape
    want_eta = not args.no_eta
    host_noise = getattr(args, "host_noise", False)
    noise = torch.randn(nx * ny * nz, device="cuda").reshape(nx, ny, nz) if host_noise else None
    if args.xgen_split is not None:
        from saclaymocks_gb300 import _lib
        _lib.xgen_split(args.xgen_split)
    if args.no_prefetch:
        from saclaymocks_gb300 import _lib
        _lib.tune_flag(_lib.SMK_TUNE_PREFETCH, 0)
    boxes = grf.alloc_boxes(nx, ny, nz, want_eta=want_eta)
    ws = grf.GrfWorkspace(1)
    amp = grf.pk_normalisation(nx, ny, nz)
    tuned = None
    if args.variants:
        tuned = set_variants(args.variants, nx, ny, nz)
    elif not args.no_tune:
        from saclaymocks_gb300 import tune
        tuned = tune.tune_grf(nx, ny, nz, gpu_noise=not host_noise, out=boxes, workspace=ws, use_cache=False,
                              xi_chunk_kz=xi_chunk(args, nz))
    xi = xi_chunk(args, nz)
    for _ in range(args.warmup):
        grf.make_boxes(nx, ny, nz, seed=1, noise=noise, amp=amp, out=boxes, workspace=ws, want_eta=want_eta,
                       xi_chunk_kz=xi)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(args.steps)]
    for e in [x for row in evs for x in row]:
        e.record()
    torch.cuda.synchronize()
    for k in range(args.steps):
        out = grf.make_boxes(nx, ny, nz, seed=1, noise=noise, amp=amp, out=boxes, workspace=ws, pass_events=evs[k],
                             want_eta=want_eta, xi_chunk_kz=xi)
    torch.cuda.synchronize()
    out.check()
    pass_ms = np.mean([[evs[k][i].elapsed_time(evs[k][i + 1]) for i in range(5)]
                       for k in range(args.steps)], axis=0)
    print(json.dumps({"grf_shape": shape, "noise": "host" if host_noise else "gpu", "xi_chunk_kz": xi,
                      "pass_ms": [round(float(x), 4) for x in pass_ms], "tuned": tuned,
                      "grf_cells_per_s": nx * ny * nz / (pass_ms.sum() * 1e-3)}))


def run_skewers_only(args, spec):
    """The skewer stage alone (the ncu profiling case): GPU-noise boxes of NX,NY,NZ, NSK skewers
    of the production chunk's kind (400-1200 pixels within 10 deg of +z, Philox small scales on
    2048 points, a(z) power law), W + K launches timed with CUDA events."""
    import numpy as np
    import torch

    from saclaymocks_gb300 import _lib, grf, spectra
    nx, ny, nz, nsk = spec
    out = grf.make_boxes(nx, ny, nz, seed=1)
    table = spectra.skewers_cone(nsk, np.array([nx, ny, nz]) * 2.19, seed=1, npix_range=(400, 1200))
    scfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=2048, pmiss=spectra.pmiss_gauss(0.05, 2.0),
                                 seed=1, abc_mode=_lib.SMK_ABC_POWERLAW, a=0.1, a_zref1=3.2, a_power=4.5,
                                 b=1.58, c=0.6, z_lo=1.8, z_hi=3.6)
    r = spectra.SkewerRunner(table, scfg)
    flux = torch.empty(table.total_pixels, dtype=torch.float32, device="cuda")

    def step():
        r.run(out.delta_pad[0], out.eta_pad[0], nx=nx, ny=ny, nz=nz, pitch=out.pitch, dcell=2.19, flux=flux)
    for _ in range(args.warmup):
        step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    print(json.dumps({"skewer_shape": list(spec), "pixels": table.total_pixels, "ms": ms,
                      "pixels_per_s": table.total_pixels / (ms * 1e-3)}))


def run_fit_only(args, nsk):
    """The fit kernels alone (the ncu profiling case): NSK skewers of 400-1200 pixels with
    Gaussian fields, redshift rising along each skewer (3e-4 per pixel from a uniform start in
    1.8-3.4, as on a line of sight), 10 z bins x (a, b, c), 32 log-k bins; W + K
    loss-and-gradient evaluations."""
    import numpy as np
    import torch

    from saclaymocks_gb300 import fit
    rng = np.random.RandomState(0)
    lengths = rng.randint(400, 1201, nsk).astype(np.int32)
    n = int(lengths.sum())
    delta = torch.randn(n, device="cuda") * 1.2
    eta = torch.randn(n, device="cuda") * 0.4
    z0 = rng.uniform(1.8, 3.4, nsk)
    first = np.concatenate([[0], np.cumsum(lengths[:-1], dtype=np.int64)])
    idx = np.arange(n) - np.repeat(first, lengths)
    z = torch.from_numpy(np.minimum(np.repeat(z0, lengths) + 3e-4 * idx, 3.6)).cuda()
    prob = fit.FitProblem(delta, eta, None, z, lengths, np.linspace(1.8, 3.6, 11),
                          np.logspace(np.log10(0.05), np.log10(15.0), 33), 0.2)
    truth = np.tile([0.1, 1.58, 0.6], (10, 1))
    mz, pk, _ = prob.reductions(truth)
    th0 = np.tile([0.15, 1.3, 0.4], (10, 1))
    for _ in range(args.warmup):
        prob.loss_grad(th0, mz, pk)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        prob.loss_grad(th0, mz, pk)
    torch.cuda.synchronize()
    s = (time.perf_counter() - t0) / args.steps
    print(json.dumps({"fit_case": nsk, "pixels": n, "s_per_grad": s}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="256^3 box + 2000 skewers (quick check)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tune", action="store_true", help="built-in tile variants, no autotuning")
    ap.add_argument("--no-batching", action="store_true", help="skip the batched / graph-replay leg")
    ap.add_argument("--no-eta", action="store_true", help="--grf-shape: delta box only")
    ap.add_argument("--no-prefetch", action="store_true", help="--grf-shape: no L2 prefetch of the next tile")
    ap.add_argument("--xgen-split", type=int, default=None, choices=[-1, 0, 1],
                    help="--grf-shape: x pass as one launch (0), two one-field launches (1), by footprint (-1)")
    ap.add_argument("--precision", default=None, const="1536,100000,1024", nargs="?",
                    help="only the FP32-vs-FP64 precision report: N,skewers,pixels (default 1536^3, 1e5 x 1024)")
    ap.add_argument("--variants", default=None,
                    help="fixed tile variants, e.g. xgen=5,line=5,zinv=4 (no autotuning)")
    ap.add_argument("--xi-chunk", type=int, default=-1,
                    help="GPU-noise x pass into a blocked intermediate, this many k_z columns per chunk "
                         "(0: in place, -1: one chunk)")
    ap.add_argument("--no-precision", action="store_true", help="skip the 1536^3 FP32-vs-FP64 precision leg")
    ap.add_argument("--no-fit", action="store_true", help="skip the (a,b,c) fit leg")
    ap.add_argument("--no-host-noise", action="store_true", help="skip the host-noise (5-pass) GRF leg")
    ap.add_argument("--fit-steps", type=int, default=20, help="Adam steps of the fit leg")
    ap.add_argument("--fit-case", type=int, default=0,
                    help="NSK: time only the fit's loss + gradient on NSK random skewers (profiling case)")
    ap.add_argument("--skewer-shape", default=None,
                    help="NX,NY,NZ,NSK: time only the skewer stage on boxes of this shape (profiling case)")
    ap.add_argument("--grf-shape", default=None,
                    help="NX,NY,NZ: time only the GRF boxes of this shape (profiling case)")
    ap.add_argument("--host-noise", action="store_true",
                    help="--grf-shape: the five-pass path on a dense device noise box")
    ap.add_argument("--selftest-replicas", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # no launcher: one replica process per GPU, rank 0 prints the job's line
        sys.exit(spawn_replicas(args.gpus, sys.argv[1:]))
    if args.selftest_replicas:
        selftest_replicas(args)
        return
    cfg = SMALL if args.small else PRODUCTION
    if args.grf_shape:
        run_grf_only(args, [int(x) for x in args.grf_shape.split(",")])
        return
    if args.fit_case:
        run_fit_only(args, args.fit_case)
        return
    if args.skewer_shape:
        run_skewers_only(args, [int(x) for x in args.skewer_shape.split(",")])
        return
    if args.precision:
        n, nsk, npix = (int(x) for x in args.precision.split(","))
        print(json.dumps({"precision": precision_leg(n=n, nsk=nsk, npix=npix)}))
        return
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
