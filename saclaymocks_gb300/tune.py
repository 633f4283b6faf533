"""Autotuner of the GRF passes' tile variants (tile width W, threads per block).

For a box shape, every valid variant of each pass is timed with the per-pass CUDA events of
``smk_grf_boxes`` (all passes of one call use the i-th variant of their own table, so one
sweep of ``max(variants)`` calls times every candidate), the fastest is kept per pass and line
length class, applied through ``smk_tune_set``, and cached in JSON keyed by device name,
pass, and line length class, so later processes replay it without re-timing.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np
import torch

from . import _lib, grf

PASS_NAMES = {_lib.SMK_PASS_ZFWD: "zfwd", _lib.SMK_PASS_LINE: "line", _lib.SMK_PASS_XPASS: "xpass",
              _lib.SMK_PASS_XGEN: "xgen", _lib.SMK_PASS_ZINV: "zinv"}
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "tune_cache.json")


def length_class(n: int) -> int:
    return 0 if n <= 512 else 1 if n <= 1024 else 2 if n <= 2560 else 3


def variants(pass_id: int, n: int) -> list:
    lib = _lib.load()
    out = []
    w, t, nm = C.c_int32(), C.c_int32(), C.c_int32()
    for v in range(lib.smk_tune_count(pass_id)):
        _lib.check(lib.smk_tune_info(pass_id, v, C.byref(w), C.byref(t), C.byref(nm)))
        if nm.value >= n or nm.value == -n:     # n_max < 0: that length only
            out.append((v, w.value, t.value))
    return out


def _device_key() -> str:
    return torch.cuda.get_device_name(torch.cuda.current_device())


def apply(choices: dict):
    """choices: {(pass_id, n): variant} -> smk_tune_set for each."""
    lib = _lib.load()
    for (pid, n), v in choices.items():
        _lib.check(lib.smk_tune_set(int(pid), int(n), int(v)), "smk_tune_set")


def load_cached(shape_passes) -> dict:
    """Apply cached choices for [(pass_id, n), ...]; returns the ones found."""
    try:
        with open(CACHE) as f:
            cache = json.load(f)
    except (OSError, ValueError):
        return {}
    dev = cache.get(_device_key(), {})
    found = {}
    for pid, n in shape_passes:
        key = f"{PASS_NAMES[pid]}:{length_class(n)}"
        if key in dev:
            found[(pid, n)] = int(dev[key])
    apply(found)
    return found


def _store(choices: dict):
    try:
        with open(CACHE) as f:
            cache = json.load(f)
    except (OSError, ValueError):
        cache = {}
    dev = cache.setdefault(_device_key(), {})
    for (pid, n), v in choices.items():
        dev[f"{PASS_NAMES[pid]}:{length_class(n)}"] = int(v)
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    with open(CACHE, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)


def tune_grf(nx: int, ny: int, nz: int, dcell: float = 2.19, gpu_noise: bool = True, reps: int = 2,
             out=None, workspace=None, use_cache: bool = True, xi_chunk_kz: int = 128) -> dict:
    """Pick the fastest tile variant of every pass of smk_grf_boxes for this shape (with the x
    pass in place or, xi_chunk_kz > 0, into the blocked intermediate).
    Returns {"choices": {pass name: (variant, W, T)}, "ms": {pass name: {variant: ms}}}."""
    if gpu_noise:
        passes = [(_lib.SMK_PASS_XGEN, nx, 3), (_lib.SMK_PASS_LINE, ny, 4), (_lib.SMK_PASS_ZINV, nz, 5)]
    else:
        passes = [(_lib.SMK_PASS_ZFWD, nz, 1), (_lib.SMK_PASS_LINE, ny, 2), (_lib.SMK_PASS_XPASS, nx, 3),
                  (_lib.SMK_PASS_ZINV, nz, 5)]
    if use_cache:
        found = load_cached([(p, n) for p, n, _ in passes])
        if len(found) == len(passes):
            return {"choices": {PASS_NAMES[p]: found[(p, n)] for p, n, _ in passes}, "ms": {}, "cached": True}
    cands = {p: variants(p, n) for p, n, _ in passes}
    if out is None:
        out = grf.alloc_boxes(nx, ny, nz)
    if workspace is None:
        workspace = grf.GrfWorkspace(1)
    amp = grf.pk_normalisation(nx, ny, nz, dcell)
    noise = None if gpu_noise else torch.randn(nx * ny * nz, device="cuda").reshape(nx, ny, nz)
    lib = _lib.load()
    # coordinate descent in pass order: the candidates of one pass are timed with the other passes
    # at their current choice (the x pass's tile decides the intermediate's layout that the y
    # pass reads, so passes are not timed independently of each other)
    best = {}
    for p, n, _ in passes:
        _lib.check(lib.smk_tune_set(p, n, -1))
        best[(p, n)] = lib.smk_tune_get(p, n)
    times = {p: {} for p, _, _ in passes}
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    for e in evs:
        e.record()
    for p, n, mark in passes:
        for v, _, _ in cands[p]:
            cur = dict(best)
            cur[(p, n)] = v
            apply(cur)
            acc = []
            for k in range(1 + reps):
                grf.make_boxes(nx, ny, nz, dcell, seed=1, noise=noise, amp=amp, out=out, workspace=workspace,
                               xi_chunk_kz=xi_chunk_kz, pass_events=evs)
                torch.cuda.synchronize()
                if k:                  # the first call of a variant: launch set-up, cold caches
                    acc.append(evs[mark - 1].elapsed_time(evs[mark]))
            times[p][v] = float(np.mean(acc))
        best[(p, n)] = min(times[p], key=times[p].get)
    apply(best)
    _store(best)
    info = {p: {v: (w, t) for v, w, t in cands[p]} for p, _, _ in passes}
    return {"choices": {PASS_NAMES[p]: (best[(p, n)], *info[p][best[(p, n)]]) for p, n, _ in passes},
            "ms": {PASS_NAMES[p]: {int(v): round(m, 3) for v, m in times[p].items()} for p, _, _ in passes},
            "cached": False}


def tune_skewers(table, cfg, boxes, nx: int, ny: int, nz: int, pitch: int, dcell: float, reps: int = 3,
                 blocks=(0, 1, 2, 3), use_cache: bool = True) -> dict:
    """Pick the skewer stage's launch shape for this table: the paired schedule (two skewers of
    one small-scale FFT length per work item) or one skewer per item, and the resident blocks per
    SM of the persistent launch (SMK_TUNE_SKEWER_BLOCKS; 0: as many as fit), by timing
    smk_skewers_flux on `boxes` = (delta_pad, eta_pad).  Applies the block cap and returns
    {"choice": {"pair": bool, "blocks": int}, "ms": {"pair=..,blocks=..": ms}}; the caller builds
    its runner with the chosen schedule."""
    from . import spectra
    key = f"skewers:{int(cfg.ss_nz)}:{int(cfg.ss_mode)}"
    if use_cache:
        try:
            with open(CACHE) as f:
                dev = json.load(f).get(_device_key(), {})
        except (OSError, ValueError):
            dev = {}
        if key in dev:
            code = int(dev[key])
            _lib.tune_flag(_lib.SMK_TUNE_SKEWER_BLOCKS, code >> 1)
            return {"choice": {"pair": bool(code & 1), "blocks": code >> 1}, "ms": {}, "cached": True}
    flux = torch.empty(table.total_pixels, dtype=torch.float32, device="cuda")
    kw = dict(nx=nx, ny=ny, nz=nz, pitch=pitch, dcell=dcell, flux=flux)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    times = {}
    for pair in (True, False):
        runner = spectra.SkewerRunner(table, cfg, pair=pair)
        for b in blocks:
            _lib.tune_flag(_lib.SMK_TUNE_SKEWER_BLOCKS, int(b))
            runner.run(boxes[0], boxes[1], **kw)            # launch set-up
            torch.cuda.synchronize()
            ev[0].record()
            for _ in range(reps):
                runner.run(boxes[0], boxes[1], **kw)
            ev[1].record()
            torch.cuda.synchronize()
            times[(pair, int(b))] = ev[0].elapsed_time(ev[1]) / reps
        del runner
    pair, b = min(times, key=times.get)
    _lib.tune_flag(_lib.SMK_TUNE_SKEWER_BLOCKS, b)
    try:
        with open(CACHE) as f:
            cache = json.load(f)
    except (OSError, ValueError):
        cache = {}
    cache.setdefault(_device_key(), {})[key] = 2 * b + int(pair)
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    with open(CACHE, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    return {"choice": {"pair": pair, "blocks": b},
            "ms": {f"pair={int(p)},blocks={k}": round(t, 3) for (p, k), t in times.items()}, "cached": False}

