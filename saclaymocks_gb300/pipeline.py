"""One mock chunk end to end: the public call a user makes with HOST arrays.

``MockChunk(...).run(start, direction, npix)`` does what the make_boxes -> make_spectra ->
merge_spectra chain of the reference does for one chunk (bin/make_boxes.py main :131-437,
bin/make_spectra.py main :31-606, bin/merge_spectra.py main :16-420): GRF delta and eta_par
boxes, skewer read, small scales, FGPA, and returns the flux of every pixel to the host.
Boxes and all intermediates stay in HBM; only the skewer table goes in and the flux comes
out (pinned host buffers, asynchronous copies on the chunk's stream).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, grf, spectra


class _PendingFlux:
    """Result of MockChunk.run_async: result() waits for that step's flux copy and returns it
    (a view of a pinned host buffer, valid until the call two steps later)."""

    def __init__(self, event, pinned):
        self._event, self._pinned = event, pinned

    def result(self) -> np.ndarray:
        self._event.synchronize()
        return self._pinned.numpy()


class MockChunk:
    def __init__(self, nx, ny, nz, dcell=2.19, *, seed=1, k0=0.02, want_eta=True,
                 cfg: spectra.SpectraConfig | None = None, dpix=0.2, device="cuda", xi_chunk_kz: int = 128,
                 pair: bool = True):
        self.nx, self.ny, self.nz, self.dcell = nx, ny, nz, dcell
        self.pair = pair                   # skewer schedule: pairs of equal FFT length (False: one per item)
        self.xi_chunk_kz = xi_chunk_kz     # grf.make_boxes: blocked x-pass intermediate (0: in place)
        self.seed, self.k0, self.dpix = seed, k0, dpix
        self.cfg = cfg or spectra.SpectraConfig()
        self.device = torch.device(device)
        self.boxes = grf.alloc_boxes(nx, ny, nz, 1, want_eta, self.device)
        self.ws = grf.GrfWorkspace(1, self.device)
        self.amp = grf.pk_normalisation(nx, ny, nz, dcell, k0)
        self.stream = torch.cuda.current_stream(self.device)
        self.copy_stream = torch.cuda.Stream(self.device)
        self._runner = None
        self._key = None
        self._step = 0

    def _prepare(self, start, direction, npix, slot=0):
        """Schedule on the host, pinned staging buffers (two sets, used in turn), device table
        (H2D on the stream)."""
        table = spectra.SkewerTable(start, direction, npix, dpix=self.dpix)
        key = (table.n, table.total_pixels)
        if self._runner is None or self._key != key:
            self._runner = spectra.SkewerRunner(table, self.cfg, device=self.device, pair=self.pair)
            self._pin_in = [[torch.empty(x.shape, dtype=t, pin_memory=True) for x, t in
                             ((table.start, torch.float32), (table.direction, torch.float32),
                              (table.npix, torch.int32), (table.offset, torch.int64))] for _ in range(2)]
            self._pin_order = [torch.empty(self._runner.n_slots, dtype=torch.int32, pin_memory=True)
                               for _ in range(2)]
            self._pin_out = [torch.empty(table.total_pixels, dtype=torch.float32, pin_memory=True)
                             for _ in range(2)]
            self._flux = [torch.empty(table.total_pixels, dtype=torch.float32, device=self.device)
                          for _ in range(2)]
            self._h2d_done = [None, None]
            self._d2h_done = [None, None]
            self._key = key
        r = self._runner
        r.table = table
        order = table.schedule(self.cfg.ss_nz if self.cfg.ss_mode != _lib.SMK_SS_NONE else -1)
        if self._h2d_done[slot] is not None:
            self._h2d_done[slot].synchronize()     # this pinned set's previous copy has run
        pins = self._pin_in[slot]
        for pin, arr in zip(pins, (table.start, table.direction, table.npix, table.offset)):
            pin.numpy()[...] = arr
        self._pin_order[slot].numpy()[...] = order
        for dev, pin in zip((r.d_start, r.d_dir, r.d_npix, r.d_off), pins):
            dev.copy_(pin, non_blocking=True)
        r.d_order.copy_(self._pin_order[slot], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(self.stream)
        self._h2d_done[slot] = ev
        return r

    def h2d_bytes(self) -> int:
        return sum(p.numel() * p.element_size() for p in self._pin_in[0]) + self._pin_order[0].numel() * 4

    def d2h_bytes(self) -> int:
        return self._pin_out[0].numel() * 4

    def run_async(self, start, direction, npix, pass_events=None) -> _PendingFlux:
        """Enqueue one step: boxes, skewer table H2D, skewers, and the flux D2H on a copy
        stream, so that the copy overlaps the next step's boxes.  Steps alternate between two
        sets of buffers; the returned handle's result() waits for this step's flux.  The boxes
        are enqueued first, so the host-side schedule and pinned copies of the skewer table run
        while the GPU draws them."""
        slot = self._step & 1
        out = grf.make_boxes(self.nx, self.ny, self.nz, self.dcell, seed=self.seed, k0=self.k0,
                             amp=self.amp, want_eta=self.boxes[1] is not None, out=self.boxes,
                             workspace=self.ws, pass_events=pass_events, xi_chunk_kz=self.xi_chunk_kz)
        r = self._prepare(start, direction, npix, slot)
        if self._d2h_done[slot] is not None:
            self.stream.wait_event(self._d2h_done[slot])   # the flux buffer's last copy is done
        flux = self._flux[slot]
        r.run(out.delta_pad[0], out.eta_pad[0] if out.eta_pad is not None else None, nx=self.nx,
              ny=self.ny, nz=self.nz, pitch=out.pitch, dcell=self.dcell, flux=flux)
        ready = torch.cuda.Event()
        ready.record(self.stream)
        done = torch.cuda.Event()
        with torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(ready)
            self._pin_out[slot].copy_(flux, non_blocking=True)
            done.record(self.copy_stream)
        flux.record_stream(self.copy_stream)   # kept from reuse until the copy has run
        self._d2h_done[slot] = done
        self._step += 1
        return _PendingFlux(done, self._pin_out[slot])

    def run(self, start, direction, npix, pass_events=None) -> np.ndarray:
        """Flux of every pixel (packed, float32, host) for the host skewer table (a view of a
        pinned buffer, valid until the call two steps later)."""
        return self.run_async(start, direction, npix, pass_events).result()
