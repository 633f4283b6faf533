"""MockChunk: one chunk end to end from host skewer arrays to host flux (the public call of the
make_boxes -> make_spectra -> merge_spectra chain), synchronous and pipelined."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _chunk_and_table():
    from saclaymocks_gb300 import _lib, pipeline, spectra
    nx, ny, nz, dx = 24, 20, 32, 2.19
    cfg = spectra.SpectraConfig(ss_mode=_lib.SMK_SS_PHILOX, ss_nz=256, pmiss=spectra.pmiss_gauss(0.05, 2.0),
                                seed=5, abc_mode=_lib.SMK_ABC_POWERLAW, a=0.1, a_zref1=3.2, a_power=4.5,
                                b=1.58, c=0.6, z_lo=1.8, z_hi=3.6)
    chunk = pipeline.MockChunk(nx, ny, nz, dx, seed=3, cfg=cfg)
    L = np.array([nx, ny, nz]) * dx
    base = spectra.skewers_cone(64, L, seed=1, npix_range=(40, 120))
    # same skewer count and lengths (the buffers are reused in turn), different start points;
    # then a table of another size (buffers re-made while the earlier copies are in flight)
    tables = [spectra.SkewerTable((base.start + 1.7 * k) % L, base.direction, base.npix, dpix=base.dpix)
              for k in range(3)]
    tables.append(spectra.skewers_cone(40, L, seed=9, npix_range=(30, 90)))
    return chunk, tables


def test_mock_chunk_pipelined_steps_equal_synchronous_runs():
    """run_async keeps two buffer sets in flight; each step's flux equals the synchronous
    run() of the same table, and equals the kernel run directly on the chunk's boxes."""
    from saclaymocks_gb300 import grf
    chunk, tables = _chunk_and_table()
    sync = [chunk.run(t.start, t.direction, t.npix).copy() for t in tables]
    handles = [chunk.run_async(t.start, t.direction, t.npix) for t in tables[:2]]
    got = [handles[0].result().copy()]
    for t in tables[2:]:
        handles.append(chunk.run_async(t.start, t.direction, t.npix))
        got.append(handles[len(got)].result().copy())
    got += [h.result().copy() for h in handles[len(got):]]
    assert len(got) == len(sync)
    for a, b in zip(got, sync):
        np.testing.assert_array_equal(a, b)
    # the same flux from the runner on freshly drawn boxes
    t = tables[1]
    r = chunk._prepare(t.start, t.direction, t.npix)
    out = grf.make_boxes(chunk.nx, chunk.ny, chunk.nz, chunk.dcell, seed=chunk.seed, amp=chunk.amp)
    f = r.run(out.delta_pad[0], out.eta_pad[0], nx=chunk.nx, ny=chunk.ny, nz=chunk.nz, pitch=out.pitch,
              dcell=chunk.dcell)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(f.cpu().numpy(), sync[1])
    assert np.isfinite(sync[0]).all() and (sync[0] > 0).all() and (sync[0] <= 1).all()
