"""smk_skewers_flux_static: the allocation-free entry point, for callers that cannot allocate
device memory (its scratch is a static device array inside libsmk).  Called through the C ABI
and compared with smk_skewers_flux on the same inputs, on two calls in a row (the second call
finds the previous call's schedule and counter in the shared array).  Collected last on
purpose; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

F_ATOL = 2e-6   # the flux tolerance of the other skewer tests


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from saclaymocks_gb300 import _lib, build, grf, spectra
    build.build()
    return _lib, grf, spectra


def _call_static(_lib, runner, table, out, nx, ny, nz, flux):
    lib = _lib.load()
    sk, p = runner.structs(nx, ny, nz, out.pitch, out.dcell)
    sk.order = None          # ignored by the static entry point
    sk.n_slots = 0
    rc = lib.smk_skewers_flux_static(C.byref(sk), table.npix.ctypes.data, C.byref(p),
                                     out.delta_pad[0].data_ptr(), out.eta_pad[0].data_ptr(),
                                     flux.data_ptr(), None, None, None,
                                     torch.cuda.current_stream().cuda_stream)
    _lib.check(rc, "smk_skewers_flux_static")


@pytest.mark.parametrize("mode", ["philox", "none"])
def test_static_entry_point_matches_workspace_entry_point(env, mode):
    _lib, grf, spectra = env
    nx, ny, nz, dx = 32, 24, 40, 2.19
    out = grf.make_boxes(nx, ny, nz, dx, seed=5)
    L = np.array([nx, ny, nz]) * dx
    cfg = spectra.SpectraConfig(a=0.1, b=1.58, c=0.6, abc_mode=_lib.SMK_ABC_POWERLAW,
                                ss_mode=_lib.SMK_SS_PHILOX if mode == "philox" else _lib.SMK_SS_NONE,
                                ss_nz=2048, seed=11)
    for call in range(2):
        table = spectra.skewers_cone(300 + 57 * call, L, seed=3 + call, npix_range=(200, 1200))
        runner = spectra.SkewerRunner(table, cfg)
        ref = runner.run(out.delta_pad[0], out.eta_pad[0], nx=nx, ny=ny, nz=nz, pitch=out.pitch,
                         dcell=dx)
        got = torch.full_like(ref, -7.0)
        _call_static(_lib, runner, table, out, nx, ny, nz, got)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=0, atol=F_ATOL)


def test_static_entry_point_rejects_oversized_tables(env):
    _lib, grf, spectra = env
    lib = _lib.load()
    n = (1 << 20)             # more skewers than the static schedule holds
    sk = _lib.SmkSkewers(n=n)
    p = _lib.SmkSpectraParams()
    npix = np.ones(16, np.int32)
    rc = lib.smk_skewers_flux_static(C.byref(sk), npix.ctypes.data, C.byref(p), None, None, None,
                                     None, None, None, None)
    assert rc == _lib.SMK_EINVAL
    assert b"static scratch" in lib.smk_last_error()
