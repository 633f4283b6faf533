"""FP32 GPU path against an FP64 restatement of the same arithmetic on the same noise
(bench.precision_leg at a small size; bench.py --precision runs it at 1536^3 with 1e5 x 1024
skewers).  Bounds: box relative RMS 2e-6, max |err| 2e-5 sigma, binned P(k) 2e-5, flux 3e-6,
mean flux 1e-6, binned P1D of F/<F>-1 1e-4."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_fp32_path_vs_fp64_small():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bench
    r = bench.precision_leg(n=96, nsk=400, npix=256, nbins=24, slab=32)
    for f in ("delta", "eta_zz"):
        assert r[f]["rel_rms"] < 2e-6, r
        assert r[f]["max_abs_over_sigma"] < 2e-5, r
    assert r["pk_max_rel_diff"] < 2e-5, r
    assert r["flux_max_abs_diff"] < 3e-6, r
    assert r["mean_flux_rel_diff"] < 1e-6, r
    assert r["p1d_max_rel_diff"] < 1e-4, r
