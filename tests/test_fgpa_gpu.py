"""util.fgpa drop-in on the GPU vs the reference's util.fgpa outputs (golden) and a torch
float64 evaluation of the same formula."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def U():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from saclaymocks_gb300 import util
    return util


def test_fgpa_scalar_and_array_params_match_reference(U, golden):
    u = golden("util.npz")
    F1 = U.fgpa(u["delta"], u["eta"], u["G"], 0.1, 1.6, 0.5)
    np.testing.assert_allclose(F1, u["F_scalar"], rtol=0, atol=1e-6)
    F2 = U.fgpa(u["delta"], u["eta"], u["G"], u["a_arr"], u["b_arr"], u["c_arr"])
    np.testing.assert_allclose(F2, u["F_array"], rtol=0, atol=1e-6)


def test_fgpa_torch_path_no_rsd_and_large(U):
    g = torch.Generator(device="cuda").manual_seed(0)
    n = 10_000_019
    d = torch.randn(n, device="cuda", generator=g) * 1.2
    F = U.fgpa(d, None, 0.9, 0.12, 1.5, 0.4)
    ref = torch.exp(-0.12 * torch.exp(1.5 * 0.9 * d.double()))
    assert (F.double() - ref).abs().max().item() < 1e-6
    assert F.dtype == torch.float32 and F.is_cuda


def test_fgpa_mean_flux_known_answer(U):
    """<F> for g ~ N(0,1) with ln a = -5.3199529, b = 5.71883103 is 0.791119
    (bin/param_setting.py:112)."""
    g = torch.Generator(device="cuda").manual_seed(1)
    d = torch.randn(50_000_000, device="cuda", generator=g)
    F = U.fgpa(d, None, 1.0, float(np.exp(-5.3199529)), 5.71883103, 0.0)
    m = F.double().mean().item()
    s = F.double().std().item()
    assert m == pytest.approx(0.791119, abs=4 * 0.36 / np.sqrt(5e7))
    assert s == pytest.approx(0.360234, abs=1e-3)
