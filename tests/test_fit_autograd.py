"""The fit loss restated with torch operations in FP64 and differentiated by torch.autograd:
its value and gradient equal the oracle's hand-written loss and gradient, and FP64 central
differences with relative step h = 1e-4 agree with both.  CPU only (the GPU adjoint is checked
against the same autograd gradient in test_fit_gpu.py)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import fit as ofit     # noqa: E402


def _problem(seed=0, nsk=24):
    rng = np.random.RandomState(seed)
    lengths = rng.randint(200, 1100, size=nsk)
    lengths[:4] = lengths[4:8]
    lengths[10] = 2048                      # fills the lowest k bins
    n = int(lengths.sum())
    z = np.concatenate([rng.uniform(1.8, 3.2) + np.linspace(0, 0.4, L) for L in lengths]).clip(1.8, 3.6)
    op = ofit.ZBinProblem(rng.normal(0, 1, n), rng.normal(0, 0.4, n), rng.uniform(0.8, 1.0, n), z, lengths,
                          np.linspace(1.8, 3.6, 11), np.logspace(np.log10(0.05), np.log10(15.0), 33), 0.2)
    truth = np.tile([0.1, 1.58, 0.6], (10, 1))
    mz, pk, *_ = op.reductions(op.flux(truth))
    return op, mz, pk


def test_autograd_gradient_equals_hand_written_and_central_differences():
    op, mz, pk = _problem()
    theta = np.tile([0.15, 1.3, 0.4], (10, 1)) * np.linspace(0.95, 1.05, 10)[:, None]
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    L = ofit.torch_loss(op, th, mz, pk)
    L.backward()
    oL, og = op.loss_grad(theta, mz, pk)
    assert float(L) == pytest.approx(oL, rel=1e-12)
    np.testing.assert_allclose(th.grad.numpy(), og, rtol=1e-9, atol=1e-12 * np.abs(og).max())
    fd = op.fd_grad(theta, mz, pk, h=1e-4)
    np.testing.assert_allclose(fd, og, rtol=0, atol=5e-6 * np.abs(og).max())   # O(h^2) truncation
