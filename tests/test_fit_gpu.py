"""The (a,b,c) fit on the GPU: reductions, loss, adjoint gradient and the Adam fit against the
oracle's FP64 restatement (oracle/fit.py, whose chi2 form is pinned to fit_az.Fitter.chi2)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import fit as ofit      # noqa: E402

FD_H = 1e-2      # relative step of the fourth-order finite-difference comparator


@pytest.fixture(scope="module")
def problem_pair():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from saclaymocks_gb300 import fit
    rng = np.random.RandomState(0)
    lengths = rng.randint(40, 1100, size=64)
    lengths[:6] = lengths[6:12]             # some equal lengths -> paired skewers
    lengths[20] = 2048                      # longest supported: Bluestein M = 4096
    n = int(lengths.sum())
    delta = (rng.normal(0, 1, n)).astype(np.float32)
    eta = (rng.normal(0, 0.4, n)).astype(np.float32)
    G = rng.uniform(0.8, 1.0, n).astype(np.float32)
    z = np.concatenate([np.sort(rng.uniform(1.8, 3.6, 1)) + np.linspace(0, 0.3, L) for L in lengths])
    z = np.clip(z, 1.8, 3.6)
    zedges = np.linspace(1.8, 3.6, 11)
    kedges = np.logspace(np.log10(0.05), np.log10(15.0), 33)
    gp = fit.FitProblem(delta, eta, G, z, lengths, zedges, kedges, 0.2)
    op = ofit.ZBinProblem(delta.astype(np.float64), eta.astype(np.float64), G.astype(np.float64), z,
                          lengths, zedges, kedges, 0.2)
    truth = np.tile([0.1, 1.58, 0.6], (10, 1))
    mz, pk, *_ = op.reductions(op.flux(truth))
    return gp, op, mz, pk


def test_reductions_match_oracle(problem_pair):
    gp, op, _, _ = problem_pair
    theta = np.tile([0.13, 1.4, 0.5], (10, 1)) * np.linspace(0.9, 1.1, 10)[:, None]
    mz, pk, fbar = gp.reductions(theta)
    omz, opk, ofbar, *_ = op.reductions(op.flux(theta))
    np.testing.assert_allclose(mz, omz, rtol=2e-6)
    np.testing.assert_allclose(fbar, ofbar, rtol=2e-6)
    np.testing.assert_allclose(pk, opk, rtol=2e-4)


def test_adjoint_gradient_matches_oracle_and_fd(problem_pair):
    gp, op, mz, pk = problem_pair
    theta = np.tile([0.15, 1.3, 0.4], (10, 1))
    L, g = gp.loss_grad(theta, mz, pk)
    oL, og = op.loss_grad(theta, mz, pk)
    assert L == pytest.approx(oL, rel=1e-4)
    scale = np.abs(og).max()
    np.testing.assert_allclose(g, og, rtol=0, atol=2e-4 * scale)
    gfd = gp.fd_grad(theta, mz, pk, h=1e-3)
    np.testing.assert_allclose(g, gfd, rtol=0, atol=5e-3 * scale)


def test_autograd_function(problem_pair):
    from saclaymocks_gb300 import fit
    gp, op, mz, pk = problem_pair
    th = torch.tensor(np.tile([0.12, 1.5, 0.55], (10, 1)), dtype=torch.float64, requires_grad=True)
    L = fit.FgpaP1DLoss.apply(th, gp, mz, pk)
    L.backward()
    _, og = op.loss_grad(th.detach().numpy(), mz, pk)
    np.testing.assert_allclose(th.grad.numpy(), og, rtol=0, atol=2e-4 * np.abs(og).max())


def test_adjoint_matches_torch_autograd_of_fp64_restatement(problem_pair):
    """The adjoint gradient against torch.autograd through an FP64 torch restatement of the same
    loss (oracle.fit.torch_loss), within the FP32 tolerance 2e-4 max|g|."""
    gp, op, mz, pk = problem_pair
    theta = np.tile([0.14, 1.45, 0.45], (10, 1)) * np.linspace(0.97, 1.03, 10)[:, None]
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    ofit.torch_loss(op, th, mz, pk).backward()
    _, g = gp.loss_grad(theta, mz, pk)
    ref = th.grad.numpy()
    np.testing.assert_allclose(g, ref, rtol=0, atol=2e-4 * np.abs(ref).max())


def test_chirp_table_gives_identical_results(problem_pair):
    """The precomputed chirp spectra (one Bluestein transform saved) give the same forward
    reductions, bit for bit, as the chirps transformed in the kernels, and the same gradient to
    FP32 rounding (the inverse transform takes the conjugate of the forward chirp's spectrum,
    equal to the spectrum of the conjugate chirp up to rounding): 1e-6 max|g|.  Every Bluestein
    length is the smallest 2^a 3^b 5^c >= 2N - 1."""
    import copy
    from saclaymocks_gb300 import _lib
    gp, op, mz, pk = problem_pair
    lib = _lib.load()
    for N in (1, 2, 40, 400, 1024, 1025, 1200, 2048):
        M = lib.smk_fit_bluestein_m(N)
        assert M >= 2 * N - 1 and lib.smk_fft_supported(M)
        assert all(not lib.smk_fft_supported(m) for m in range(max(2, 2 * N - 1), M))
    theta = np.tile([0.15, 1.3, 0.4], (10, 1))
    L1, g1 = gp.loss_grad(theta, mz, pk)
    r1 = gp.reductions(theta)
    gq = copy.copy(gp)
    gq.fp = type(gp.fp).from_buffer_copy(gp.fp)
    gq.without_chirp_table()
    L0, g0 = gq.loss_grad(theta, mz, pk)
    r0 = gq.reductions(theta)
    assert L1 == L0
    np.testing.assert_allclose(g1, g0, rtol=0, atol=1e-6 * np.abs(g0).max())
    for a, b in zip(r1, r0):
        np.testing.assert_array_equal(a, b)


def test_stored_spectra_give_the_recomputed_gradient(problem_pair):
    """The backward that reads the pair spectra stored by the forward pass gives the gradient of
    the backward that transforms every pair again (1e-6 max|g|); after a forward at another
    theta the stored spectra are stale and the backward of the first state transforms again."""
    import copy
    gp, op, mz, pk = problem_pair
    assert gp.spec is not None
    t1 = np.tile([0.15, 1.3, 0.4], (10, 1))
    t2 = np.tile([0.11, 1.6, 0.7], (10, 1))
    L1, g1 = gp.loss_grad(t1, mz, pk)
    nq = copy.copy(gp)
    nq.fp = type(gp.fp).from_buffer_copy(gp.fp)
    nq.without_spectrum_store()
    L0, g0 = nq.loss_grad(t1, mz, pk)
    assert L1 == L0
    np.testing.assert_allclose(g1, g0, rtol=0, atol=1e-6 * np.abs(g0).max())
    _, s1 = gp.forward(t1, mz, pk)
    gp.forward(t2, mz, pk)                 # overwrites the stored spectra
    g_stale = gp.backward(s1)
    np.testing.assert_allclose(g_stale, g0, rtol=0, atol=1e-6 * np.abs(g0).max())


def test_fit_kernels_sized_by_longest_skewer(problem_pair):
    """The kernels' shared memory holds the Bluestein length of SmkFitProblem.n_max; a problem
    that understates it gets NaN power sums and gradient (the too-long pairs are skipped), and
    the next call with the right n_max is correct again."""
    import copy
    gp, op, mz, pk = problem_pair
    theta = np.tile([0.15, 1.3, 0.4], (10, 1))
    _, g_ok = gp.loss_grad(theta, mz, pk)
    bad = copy.copy(gp)
    bad.fp = type(gp.fp).from_buffer_copy(gp.fp)
    bad.fp.n_max = 200                     # lengths go up to 2048
    _, pk_bad, _ = bad.reductions(theta)
    assert np.isnan(pk_bad).any()
    _, g_bad = bad.loss_grad(theta, mz, pk)
    assert np.isnan(g_bad).all()
    _, g_again = gp.loss_grad(theta, mz, pk)
    np.testing.assert_allclose(g_again, g_ok, rtol=0, atol=1e-6 * np.abs(g_ok).max())


def test_adjoint_and_fd_fits_agree(problem_pair):
    """Adam from (0.15, 1.3, 0.4) with adjoint and with finite-difference gradients (fourth-order
    stencil, relative step 1e-2: truncation and the float32 rounding of the loss together keep the
    FD gradient within ~6e-5 of the adjoint one on this problem): same parameters to 5e-4
    relative after the same iterations."""
    from saclaymocks_gb300 import fit
    gp, op, mz, pk = problem_pair
    th0 = np.tile([0.15, 1.3, 0.4], (10, 1))
    ta, la, _, _ = fit.adam_fit(gp, th0, mz, pk, steps=15, lr=0.02, grad="adjoint", eps_rel=1e-2)
    tf, lf, _, _ = fit.adam_fit(gp, th0, mz, pk, steps=15, lr=0.02, grad="fd", h=FD_H, points=4,
                                eps_rel=1e-2)
    assert la[-1] < 0.5 * la[0]
    np.testing.assert_allclose(ta, tf, rtol=5e-4)
