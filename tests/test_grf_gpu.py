"""GRF boxes (make_boxes) on the GPU through the C ABI, against the reference's own output
(golden boxes from bin/make_boxes.py) and the FP64 oracle.

Tolerance (FP32 FFT path vs the FP64 oracle of the same noise): relative RMS <= 1e-6 and
max |error| <= 1e-5 * sigma_delta, per field.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import grf as ograf          # noqa: E402
from oracle import philox as ophilox     # noqa: E402

REL_RMS = 1e-6
MAX_ABS_SIGMA = 1e-5


@pytest.fixture(scope="module")
def G():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from saclaymocks_gb300 import grf
    return grf


def _err(gpu, ref):
    d = gpu.astype(np.float64) - ref.astype(np.float64)
    sig = np.std(ref)
    return np.sqrt((d ** 2).mean() / (ref.astype(np.float64) ** 2).mean()), np.abs(d).max() / sig


def _check(gpu, ref, tag):
    rr, ma = _err(gpu, ref)
    assert rr <= REL_RMS, f"{tag}: relative RMS {rr:.3e}"
    assert ma <= MAX_ABS_SIGMA, f"{tag}: max abs / sigma {ma:.3e}"


@pytest.mark.parametrize("shape", [(40, 24, 36), (45, 18, 50), (64, 20, 12), (30, 6, 160)])
def test_xgen_one_launch_equals_split_launches(G, shape):
    """The GPU-noise x pass writing delta and eta in one launch (each mode drawn once) gives
    the same boxes, bit for bit, as two one-field launches; also for odd nx, k_z extents that
    end inside a tile, batches and a velocity component."""
    from saclaymocks_gb300 import _lib
    nx, ny, nz = shape
    ps = _lib.xgen_split(1)
    try:
        ref = G.make_boxes(nx, ny, nz, 2.19, seed=23, batch=2, xi_chunk_kz=0)
        refv = G.make_boxes(nx, ny, nz, 2.19, seed=24, eta_comp="vy", vel_factor=100.0, xi_chunk_kz=0)
        _lib.xgen_split(0)
        got = G.make_boxes(nx, ny, nz, 2.19, seed=23, batch=2, xi_chunk_kz=0)
        gotv = G.make_boxes(nx, ny, nz, 2.19, seed=24, eta_comp="vy", vel_factor=100.0, xi_chunk_kz=0)
        torch.cuda.synchronize()
    finally:
        _lib.xgen_split(ps)
    assert torch.equal(got.delta, ref.delta)
    assert torch.equal(got.eta, ref.eta)
    assert torch.equal(gotv.eta, refv.eta)
    np.testing.assert_array_equal(got.sigma(), ref.sigma())


@pytest.mark.parametrize("shape", [(40, 24, 36), (45, 18, 50), (64, 20, 12), (30, 6, 160), (24, 2560, 40),
                                   (6, 1536, 96)])
@pytest.mark.parametrize("chunk", [16, 4096])
def test_blocked_intermediate_x_pass_equals_in_place(G, shape, chunk):
    """The x pass into the blocked intermediate (each mode drawn once, the y pass reading
    contiguous runs), in one chunk or several, gives the same boxes, bit for bit, as the x pass
    in place, with GPU noise and with host noise: both fields, a batch, delta alone, a velocity
    component, odd nx, k_z extents that end inside a block, y lines loaded by TMA (2560, 1536)
    and by cp.async."""
    nx, ny, nz = shape
    noise = torch.from_numpy(np.random.RandomState(6).normal(size=(nx, ny, nz)).astype(np.float32)).cuda()
    for kw in (dict(batch=2), dict(want_eta=False), dict(eta_comp="vz", vel_factor=90.0), dict(noise=noise),
               dict(noise=noise, want_eta=False), dict(noise=noise, eta_comp="xy")):
        ref = G.make_boxes(nx, ny, nz, 2.19, seed=37, xi_chunk_kz=0, **kw)
        got = G.make_boxes(nx, ny, nz, 2.19, seed=37, xi_chunk_kz=chunk, **kw)
        torch.cuda.synchronize()
        assert torch.equal(got.delta, ref.delta), kw
        if ref.eta is not None:
            assert torch.equal(got.eta, ref.eta), kw
        np.testing.assert_array_equal(got.sigma(), ref.sigma())


def test_blocked_intermediate_every_tile_variant_is_exact(G):
    """Every x-pass tile variant run into the intermediate matches the FP64 oracle."""
    import ctypes as C
    from saclaymocks_gb300 import _lib, tune
    lib = _lib.load()
    pid = _lib.SMK_PASS_XGEN
    for v, w, t, n in _all_variants(pid):
        nx, ny, nz = n, 8, 72
        _lib.check(lib.smk_tune_set(pid, nx, v))
        try:
            out = G.make_boxes(nx, ny, nz, 2.19, seed=19, xi_chunk_kz=32)
            torch.cuda.synchronize()
        finally:
            lib.smk_tune_set(pid, nx, -1)
        nk = ophilox.kspace_noise(nx, ny, nz, 19)
        o64 = ograf.grf_from_modes(nk, nz, 2.19, 0.02, eta=("zz",), precision="f64")
        _check(out.delta[0].cpu().numpy(), o64["delta"], f"xgi variant {v} (W={w}, T={t})")
        _check(out.eta[0].cpu().numpy(), o64["eta_zz"], f"xgi variant {v} eta")


@pytest.mark.parametrize("shape", [(24, 2560, 40), (6, 1536, 96), (10, 600, 72), (8, 45, 24)])
def test_y_pass_tma_loads_equal_cp_async(G, shape):
    """The y pass loading its tiles with TMA tensor copies gives the same boxes, bit for bit, as
    the cp.async loads (GPU noise and host noise; y lengths with 256-, 200- and 45-row boxes)."""
    from saclaymocks_gb300 import _lib
    nx, ny, nz = shape
    noise = torch.from_numpy(np.random.RandomState(4).normal(size=(nx, ny, nz)).astype(np.float32)).cuda()
    prev = _lib.tune_flag(_lib.SMK_TUNE_TMA, 0)
    try:
        ref = G.make_boxes(nx, ny, nz, 2.19, seed=41, batch=2)
        refh = G.make_boxes(nx, ny, nz, 2.19, noise=noise)
        for mode in (1, 2):   # TMA loads; TMA loads and TMA tensor stores
            _lib.tune_flag(_lib.SMK_TUNE_TMA, mode)
            got = G.make_boxes(nx, ny, nz, 2.19, seed=41, batch=2)
            goth = G.make_boxes(nx, ny, nz, 2.19, noise=noise)
            torch.cuda.synchronize()
            assert torch.equal(got.delta, ref.delta)
            assert torch.equal(got.eta, ref.eta)
            assert torch.equal(goth.delta, refh.delta)
            assert torch.equal(goth.eta, refh.eta)
    finally:
        _lib.tune_flag(_lib.SMK_TUNE_TMA, prev)


@pytest.mark.parametrize("shape", [(8, 512, 16), (4, 2560, 8)])
def test_y_pass_tma_wait_running_out_is_reported(G, shape):
    """A y-pass TMA wait that runs out (the barrier made to expect more bytes than its copies
    bring) ends within its limit, leaves NaN that the box check reports as SMK_ENULLBOX, and
    the next call on the same context is correct again; at y = 2560 the tile load is split in
    two halves (the first stage starts on the first) and the first half's wait runs out."""
    from saclaymocks_gb300 import _lib
    from saclaymocks_gb300._lib import SmkError
    nx, ny, nz = shape
    good = G.make_boxes(nx, ny, nz, 2.19, seed=7)
    torch.cuda.synchronize()
    prev = _lib.tune_flag(_lib.SMK_TUNE_TMA, 1)
    _lib.tune_flag(_lib.SMK_TUNE_TMA_WAIT_TEST, 1)
    try:
        bad = G.make_boxes(nx, ny, nz, 2.19, seed=7)
        torch.cuda.synchronize()
    finally:
        _lib.tune_flag(_lib.SMK_TUNE_TMA_WAIT_TEST, 0)
        _lib.tune_flag(_lib.SMK_TUNE_TMA, prev)
    with pytest.raises(SmkError) as e:
        bad.check()
    assert e.value.status == _lib.SMK_ENULLBOX
    again = G.make_boxes(nx, ny, nz, 2.19, seed=7)
    torch.cuda.synchronize()
    again.check()
    assert torch.equal(again.delta, good.delta)


@pytest.mark.parametrize("tag", ["cube16", "rect"])
def test_grf_matches_reference_golden(G, golden, tag):
    f = golden(f"grf_{tag}.npz")
    NX, NY, NZ = int(f["NX"]), int(f["NY"]), int(f["NZ"])
    noise = ograf.draw_noise(NX, NY, NZ, int(f["seed"]))
    out = G.make_boxes(NX, NY, NZ, float(f["DX"]), noise=torch.from_numpy(noise).cuda(),
                       k0=float(f["k0"]))
    torch.cuda.synchronize()
    d = out.delta[0].cpu().numpy()
    e = out.eta[0].cpu().numpy()
    _check(d, f["delta"], "delta vs make_boxes")
    _check(e, f["eta_zz"], "eta_zz vs make_boxes")
    o64 = ograf.grf_boxes(noise, float(f["DX"]), float(f["k0"]), eta=("zz",), precision="f64")
    _check(d, o64["delta"], "delta vs FP64 oracle")
    _check(e, o64["eta_zz"], "eta_zz vs FP64 oracle")
    assert out.sigma()[0] == pytest.approx(float(f["sigma"]), rel=1e-5)
    out.check()


def test_grf_pk_grid_mode_is_the_reference_multiply(G, golden):
    """SMK_PK_GRID multiplies by the reference's own P0 grid (bin/make_boxes.py:290)."""
    f = golden("grf_cube16.npz")
    noise = ograf.draw_noise(16, 16, 16, int(f["seed"]))
    out = G.make_boxes(16, 16, 16, float(f["DX"]), noise=torch.from_numpy(noise).cuda(),
                       pk_grid=torch.from_numpy(f["P0"]).cuda())
    torch.cuda.synchronize()
    _check(out.delta[0].cpu().numpy(), f["delta"], "delta (P-grid) vs make_boxes")
    _check(out.eta[0].cpu().numpy(), f["eta_zz"], "eta_zz (P-grid) vs make_boxes")


# every tile class (n <= 512, <= 1024, <= 2560, <= 4096) on each axis, radices 2, 3, 4, 5, 8
SHAPES = [(32, 24, 40), (12, 600, 10), (2560, 4, 6), (4, 6, 2560), (6, 4000, 4), (4, 4, 4096),
          (2, 2, 2), (30, 18, 50), (1024, 8, 12), (10, 1536, 8), (5, 3, 40), (5, 9, 6)]   # odd row counts


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}x{c}" for a, b, c in SHAPES])
def test_grf_shapes_vs_fp64_oracle(G, shape):
    nx, ny, nz = shape
    rs = np.random.RandomState(nx * 7 + ny * 3 + nz)
    noise = rs.normal(size=shape).astype(np.float32)
    out = G.make_boxes(nx, ny, nz, 2.19, noise=torch.from_numpy(noise).cuda())
    torch.cuda.synchronize()
    o64 = ograf.grf_boxes(noise, 2.19, 0.02, eta=("zz",), precision="f64")
    _check(out.delta[0].cpu().numpy(), o64["delta"], f"delta {shape}")
    _check(out.eta[0].cpu().numpy(), o64["eta_zz"], f"eta {shape}")
    # padding past nz is untouched by nothing else: the view excludes it
    assert out.delta.shape == (1, nx, ny, nz)


def test_grf_batch_equals_single_boxes(G):
    nx, ny, nz, B = 16, 12, 20, 3
    rs = np.random.RandomState(5)
    noise = rs.normal(size=(B, nx, ny, nz)).astype(np.float32)
    out = G.make_boxes(nx, ny, nz, 2.19, noise=torch.from_numpy(noise).cuda(), batch=B)
    torch.cuda.synchronize()
    sig = out.sigma()
    for b in range(B):
        o64 = ograf.grf_boxes(noise[b], 2.19, 0.02, eta=("zz",), precision="f64")
        _check(out.delta[b].cpu().numpy(), o64["delta"], f"batch member {b}")
        _check(out.eta[b].cpu().numpy(), o64["eta_zz"], f"batch member {b} eta")
        assert sig[b] == pytest.approx(np.std(o64["delta"]), rel=1e-5)


@pytest.mark.parametrize("shape", [(24, 20, 18), (15, 9, 10), (16, 16, 16), (600, 6, 4)])
def test_grf_philox_mode_matches_oracle_modes(G, shape):
    """GPU noise mode: the Fourier modes drawn in the x pass (Hermitian kz = 0, nz/2 planes,
    odd and even axes) against the numpy restatement of the same Philox draws."""
    nx, ny, nz = shape
    seed = 123
    out = G.make_boxes(nx, ny, nz, 2.19, seed=seed, batch=2)
    torch.cuda.synchronize()
    for b in range(2):
        nk = ophilox.kspace_noise(nx, ny, nz, seed + b)
        o64 = ograf.grf_from_modes(nk, nz, 2.19, 0.02, eta=("zz",), precision="f64")
        _check(out.delta[b].cpu().numpy(), o64["delta"], f"philox delta {b}")
        _check(out.eta[b].cpu().numpy(), o64["eta_zz"], f"philox eta {b}")


def test_grf_rejects_misaligned_boxes(G):
    """Boxes not on a 16-byte boundary are refused on the host (SMK_EINVAL), before any launch."""
    import ctypes as C
    from saclaymocks_gb300 import _lib
    nx, ny, nz = 8, 6, 10
    p = _lib.SmkGrfParams()
    p.nx, p.ny, p.nz, p.batch, p.dcell = nx, ny, nz, 1, 2.19
    p.noise_mode, p.pk_mode, p.k0, p.amp, p.seed, p.want_eta = _lib.SMK_NOISE_PHILOX, _lib.SMK_PK_ANALYTIC, 0.02, 1.0, 1, 1
    buf = torch.zeros(2 * nx * ny * _lib.load().smk_grf_pitch(nz) + 16, device="cuda")
    base = buf.data_ptr()
    rc = _lib.load().smk_grf_boxes(C.byref(p), base + 8, base + 4096, None, None, 0, None)
    assert rc == _lib.SMK_EINVAL
    rc = _lib.load().smk_grf_boxes(C.byref(p), base, base + 4100, None, None, 0, None)
    assert rc == _lib.SMK_EINVAL


def test_kspace_noise_is_hermitian_on_the_real_planes():
    nk = ophilox.kspace_noise(6, 5, 8, 3)
    for p in (0, 4):
        pl = nk[:, :, p]
        mir = np.conj(pl[(-np.arange(6)) % 6][:, (-np.arange(5)) % 5])
        np.testing.assert_allclose(pl, mir, rtol=0, atol=0)
    # unnormalised |X|^2 averages N = nx*ny*nz
    big = ophilox.kspace_noise(32, 32, 32, 9)
    assert np.mean(np.abs(big[:, :, 1:16]) ** 2) == pytest.approx(32 ** 3, rel=0.02)


def test_grf_philox_recovers_input_pk(G):
    """GPU noise mode, checked statistically: the measured P(k) matches the mode-averaged input
    spectrum within cosmic variance (relative sigma sqrt(2/n_modes)) in every k bin."""
    n, dx = 128, 2.19
    out = G.make_boxes(n, n, n, dx, seed=7, want_eta=False)
    torch.cuda.synchronize()
    d = out.delta[0].cpu().numpy()
    A = ograf.pk_normalisation(n, n, n, dx, 0.02)
    kb = np.linspace(2 * np.pi / (n * dx), np.pi / dx, 17)
    km, pm, nm, pin = ograf.measured_pk(d, dx, kb, lambda k: A * ograf.pk_shape(k, 0.02))
    ok = nm > 50
    z = (pm[ok] - pin[ok]) / (pin[ok] * np.sqrt(2.0 / nm[ok]))
    assert np.all(np.abs(z) < 5), z
    assert abs(np.mean(z)) < 3.0


def test_pk_normalisation_fp64(G):
    for shape in [(16, 16, 16), (64, 48, 40), (256, 256, 256)]:
        a = G.pk_normalisation(*shape, 2.19, 0.02)
        # P~(k) is evaluated in float32 per mode and summed in FP64
        assert a == pytest.approx(ograf.pk_normalisation(*shape, 2.19, 0.02), rel=5e-7)


def test_grf_rejects_bad_sizes(G):
    from saclaymocks_gb300._lib import SmkError, SMK_EINVAL, SMK_ENOTSUPP
    with pytest.raises(SmkError) as e:
        G.make_boxes(16, 16, 15)              # odd nz
    assert e.value.status == SMK_EINVAL
    with pytest.raises(SmkError) as e:
        G.make_boxes(14, 16, 16)              # 14 = 2 * 7
    assert e.value.status == SMK_ENOTSUPP
    with pytest.raises(SmkError) as e:
        G.make_boxes(16, 8192, 16)            # axis longer than 4096
    assert e.value.status == SMK_ENOTSUPP


VARIANT_AXES = {  # pass -> which axis is its line, shapes per length class
    "zfwd": 2, "zinv": 2, "line": 1, "xpass": 0, "xgen": 0}
CLASS_LEN = {512: 40, 1024: 600, 2560: 1536, 4096: 4000}


def _all_variants(pid):
    """(variant, W, threads, test length) of every variant of a pass: a length of its class, or
    the one length of a variant compiled for a fixed length (n_max < 0)."""
    import ctypes as C
    from saclaymocks_gb300 import _lib
    lib = _lib.load()
    out = []
    w, t, nm = C.c_int32(), C.c_int32(), C.c_int32()
    for v in range(lib.smk_tune_count(pid)):
        _lib.check(lib.smk_tune_info(pid, v, C.byref(w), C.byref(t), C.byref(nm)))
        out.append((v, w.value, t.value, -nm.value if nm.value < 0 else CLASS_LEN[nm.value]))
    return out


def test_fixed_length_variants_equal_run_time_plan_variants(G):
    """A variant compiled for one length (its FFT plan as constants) gives the same boxes, bit
    for bit, as the variant of the same tile (W, threads) that reads the plan at run time."""
    import ctypes as C
    from saclaymocks_gb300 import _lib
    lib = _lib.load()
    checked = 0
    for pid, axis in ((_lib.SMK_PASS_LINE, 1), (_lib.SMK_PASS_XGEN, 0), (_lib.SMK_PASS_XPASS, 0),
                      (_lib.SMK_PASS_ZFWD, 2), (_lib.SMK_PASS_ZINV, 2)):
        info = {}
        w, t, nm = C.c_int32(), C.c_int32(), C.c_int32()
        for v in range(lib.smk_tune_count(pid)):
            _lib.check(lib.smk_tune_info(pid, v, C.byref(w), C.byref(t), C.byref(nm)))
            info[v] = (w.value, t.value, nm.value)
        for vf, (wf, tf, nf) in info.items():
            if nf >= 0:
                continue
            n = -nf
            twin = [v for v, (wv, tv, nv) in info.items() if (wv, tv) == (wf, tf) and nv >= n]
            if not twin:
                continue            # checked against the oracle by the every-variant tests
            shape = [6, 4, 8]
            shape[axis] = n
            noise = None
            if pid in (_lib.SMK_PASS_XPASS, _lib.SMK_PASS_ZFWD):
                noise = torch.from_numpy(np.random.RandomState(3).normal(size=shape).astype(np.float32)).cuda()
            res = []
            for v in (vf, twin[0]):
                _lib.check(lib.smk_tune_set(pid, n, v))
                try:
                    for xi in (0, 32):
                        o = G.make_boxes(*shape, 2.19, seed=23, noise=noise, xi_chunk_kz=xi)
                        torch.cuda.synchronize()
                        res.append((o.delta[0].clone(), o.eta[0].clone()))
                finally:
                    lib.smk_tune_set(pid, n, -1)
            for (d0, e0), (d1, e1) in zip(res[:2], res[2:]):
                assert torch.equal(d0, d1) and torch.equal(e0, e1), f"pass {pid} variant {vf} vs {twin[0]}"
            checked += 1
    assert checked >= 1


@pytest.mark.parametrize("pname", ["zfwd", "line", "xpass", "xgen", "zinv"])
def test_every_tile_variant_is_exact(G, pname):
    """Each tile variant (W, threads) of each pass reproduces the FP64 oracle."""
    from saclaymocks_gb300 import _lib, tune
    pid = {v: k for k, v in tune.PASS_NAMES.items()}[pname]
    lib = _lib.load()
    gpu_noise = pname == "xgen"
    for v, w, t, n in _all_variants(pid):
        shape = [6, 4, 8]
        shape[VARIANT_AXES[pname]] = n
        nx, ny, nz = shape
        _lib.check(lib.smk_tune_set(pid, n, v))
        try:
            if gpu_noise:
                out = G.make_boxes(nx, ny, nz, 2.19, seed=17, xi_chunk_kz=0)   # the in-place x pass
                nk = ophilox.kspace_noise(nx, ny, nz, 17)
                o64 = ograf.grf_from_modes(nk, nz, 2.19, 0.02, eta=("zz",), precision="f64")
            else:
                noise = np.random.RandomState(v).normal(size=shape).astype(np.float32)
                out = G.make_boxes(nx, ny, nz, 2.19, noise=torch.from_numpy(noise).cuda())
                o64 = ograf.grf_boxes(noise, 2.19, 0.02, eta=("zz",), precision="f64")
            torch.cuda.synchronize()
            _check(out.delta[0].cpu().numpy(), o64["delta"], f"{pname} variant {v} (W={w}, T={t})")
            _check(out.eta[0].cpu().numpy(), o64["eta_zz"], f"{pname} variant {v} eta")
        finally:
            lib.smk_tune_set(pid, n, -1)


def test_philox_batch_member_equals_single_call(G):
    """One batched call of B boxes (box b drawn from seed + b) gives the same boxes, bit for
    bit, as B single-box calls with seeds seed + b."""
    nx, ny, nz, B, seed = 20, 18, 24, 4, 100
    out = G.make_boxes(nx, ny, nz, 2.19, seed=seed, batch=B)
    for b in range(B):
        one = G.make_boxes(nx, ny, nz, 2.19, seed=seed + b)
        torch.cuda.synchronize()
        assert torch.equal(out.delta[b], one.delta[0])
        assert torch.equal(out.eta[b], one.eta[0])


def test_grf_replayed_from_a_cuda_graph_equals_eager(G):
    """smk_grf_boxes is stream-ordered and sync-free, so it can be captured in a CUDA graph;
    a replay reproduces the eager call bit for bit."""
    nx, ny, nz = 24, 20, 30
    amp = G.pk_normalisation(nx, ny, nz)
    eager = G.make_boxes(nx, ny, nz, 2.19, seed=9, amp=amp)
    out = G.alloc_boxes(nx, ny, nz)
    ws = G.GrfWorkspace(1)
    G.make_boxes(nx, ny, nz, 2.19, seed=9, amp=amp, out=out, workspace=ws)   # launch set-up outside capture
    torch.cuda.synchronize()
    out[0].zero_()
    out[1].zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        G.make_boxes(nx, ny, nz, 2.19, seed=9, amp=amp, out=out, workspace=ws)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out[0][..., :nz], eager.delta)
    assert torch.equal(out[1][..., :nz], eager.eta)


def test_xgen_split_launches_equal_one_launch(G):
    """The GPU-noise x pass written as two one-field launches (the large-box form) gives the
    same boxes, bit for bit, as the one-launch form."""
    from saclaymocks_gb300 import _lib
    nx, ny, nz = 40, 24, 36
    prev = _lib.xgen_split(0)
    try:
        one = G.make_boxes(nx, ny, nz, 2.19, seed=21, batch=2)
        _lib.xgen_split(1)
        two = G.make_boxes(nx, ny, nz, 2.19, seed=21, batch=2)
        torch.cuda.synchronize()
    finally:
        _lib.xgen_split(prev)
    assert torch.equal(one.delta, two.delta)
    assert torch.equal(one.eta, two.eta)
    delta_only = G.make_boxes(nx, ny, nz, 2.19, seed=21, batch=2, want_eta=False)
    torch.cuda.synchronize()
    assert torch.equal(delta_only.delta, one.delta)


@pytest.mark.parametrize("tag", ["cube16", "rect"])
def test_lognormal_and_velocity_boxes_match_reference_golden(G, golden, tag):
    """boxln_1..3 (SMK_PK_GRID with the Pln grids, delta box only) and vx, vy, vz
    (SMK_ETA_VX/VY/VZ, vel_factor = H0 dD/dz(0)) against the reference's main()."""
    f = golden(f"grf_{tag}.npz")
    NX, NY, NZ = int(f["NX"]), int(f["NY"]), int(f["NZ"])
    dx, k0 = float(f["DX"]), float(f["k0"])
    noise = torch.from_numpy(ograf.draw_noise(NX, NY, NZ, int(f["seed"]))).cuda()
    for i in (1, 2, 3):
        out = G.make_boxes(NX, NY, NZ, dx, noise=noise, pk_grid=torch.from_numpy(f[f"Pln{i}"]).cuda(),
                           want_eta=False)
        torch.cuda.synchronize()
        _check(out.delta[0].cpu().numpy(), f[f"boxln_{i}"], f"boxln_{i}")
    vf = float(f["H0"]) * float(f["dgrowth0"])
    for c in ("vx", "vy", "vz"):
        out = G.make_boxes(NX, NY, NZ, dx, noise=noise, k0=k0, eta_comp=c, vel_factor=vf)
        torch.cuda.synchronize()
        _check(out.delta[0].cpu().numpy(), f["delta"], f"delta with {c}")
        _check(out.eta[0].cpu().numpy(), f[c], c)
    # the same components in GPU-noise mode against the FP64 oracle on the drawn modes
    nk = ophilox.kspace_noise(NX, NY, NZ, 77)
    o64 = ograf.grf_from_modes(nk, NZ, dx, k0, eta=(), precision="f64", velocity=(float(f["H0"]), float(f["dgrowth0"])))
    for c in ("vx", "vy", "vz"):
        out = G.make_boxes(NX, NY, NZ, dx, seed=77, k0=k0, eta_comp=c, vel_factor=vf)
        torch.cuda.synchronize()
        _check(out.eta[0].cpu().numpy(), o64[c], f"philox {c}")


@pytest.mark.parametrize("gpu_noise", [True, False])
def test_tuner_choices_are_valid_and_exact(G, gpu_noise):
    """tune.tune_grf times every candidate of each pass by coordinate descent (the x pass first:
    its tile sets the intermediate's layout the y pass reads), applies the fastest, and the boxes
    made with its choices match the FP64 oracle; the built-in choice comes back afterwards."""
    from saclaymocks_gb300 import _lib, tune
    lib = _lib.load()
    nx, ny, nz = 48, 600, 40
    noise = None if gpu_noise else np.random.RandomState(4).normal(size=(nx, ny, nz)).astype(np.float32)
    passes = ([(_lib.SMK_PASS_XGEN, nx), (_lib.SMK_PASS_LINE, ny), (_lib.SMK_PASS_ZINV, nz)] if gpu_noise else
              [(_lib.SMK_PASS_ZFWD, nz), (_lib.SMK_PASS_LINE, ny), (_lib.SMK_PASS_XPASS, nx), (_lib.SMK_PASS_ZINV, nz)])
    builtin = {p: lib.smk_tune_get(p, n) for p, n in passes}
    try:
        res = tune.tune_grf(nx, ny, nz, 2.19, gpu_noise=gpu_noise, reps=1, use_cache=False, xi_chunk_kz=16)
        for p, n in passes:
            name = tune.PASS_NAMES[p]
            cands = [v for v, _, _ in tune.variants(p, n)]
            assert sorted(int(v) for v in res["ms"][name]) == sorted(cands)
            v = res["choices"][name][0]
            assert res["ms"][name][v] == min(res["ms"][name].values())
            assert lib.smk_tune_get(p, n) == v
        if gpu_noise:
            out = G.make_boxes(nx, ny, nz, 2.19, seed=31, xi_chunk_kz=16)
            nk = ophilox.kspace_noise(nx, ny, nz, 31)
            o64 = ograf.grf_from_modes(nk, nz, 2.19, 0.02, eta=("zz",), precision="f64")
        else:
            out = G.make_boxes(nx, ny, nz, 2.19, noise=torch.from_numpy(noise).cuda(), xi_chunk_kz=16)
            o64 = ograf.grf_boxes(noise, 2.19, 0.02, eta=("zz",), precision="f64")
        torch.cuda.synchronize()
        _check(out.delta[0].cpu().numpy(), o64["delta"], "tuned delta")
        _check(out.eta[0].cpu().numpy(), o64["eta_zz"], "tuned eta")
    finally:
        for p, n in passes:
            lib.smk_tune_set(p, n, -1)
    assert {p: lib.smk_tune_get(p, n) for p, n in passes} == builtin
