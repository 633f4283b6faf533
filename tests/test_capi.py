"""The C-ABI library: it loads without a GPU, exports every function include/smk.h declares,
and its host-only entry points (plans, pitch, schedule, status checks, argument validation)
behave as documented."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from saclaymocks_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "smk.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(smk_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), f"{n} declared in smk.h but not exported"
        assert n in _lib.EXPORTED, f"{n} has no ctypes prototype"


def test_fft_support_and_pitch(lib):
    assert all(lib.smk_fft_supported(n) for n in (2, 3, 5, 16, 18, 600, 1536, 2560, 4000, 4096))
    assert not any(lib.smk_fft_supported(n) for n in (1, 7, 14, 4097, 8192, 2 * 4096))
    for nz in (2, 16, 18, 256, 1536):
        p = lib.smk_grf_pitch(nz)
        assert p >= 2 * (nz // 2 + 1) and p % 8 == 0 and p - 2 * (nz // 2 + 1) < 8


def test_schedule_pairs_equal_fft_lengths(lib):
    rs = np.random.RandomState(0)
    npix = rs.randint(1, 2000, 1001).astype(np.int32)
    order = np.empty(2 * len(npix) + 16, np.int32)
    n = C.c_int64()
    assert lib.smk_skewer_schedule(len(npix), npix.ctypes.data, 0, order.ctypes.data, C.byref(n)) == 0
    o = order[:n.value]
    assert n.value % 2 == 0
    assert sorted(o[o >= 0].tolist()) == list(range(len(npix)))   # every skewer exactly once
    rule = lambda m: 256 * 2 ** int(np.ceil(max(0, np.log2((m + 50) / 256))))  # noqa: E731
    for a, b in o.reshape(-1, 2):
        if b >= 0:
            assert rule(npix[a]) == rule(npix[b])
            assert npix[a] >= npix[b]
    # fixed length shorter than a skewer, and lengths past 4096, are rejected
    assert lib.smk_skewer_schedule(len(npix), npix.ctypes.data, 1024, order.ctypes.data, C.byref(n)) \
        == _lib.SMK_EINVAL
    big = np.array([5000], np.int32)
    assert lib.smk_skewer_schedule(1, big.ctypes.data, 0, order.ctypes.data, C.byref(n)) == _lib.SMK_ENOTSUPP
    assert lib.smk_skewer_schedule(1, big.ctypes.data, -1, order.ctypes.data, C.byref(n)) == 0


def test_grf_check_flags_null_and_nan_boxes(lib):
    ok = np.array([1.0, 100.0, 0.0, 0.0])
    sig = C.c_double()
    assert lib.smk_grf_check(ok.ctypes.data_as(C.POINTER(C.c_double)), 100, C.byref(sig)) == 0
    assert sig.value == pytest.approx(np.sqrt(1.0 - 1e-4))
    zero = np.zeros(4)
    assert lib.smk_grf_check(zero.ctypes.data_as(C.POINTER(C.c_double)), 100, None) == _lib.SMK_ENULLBOX
    bad = np.array([1.0, 100.0, 3.0, 0.0])
    assert lib.smk_grf_check(bad.ctypes.data_as(C.POINTER(C.c_double)), 100, None) == _lib.SMK_ENULLBOX
    assert b"non-finite" in lib.smk_last_error()


def test_argument_validation_needs_no_gpu(lib):
    """Invalid calls are refused on the host before any CUDA call."""
    p = _lib.SmkGrfParams(nx=16, ny=16, nz=15, batch=1, dcell=2.19, k0=0.02, amp=1.0,
                          noise_mode=_lib.SMK_NOISE_PHILOX)
    assert lib.smk_grf_boxes(C.byref(p), 0x1000, None, None, None, 0, None) == _lib.SMK_EINVAL
    p.nz = 16
    p.nx = 14
    assert lib.smk_grf_boxes(C.byref(p), 0x1000, None, None, None, 0, None) == _lib.SMK_ENOTSUPP
    p.nx = 16
    p.amp = 0.0                           # normalisation on the device needs a workspace
    assert lib.smk_grf_boxes(C.byref(p), 0x1000, None, None, None, 0, None) == _lib.SMK_EWORKSPACE
    assert lib.smk_grf_boxes(None, 0x1000, None, None, None, 0, None) == _lib.SMK_EINVAL
    assert lib.smk_fgpa(-1, None, None, None, 0, None, 0, None, 0, None, 0, None, None) == _lib.SMK_EINVAL
    assert lib.smk_fgpa(0, None, None, None, 0, None, 0, None, 0, None, 0, None, None) == 0
    sk = _lib.SmkSkewers(n=1, n_slots=3)
    sp = _lib.SmkSpectraParams()
    assert lib.smk_skewers_flux(C.byref(sk), C.byref(sp), None, None, 0x1000, None, None, None,
                                None, 0, None) == _lib.SMK_EINVAL
    empty = _lib.SmkSkewers(n=0, n_slots=0)            # an empty table is a no-op
    assert lib.smk_skewers_flux(C.byref(empty), C.byref(sp), None, None, None, None, None, None,
                                None, 0, None) == 0
    assert lib.smk_strerror(_lib.SMK_ENULLBOX).startswith(b"SMK_ENULLBOX")


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(_lib.SmkError):
        _lib.load(str(tmp_path / "libsmk.so"))


def test_tune_flags(lib):
    """smk_tune_flag is host-only state: bad flags and values are rejected, the previous value
    comes back through the out pointer."""
    prev = C.c_int32(7)
    assert lib.smk_tune_flag(_lib.SMK_TUNE_XGEN_SPLIT, 3, C.byref(prev)) == _lib.SMK_EINVAL
    assert lib.smk_tune_flag(9, 0, C.byref(prev)) == _lib.SMK_EINVAL
    assert lib.smk_tune_flag(_lib.SMK_TUNE_XGEN_SPLIT, 1, C.byref(prev)) == _lib.SMK_OK
    assert prev.value == -1
    assert _lib.xgen_split(-1) == 1
    assert _lib.xgen_split(-1) == -1
    assert _lib.tune_flag(_lib.SMK_TUNE_PREFETCH, 0) == 1
    assert _lib.tune_flag(_lib.SMK_TUNE_PREFETCH, 1) == 0
    assert lib.smk_tune_flag(_lib.SMK_TUNE_PREFETCH, 2, None) == _lib.SMK_EINVAL


def test_tma_flags(lib):
    """The y pass's TMA mode, the TMA wait test switch and the skewer kernel's block cap are
    host-only settings with checked ranges."""
    for flag, good, bad in ((_lib.SMK_TUNE_TMA, (0, 1, 2), (3, -1)),
                            (_lib.SMK_TUNE_TMA_WAIT_TEST, (0, 1), (2, -1)),
                            (_lib.SMK_TUNE_SKEWER_BLOCKS, (0, 1, 4, 32), (33, -1))):
        first = _lib.tune_flag(flag, good[0])
        for v in good[1:]:
            _lib.tune_flag(flag, v)
        assert _lib.tune_flag(flag, first) == good[-1]
        for v in bad:
            assert lib.smk_tune_flag(flag, v, None) == _lib.SMK_EINVAL
    assert _lib.tune_flag(_lib.SMK_TUNE_TMA_WAIT_TEST, 0) == 0


def test_grf_workspace_size_and_alignment_need_no_gpu(lib):
    """The workspace query (256 bytes: the FP64 normalisation accumulator) and the 16-byte
    alignment rule of the boxes are host-side: a misaligned delta, eta or workspace is refused
    with SMK_EINVAL before any CUDA call."""
    p = _lib.SmkGrfParams()
    p.nx, p.ny, p.nz, p.batch, p.dcell = 10, 6, 40, 2, 2.19
    p.noise_mode, p.pk_mode, p.k0, p.amp, p.want_eta = _lib.SMK_NOISE_PHILOX, _lib.SMK_PK_ANALYTIC, 0.02, 1.0, 1
    lib.smk_grf_workspace_size.restype = C.c_size_t
    assert lib.smk_grf_workspace_size(C.byref(p)) == 256
    # blocked x-pass intermediate: one chunk of roundup(xi_chunk_kz, 16) k_z columns (at most
    # roundup(nz/2+1, 16)) for each field
    p.xi_chunk_kz = 20
    assert lib.smk_grf_workspace_size(C.byref(p)) == 256 + 2 * 2 * 10 * 6 * 32 * 8
    p.xi_chunk_kz = 5000
    assert lib.smk_grf_workspace_size(C.byref(p)) == 256 + 2 * 2 * 10 * 6 * 32 * 8
    p.want_eta = 0
    assert lib.smk_grf_workspace_size(C.byref(p)) == 256 + 2 * 10 * 6 * 32 * 8
    p.want_eta, p.xi_chunk_kz = 1, 0
    base = 1 << 20   # never dereferenced: the call returns before touching memory
    for d, e, w in ((base + 8, base + 4096, None), (base, base + 4100, None), (base, base + 4096, base + 4)):
        assert lib.smk_grf_boxes(C.byref(p), d, e, None, w, 0, None) == _lib.SMK_EINVAL
