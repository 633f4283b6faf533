// Tile variants of the x passes (host noise: xpass; GPU noise: xgen).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_xpass(int v, const XArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_xpass<TileCfg<W, T, R, B>>(a, st);
    SMK_X_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "xpass: no tile variant %d", v);
}

int run_xgen(int v, const XGenArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_xgen<TileCfg<W, T, R, B>>(a, st);
    SMK_XGEN_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "xgen: no tile variant %d", v);
}

int run_xinv(int v, const XGenArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_xinv<TileCfg<W, T, R, B>>(a, st);
    SMK_XGEN_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "xinv: no tile variant %d", v);
}

int run_kgen(const XGenArgs& a, cudaStream_t st) {
    constexpr int T = 256;
    if (a.sh < 1) return fail(SMK_EINVAL, "kgen: staged blocks of at least 2 columns");
    const size_t smem = (size_t)a.nx * 8 + (size_t)a.nzh * 4 + 16;
    const int64_t wt = (int64_t)1 << a.sh;
    const int64_t lines = ceil_div(a.nzh, wt) * a.batch * a.ny;
    int grid = 0, rc;
    if ((rc = persistent_grid(kgen_kernel<T>, T, smem, lines, &grid))) return rc;
    kgen_kernel<T><<<grid, T, smem, st>>>(a);
    return check_launch("kgen_kernel");
}

}  // namespace smk
