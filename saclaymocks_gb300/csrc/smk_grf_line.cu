// Tile variants of the strided c2c pass along y, inverse (the forward is in smk_grf_linef.cu, so
// that the two compile in parallel).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_line_inv(int v, const LineArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_line<TileCfg<W, T, R, B, SMK_NFIX(N), 1>>(a, true, st);
    SMK_LINE_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "line: no tile variant %d", v);
}

int run_line(int v, const LineArgs& a, bool inv, cudaStream_t st) {
    return inv ? run_line_inv(v, a, st) : run_line_fwd(v, a, st);
}

}  // namespace smk
