// Tile variants of the strided c2c pass along y, forward (host-noise path).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_line_fwd(int v, const LineArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_line<TileCfg<W, T, R, B, SMK_NFIX(N), 0>>(a, false, st);
    SMK_LINE_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "line: no tile variant %d", v);
}

}  // namespace smk
