// Tile variants of the host-noise x pass into the blocked intermediate (xpi).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_xpi(int v, const XArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_xpi<TileCfg<W, T, R, B, SMK_NFIX(N)>>(a, st);
    SMK_X_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "xpi: no tile variant %d", v);
}

}  // namespace smk
