// Tile variants of the host-noise x pass in place in the boxes (xpass; xpi, into the blocked
// intermediate, is in smk_grf_xpi.cu).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_xpass(int v, const XArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_xpass<TileCfg<W, T, R, B, SMK_NFIX(N)>>(a, st);
    SMK_X_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "xpass: no tile variant %d", v);
}

}  // namespace smk
