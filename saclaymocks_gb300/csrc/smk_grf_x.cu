// Tile variants of the GPU-noise x pass in place in the boxes (xgen; xgi, into the blocked
// intermediate, is in smk_grf_xi.cu).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_xgen(int v, const XGenArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_xgen<TileCfg<W, T, R, B, SMK_NFIX(N)>>(a, st);
    SMK_XGEN_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "xgen: no tile variant %d", v);
}

}  // namespace smk
