// Tile variants of the GPU-noise x pass into the blocked intermediate (xgi).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_xgi(int v, const XGenArgs& a, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_xgi<TileCfg<W, T, R, B, SMK_NFIX(N)>>(a, st);
    SMK_XGEN_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "xgi: no tile variant %d", v);
}

}  // namespace smk
