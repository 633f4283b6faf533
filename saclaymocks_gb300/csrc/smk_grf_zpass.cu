// Tile variants of the z passes (r2c of host noise, c2r + statistics).
#include "smk_grf_kernels.cuh"

namespace smk {

int run_zfwd(int v, const ZFwdArgs& a, int64_t rows_per_box, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_zfwd<TileCfg<W, T, R, B, SMK_NFIX(N)>>(a, rows_per_box, st);
    SMK_Z_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "zfwd: no tile variant %d", v);
}

int run_zinv(int v, const ZInvArgs& a, int64_t rows_per_box, cudaStream_t st) {
    int i = 0;
#define X(W, T, N, R, B) \
    if (v == i++) return launch_zinv<TileCfg<W, T, R, B, SMK_NFIX(N)>>(a, rows_per_box, st);
    SMK_ZINV_VARIANTS(X)
#undef X
    return fail(SMK_EINVAL, "zinv: no tile variant %d", v);
}

}  // namespace smk
