// Elementwise FGPA (util.fgpa) on GB300: flux = exp(-a exp(b G (delta + c eta))), float32,
// each parameter a per-element array or a scalar.  HBM bound: 8-24 bytes per element.
#include <algorithm>

#include "smk_common.cuh"

namespace smk {

struct FgpaArgs {
    int64_t n;
    const float* delta;
    const float* eta;
    const float* G;
    const float* a;
    const float* b;
    const float* c;
    float G0, a0, b0, c0;
    float* flux;
};

__device__ __forceinline__ float ld_or(const float* p, int64_t i, float v) { return p ? __ldg(p + i) : v; }

__global__ void __launch_bounds__(256) fgpa_kernel(const FgpaArgs a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = __ldg(a.delta + i);
        const float e = a.eta ? __ldg(a.eta + i) : 0.f;
        const float G = ld_or(a.G, i, a.G0);
        const float pa = ld_or(a.a, i, a.a0), pb = ld_or(a.b, i, a.b0), pc = ld_or(a.c, i, a.c0);
        a.flux[i] = expf(-pa * expf(pb * G * (d + pc * e)));
    }
}

}  // namespace smk

using namespace smk;

extern "C" int smk_fgpa(int64_t n, const float* delta, const float* eta, const float* G, float G0, const float* a,
                        float a0, const float* b, float b0, const float* c, float c0, float* flux, void* stream) {
    if (n < 0) return fail(SMK_EINVAL, "smk_fgpa: n < 0");
    if (n == 0) return SMK_OK;
    if (!delta || !flux) return fail(SMK_EINVAL, "smk_fgpa: null delta or flux");
    FgpaArgs args{n, delta, eta, G, a, b, c, G0, a0, b0, c0, flux};
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)std::max(nsm, 1) * 8);
    fgpa_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(args);
    return check_launch("fgpa_kernel");
}
