// Host-side pieces of libsmk: status strings, thread-local error message, FFT radix plans,
// and the skewer work schedule.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include <mutex>

#include "smk_fft.cuh"

namespace smk {

static thread_local char g_last_error[512] = "";

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int check_launch(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SMK_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    return SMK_OK;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, looked up once (no link against libcuda).
static EncodeTiledFn encode_tiled_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

bool encode_map_3d_8b(CUtensorMap* m, const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t s1,
                      uint64_t s2, uint32_t b0, uint32_t b1) {
    const EncodeTiledFn fn = encode_tiled_fn();
    if (!fn || ((uintptr_t)base & 15) || ((s1 * 8) & 15) || ((s2 * 8) & 15) || ((b0 * 8) & 15) || b0 > 256 || b1 > 256)
        return false;
    const cuuint64_t dims[3] = {d0, d1, d2};
    const cuuint64_t strides[2] = {s1 * 8, s2 * 8};
    const cuuint32_t box[3] = {b0, b1, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void*>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 5D map of 8-byte elements: dims d[0..4] (d[0] innermost, contiguous), element strides
// st[1..4] (multiples of 2 elements), box b[0..4]; out-of-range elements read as zero.
bool encode_map_5d_8b(CUtensorMap* m, const void* base, const uint64_t* d, const uint64_t* st, const uint32_t* b) {
    const EncodeTiledFn fn = encode_tiled_fn();
    if (!fn || ((uintptr_t)base & 15) || ((b[0] * 8) & 15)) return false;
    cuuint64_t dims[5], strides[4];
    cuuint32_t box[5], es[5];
    for (int i = 0; i < 5; ++i) {
        if (b[i] < 1 || b[i] > 256 || d[i] < 1) return false;
        dims[i] = d[i];
        box[i] = b[i];
        es[i] = 1;
        if (i > 0) {
            if ((st[i] * 8) & 15) return false;
            strides[i - 1] = st[i] * 8;
        }
    }
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, const_cast<void*>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace smk

extern "C" {

const char* smk_strerror(int status) {
    switch (status) {
        case SMK_OK: return "SMK_OK";
        case SMK_EINVAL: return "SMK_EINVAL: invalid argument";
        case SMK_ENOTSUPP: return "SMK_ENOTSUPP: size not supported by the kernels";
        case SMK_ECUDA: return "SMK_ECUDA: CUDA error";
        case SMK_EWORKSPACE: return "SMK_EWORKSPACE: workspace missing or too small";
        case SMK_ENULLBOX: return "SMK_ENULLBOX: box is null or holds non-finite values";
        default: return "SMK_E?: unknown status";
    }
}

const char* smk_last_error(void) { return smk::g_last_error; }

int smk_version(void) { return 100; }

int smk_fft_supported(int32_t n) {
    smk::FftPlan p;
    return smk::make_plan(n, &p) ? 1 : 0;
}

int smk_skewer_schedule(int64_t n, const int32_t* npix_host, int32_t ss_nz, int32_t* order_out,
                        int64_t* n_slots_out) {
    if (n < 0 || (n > 0 && (!npix_host || !order_out)) || !n_slots_out)
        return smk::fail(SMK_EINVAL, "smk_skewer_schedule: null argument");
    if (n > INT32_MAX) return smk::fail(SMK_EINVAL, "smk_skewer_schedule: too many skewers");
    // order: small-scale FFT length (the pairing constraint), then length, both descending
    struct Key { int32_t nz, np, s; };
    std::vector<Key> key((size_t)n);
    for (int64_t s = 0; s < n; ++s) {
        const int32_t np = npix_host[s];
        if (np < 0 || np > (1 << 24))
            return smk::fail(SMK_EINVAL, "smk_skewer_schedule: npix %d outside 0..2^24", np);
        int32_t nz = ss_nz;
        if (nz < 0) {
            nz = 0;  // no small-scale field: one class, pairs by length only
        } else if (nz == 0) {
            nz = 256;
            while (nz < np + 50 && nz <= smk::FFT_MAX_N) nz *= 2;
            if (nz > smk::FFT_MAX_N)
                return smk::fail(SMK_ENOTSUPP, "smk_skewer_schedule: skewer %lld needs a "
                                 "small-scale FFT longer than %d", (long long)s, smk::FFT_MAX_N);
        } else if (np > nz) {
            return smk::fail(SMK_EINVAL, "smk_skewer_schedule: skewer %lld has %d pixels, more "
                             "than the small-scale FFT length %d", (long long)s, np, nz);
        }
        key[(size_t)s] = {nz, np, (int32_t)s};
    }
    std::stable_sort(key.begin(), key.end(), [](const Key& a, const Key& b) {
        return a.nz != b.nz ? a.nz > b.nz : a.np > b.np;
    });
    int64_t k = 0;
    for (size_t i = 0; i < key.size();) {
        size_t j = i;
        while (j < key.size() && key[j].nz == key[i].nz) ++j;
        for (size_t q = i; q < j; ++q) order_out[k++] = key[q].s;
        if ((j - i) & 1) order_out[k++] = -1;
        i = j;
    }
    *n_slots_out = k;
    return SMK_OK;
}

}  // extern "C"
