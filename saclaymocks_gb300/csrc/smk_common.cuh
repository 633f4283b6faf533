// Shared device/host helpers of libsmk: status reporting, complex arithmetic,
// Philox4x32-10 counter-based random numbers, twiddle factors.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/smk.h"

namespace smk {

// Process-wide cap on the skewer kernel's resident blocks per SM (SMK_TUNE_SKEWER_BLOCKS; 0:
// as many as fit), defined in smk_skewers.cu.
extern std::atomic<int> g_skewer_blocks;

// ------------------------------------------------------------------ status (host)
// Records a message for smk_last_error() and returns the code.
int fail(int code, const char* fmt, ...);
// Checks cudaGetLastError() after launches: SMK_ECUDA with the CUDA message on failure.
int check_launch(const char* what);

inline int64_t div_up(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Host: tiled TMA map over an array of 8-byte elements (complex float) with dims (d0, d1, d2),
// element strides s1 (dim 1) and s2 (dim 2), boxes of b0 x b1 x 1, zero fill outside; false if
// the driver cannot encode it (the caller then loads without TMA).
bool encode_map_3d_8b(CUtensorMap* m, const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t s1,
                      uint64_t s2, uint32_t b0, uint32_t b1);

bool encode_map_5d_8b(CUtensorMap* m, const void* base, const uint64_t* d, const uint64_t* st, const uint32_t* b);

// ------------------------------------------------------------------ complex helpers
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// exp(-2 pi i m / n) for 0 <= m < n <= 2^24.  The angle is reduced to a quadrant with
// integer arithmetic so the float argument of sincospif stays in [0, 0.5) and is the
// correctly rounded value of rem/(2n): the twiddle is accurate to about 1 ulp.
__device__ __forceinline__ float2 twiddle(int m, int n) {
    const int m4 = 4 * m;
    const int q = m4 / n;
    const int rem = m4 - q * n;
    float s, c;
    sincospif(0.5f * ((float)rem / (float)n), &s, &c);
    // angle = q*pi/2 + phi, phi = (pi/2)*rem/n; result = (cos(angle), -sin(angle))
    switch (q & 3) {
        case 0: return make_float2(c, -s);
        case 1: return make_float2(-s, -c);
        case 2: return make_float2(-c, s);
        default: return make_float2(s, c);
    }
}

// ------------------------------------------------------------------ asynchronous copies
// cp.async global -> shared of `bytes` (4, 8 or 16) with zero fill of the rest of the
// `size`-byte slot: no register staging, so a thread keeps many copies in flight.  A
// source that is not read (src_bytes == 0) is still given a valid address by the caller.
template <int SIZE>
__device__ __forceinline__ void cp_async(void* smem_dst, const void* gmem_src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    if (SIZE == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem_src), "r"(src_bytes));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(gmem_src), "n"(SIZE),
                     "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ------------------------------------------------------------------ TMA tensor loads + mbarrier
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Makes barrier initialisation visible to the asynchronous (TMA) proxy.
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
// One arrival that also expects `bytes` of transactions (the TMA copies of this phase).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}
// Waits for the phase of the given parity to complete, for at most ~`limit` clock cycles;
// false on time-out (the caller flags its results instead of waiting on).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, long long limit) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}
// Orders this thread's earlier generic-proxy shared-memory accesses before later TMA writes.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// Tiled 3D TMA load of one box at (x, y, z) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// Tiled 5D TMA load of one box at (c0 .. c4) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3, int c4) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n"
        ::"r"(smem_u32(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
        : "memory");
}

// Tiled 3D TMA store of one box from shared memory at (x, y, z) (elements outside the map's
// dims are not written), in the thread's current bulk group.
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int x, int y, int z) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n"
                 ::"l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// Waits until the shared-memory sources of this thread's bulk stores have been read.
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// Waits until this thread's bulk stores are complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

// Hints that pull the next tile's bytes into L2 while the current tile is transformed: one
// cache line, or a 16-byte-aligned run of bytes (a multiple of 16) with the bulk form.
__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
}
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}

// ------------------------------------------------------------------ Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
// easy as 1, 2, 3" (SC'11): 10 rounds of the 4x32 Philox bijection keyed by the seed.
struct u32x4 { uint32_t v[4]; };

__host__ __device__ __forceinline__ u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)M0 * ctr.v[0];
        const uint64_t p1 = (uint64_t)M1 * ctr.v[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        u32x4 o;
        o.v[0] = hi1 ^ ctr.v[1] ^ k0;
        o.v[1] = lo1;
        o.v[2] = hi0 ^ ctr.v[3] ^ k1;
        o.v[3] = lo0;
        ctr = o;
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

// Hardware special functions on normal arguments (PTX .approx with .ftz: only subnormal inputs and
// outputs would differ from rsqrtf / __log2f / __sinf / __cosf, and none arise where these are
// used), without the subnormal range handling that the non-ftz forms add.
__device__ __forceinline__ float hw_rsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float hw_log2(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void hw_sincos(float x, float* s, float* c) {
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(*s) : "f"(x));
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(*c) : "f"(x));
}

// The same block with the round keys precomputed (rk0[r] = k0 + r W0, rk1[r] = k1 + r W1, mod 2^32):
// keys held in kernel parameters enter the XORs as constant operands, no key additions per round.
__host__ __device__ __forceinline__ u32x4 philox4x32_10_rk(u32x4 ctr, const uint32_t* rk0, const uint32_t* rk1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)M0 * ctr.v[0];
        const uint64_t p1 = (uint64_t)M1 * ctr.v[2];
        u32x4 o;
        o.v[0] = (uint32_t)(p1 >> 32) ^ ctr.v[1] ^ rk0[r];
        o.v[1] = (uint32_t)p1;
        o.v[2] = (uint32_t)(p0 >> 32) ^ ctr.v[3] ^ rk1[r];
        o.v[3] = (uint32_t)p0;
        ctr = o;
    }
    return ctr;
}
inline void philox_round_keys(uint64_t seed, uint32_t rk0[10], uint32_t rk1[10]) {
    for (int r = 0; r < 10; ++r) {
        rk0[r] = (uint32_t)seed + (uint32_t)r * 0x9E3779B9u;
        rk1[r] = (uint32_t)(seed >> 32) + (uint32_t)r * 0xBB67AE85u;
    }
}

// Stream tags keep the Fourier-mode noise of the boxes and the skewer noise in disjoint
// counter spaces.
enum : uint32_t { STREAM_KMODE = 0x4Bu, STREAM_SKEWER = 0x53u };

// Four N(0,1) deviates from one Philox block: Box-Muller on (x0,x1) and (x2,x3).  The top
// 23 bits m of each word become floats by exponent insertion (no integer conversion):
// v = 1 + m 2^-23 in [1, 2), exact; u = 2 - v = 1 - m 2^-23 in (0, 1] for the radius and
// pi (2v - 3) in [-pi, pi) for the angle, i.e. pi (t - 1) with t = m 2^-22 in [0, 2).  The
// angle uses the hardware sine/cosine (absolute error < 4e-7 on [-pi, pi)) with the signs
// flipped back; the radius -2 ln u the hardware base-2 logarithm (absolute error ~1e-7 near
// u = 1, so deviates of radius < 0.01, probability 5e-5, carry absolute errors up to ~1e-5)
// and the reciprocal square root.
__device__ __forceinline__ void gauss4(u32x4 r, float g[4]) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float u1 = 2.0f - __uint_as_float(0x3F800000u | (r.v[2 * h] >> 9));
        const float v = __uint_as_float(0x3F800000u | (r.v[2 * h + 1] >> 9));
        const float x = -1.3862943611198906f * hw_log2(u1);                             // -2 ln 2 log2(u)
        const float rad = x > 0.0f ? x * hw_rsqrt(x) : 0.0f;
        float s, c;
        hw_sincos(fmaf(v, 6.28318530717958648f, -9.42477796076937972f), &s, &c);
        g[2 * h] = -rad * c;
        g[2 * h + 1] = -rad * s;
    }
}

// Gaussians of group q (cells 4q..4q+3) of row `row` for seed `seed`, stream `tag`.
__device__ __forceinline__ void philox_gauss4(uint64_t seed, uint64_t row, uint32_t q, uint32_t tag,
                                              float g[4]) {
    u32x4 c;
    c.v[0] = q;
    c.v[1] = (uint32_t)row;
    c.v[2] = (uint32_t)(row >> 32);
    c.v[3] = tag;
    gauss4(philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32)), g);
}

}  // namespace smk
