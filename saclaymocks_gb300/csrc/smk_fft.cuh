// Line-FFT engine of libsmk: mixed-radix (2,3,4,5,8) in-place transforms of W lines held in
// shared memory, all lines sharing one twiddle table.
//
// Tile layout: element e of line w sits at s[e*SN + w] (lines interleaved, SN >= W), so a
// tile of W consecutive columns of a strided axis is loaded with W*8-byte contiguous runs.
//
// Forward transforms are decimation in frequency (DIF): stage s of radix R works on blocks
// of L = n / (R_0 ... R_{s-1}) elements; with m = L/R, butterfly (block, q) reads the R
// elements block*L + q + r*m, applies an R-point DFT and multiplies output r by
// W_L^{r q} = exp(-2 pi i r q / L), writing back to the same slots.  Natural-order input
// leaves the spectrum in mixed-radix digit-reversed order: slot p holds frequency
// freq_of_slot(p).  Inverse transforms (INV) are the adjoint sequence: decimation in time,
// stages in reverse order, conjugate twiddles applied before an inverse R-point DFT, taking
// digit-reversed input back to natural order (unnormalised).  So a forward + pointwise
// operation + inverse needs no permutation; code that needs frequency k reads slot
// slot_of_freq(k).  Butterflies of a stage are independent and in place: a thread holds one
// butterfly at a time and the block synchronises only between stages.
#pragma once

#include "smk_common.cuh"

namespace smk {

constexpr int FFT_MAX_N = 4096;
constexpr int FFT_MAX_STAGES = 12;

struct FftPlan {
    int n;
    int nst;
    int r[FFT_MAX_STAGES];        // radix of stage s (DIF order)
    int m[FFT_MAX_STAGES];        // L_s / R_s: stride between the inputs of a butterfly
    int tstep[FFT_MAX_STAGES];    // n / L_s: twiddle-table step
    uint32_t magic[FFT_MAX_STAGES];  // floor(2^32/m) + 1: x / m == umulhi(x, magic) for x < 2^16
};

// Host: radix plan of n (8s first, then 4s/2 for the rest of the power of two, 3s, 5s).
// Returns false unless 2 <= n <= FFT_MAX_N and n = 2^a 3^b 5^c.
bool make_plan(int n, FftPlan* p);

__device__ __forceinline__ int div_m(const FftPlan& pl, int st, int x) {
    return pl.m[st] == 1 ? x : (int)__umulhi((unsigned)x, pl.magic[st]);
}

// Frequency held by slot p after a forward (DIF) transform.
__device__ __forceinline__ int freq_of_slot(const FftPlan& pl, int p) {
    int k = 0, mult = 1;
    for (int st = 0; st < pl.nst; ++st) {
        const int d = div_m(pl, st, p);
        p -= d * pl.m[st];
        k += d * mult;
        mult *= pl.r[st];
    }
    return k;
}

// Slot that holds frequency k after a forward (DIF) transform (inverse of freq_of_slot).
__device__ __forceinline__ int slot_of_freq(const FftPlan& pl, int k) {
    int p = 0;
    for (int st = 0; st < pl.nst; ++st) {
        const int R = pl.r[st];
        const int q = k / R;
        p += (k - q * R) * pl.m[st];
        k = q;
    }
    return p;
}

// ------------------------------------------------------------------ R-point DFTs
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {  // * (-i) forward, * (+i) inverse
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
    __device__ __forceinline__ static void run(float2* v) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <bool INV>
struct Dft<3, INV> {
    __device__ __forceinline__ static void run(float2* v) {
        const float h = 0.86602540378443864676f;  // sin(2 pi / 3)
        const float2 a = cadd(v[1], v[2]);
        const float2 b = csub(v[1], v[2]);
        const float2 t = make_float2(v[0].x - 0.5f * a.x, v[0].y - 0.5f * a.y);
        const float2 u = cscale(mul_mi<INV>(b), h);
        v[0] = cadd(v[0], a);
        v[1] = cadd(t, u);
        v[2] = csub(t, u);
    }
};

template <bool INV>
struct Dft<4, INV> {
    __device__ __forceinline__ static void run(float2* v) {
        const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        const float2 t2 = cadd(v[1], v[3]), t3 = mul_mi<INV>(csub(v[1], v[3]));
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    }
};

template <bool INV>
struct Dft<5, INV> {
    __device__ __forceinline__ static void run(float2* v) {
        const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
        const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
        const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
        const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
        const float2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
        const float2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
        const float2 x0 = v[0];
        const float2 t1 = make_float2(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
        const float2 t2 = make_float2(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
        const float2 u1 = mul_mi<INV>(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
        const float2 u2 = mul_mi<INV>(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
        v[0] = make_float2(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
        v[1] = cadd(t1, u1);
        v[4] = csub(t1, u1);
        v[2] = cadd(t2, u2);
        v[3] = csub(t2, u2);
    }
};

template <bool INV>
struct Dft<8, INV> {
    __device__ __forceinline__ static void run(float2* v) {
        const float h = 0.70710678118654752440f;  // 1/sqrt(2)
        float2 a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            a[q] = cadd(v[q], v[q + 4]);
            b[q] = csub(v[q], v[q + 4]);
        }
        // b[q] *= exp(-+ i pi q / 4)
        if (!INV) {
            b[1] = make_float2(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));
            b[2] = mul_mi<false>(b[2]);
            b[3] = make_float2(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));
        } else {
            b[1] = make_float2(h * (b[1].x - b[1].y), h * (b[1].x + b[1].y));
            b[2] = mul_mi<true>(b[2]);
            b[3] = make_float2(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y));
        }
        Dft<4, INV>::run(a);
        Dft<4, INV>::run(b);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v[2 * q] = a[q];
            v[2 * q + 1] = b[q];
        }
    }
};

// ------------------------------------------------------------------ one in-place stage
template <int R, bool INV, int W, int SN, int T>
__device__ __forceinline__ void fft_stage(float2* __restrict__ s, const float2* __restrict__ tw,
                                          const FftPlan& pl, const int st) {
    const int m = pl.m[st];
    const int tstep = pl.tstep[st];
    const int nb = (pl.n / R) * W;
#pragma unroll(T >= 1024 ? 1 : 2)
    for (int bf = threadIdx.x; bf < nb; bf += T) {
        const int j = bf / W, w = bf % W;
        const int blk = div_m(pl, st, j);
        const int q = j - blk * m;
        float2* p = s + (blk * R * m + q) * SN + w;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = p[r * m * SN];
        if (INV) {
            if (q != 0) {
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = cmulc(v[r], tw[r * q * tstep]);
            }
            Dft<R, true>::run(v);
        } else {
            Dft<R, false>::run(v);
            if (q != 0) {
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * q * tstep]);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) p[r * m * SN] = v[r];
    }
    __syncthreads();
}

template <bool INV, int W, int SN, int T>
__device__ __forceinline__ void fft_stage_any(float2* s, const float2* tw, const FftPlan& pl, int st) {
    switch (pl.r[st]) {
        case 8: fft_stage<8, INV, W, SN, T>(s, tw, pl, st); break;
        case 4: fft_stage<4, INV, W, SN, T>(s, tw, pl, st); break;
        case 2: fft_stage<2, INV, W, SN, T>(s, tw, pl, st); break;
        case 3: fft_stage<3, INV, W, SN, T>(s, tw, pl, st); break;
        default: fft_stage<5, INV, W, SN, T>(s, tw, pl, st); break;
    }
}

// Full transform of the W lines of the tile: forward natural -> digit-reversed, inverse
// digit-reversed -> natural (unnormalised).  The caller synchronises after filling s; on
// return the block is synchronised.
template <bool INV, int W, int SN, int T>
__device__ __forceinline__ void fft_tile(float2* __restrict__ s, const float2* __restrict__ tw,
                                         const FftPlan& pl) {
    if (!INV) {
        for (int st = 0; st < pl.nst; ++st) fft_stage_any<false, W, SN, T>(s, tw, pl, st);
    } else {
        for (int st = pl.nst - 1; st >= 0; --st) fft_stage_any<true, W, SN, T>(s, tw, pl, st);
    }
}

// Twiddle table tw[m] = exp(-2 pi i m / n), m < n, filled by the block (no barrier).
template <int T>
__device__ __forceinline__ void fill_twiddles(float2* tw, int n) {
    for (int m = threadIdx.x; m < n; m += T) tw[m] = twiddle(m, n);
}

}  // namespace smk
