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

#include <type_traits>

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
    // Per-stage twiddle tables (warp engine): stage s with m > 1 keeps W_L^(r q), L = R m, for
    // q < m, 1 <= r < R at twoff[s] + q (R - 1) + r - 1, so lanes with different q read
    // different banks; twn = total entries (< n + n/8).
    int twoff[FFT_MAX_STAGES];
    int twn;
};

// Radix plan of n (host or device).  rmax >= 16: 16s first; a single factor 2 left over becomes a
// radix-32 stage (rmax >= 32), else joins a 5 (radix 10) or a 3 (radix 6), else stays a 2;
// rmax 8: 8s, then 4s / 2.  3s and 5s follow.
// Returns false unless 2 <= n <= FFT_MAX_N and n = 2^a 3^b 5^c.
// mid: a three-stage plan (R, R, x) becomes (R, x, R) (the warp z pass's conflict-free order).
__host__ __device__ constexpr bool make_plan(int n, FftPlan* p, int rmax = 16, bool mid = false) {
    if (n < 2 || n > FFT_MAX_N) return false;
    int m = n, p2 = 0, p3 = 0, p5 = 0;
    while (m % 2 == 0) { m /= 2; ++p2; }
    while (m % 3 == 0) { m /= 3; ++p3; }
    while (m % 5 == 0) { m /= 5; ++p5; }
    if (m != 1) return false;
    // rmax >= 16: radix-16 stages (a radix-32 one when one factor 2 is left over and
    // rmax >= 32), then 8, 4 or 2 for the rest of the power of two; rmax 8: 8s, then 4s / 2.
    // 3s and 5s follow.
    int rad[32] = {}, nr = 0;
    if (rmax >= 16) {
        while (p2 >= 4) { rad[nr++] = 16; p2 -= 4; }
        if (p2 == 1 && nr > 0 && rmax >= 32) {
            rad[0] = 32;
        } else if (p2 == 1 && p5 > 0) {
            rad[nr++] = 10;
            --p5;
        } else if (p2 == 1 && p3 > 0) {
            rad[nr++] = 6;
            --p3;
        } else if (p2 > 0) {
            rad[nr++] = 1 << p2;
        }
    } else {
        while (p2 >= 3 && p2 - 3 != 1) { rad[nr++] = 8; p2 -= 3; }
        while (p2 >= 2) { rad[nr++] = 4; p2 -= 2; }
        if (p2 == 1) rad[nr++] = 2;
    }
    for (int i = 0; i < p3; ++i) rad[nr++] = 3;
    for (int i = 0; i < p5; ++i) rad[nr++] = 5;
    if (nr > FFT_MAX_STAGES) return false;
    if (mid && nr == 3 && rad[0] == rad[1] && rad[2] != rad[0]) {
        rad[2] = rad[1];   // (R, R, x) -> (R, x, R)
        rad[1] = (n / rad[0]) / rad[0];
    }
    p->n = n;
    p->nst = nr;
    int L = n, tw = 0;
    for (int s = 0; s < nr; ++s) {
        p->r[s] = rad[s];
        p->m[s] = L / rad[s];
        p->tstep[s] = n / L;
        p->magic[s] = p->m[s] == 1 ? 0u : (uint32_t)((1ull << 32) / (uint64_t)p->m[s] + 1ull);
        p->twoff[s] = tw;
        if (p->m[s] > 1) tw += p->m[s] * (rad[s] - 1);
        L = p->m[s];
    }
    for (int s = nr; s < FFT_MAX_STAGES; ++s) p->twoff[s] = tw;
    p->twn = tw;
    return true;
}

// The plan of a length fixed at compile time (FixedPlan<n, rmax>::P.r[st] etc. are constants).
template <int N, int RMAX, bool MID = false>
struct FixedPlan {
    __host__ __device__ static constexpr FftPlan make() {
        FftPlan p{};
        make_plan(N, &p, RMAX, MID);
        return p;
    }
    static constexpr FftPlan P = make();
    static_assert(P.n == N, "FixedPlan: length not supported by the engine");
};

// True when two plans have the same stages (the tables of one serve the other).
__host__ __device__ inline bool same_plan(const FftPlan& a, const FftPlan& b) {
    if (a.n != b.n || a.nst != b.nst) return false;
    for (int s = 0; s < a.nst; ++s)
        if (a.r[s] != b.r[s]) return false;
    return true;
}

// Largest radix a kernel of T threads per block runs in registers without spilling (the
// register budget per thread is 65536 / T): radix 32 for <= 256 threads, 16 for 512, 8 above.
__host__ __device__ constexpr int fft_max_radix(int T) { return T >= 1024 ? 8 : (T >= 512 ? 16 : 32); }

// True when every stage radix of the plan is <= rmax (the kernel compiled that radix).
inline bool plan_fits(const FftPlan& p, int rmax) {
    for (int s = 0; s < p.nst; ++s)
        if (p.r[s] > rmax) return false;
    return true;
}

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
__host__ __device__ __forceinline__ float2 mul_mi(float2 a) {  // * (-i) forward, * (+i) inverse
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
    __host__ __device__ __forceinline__ static void run(float2* v) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <bool INV>
struct Dft<3, INV> {
    __host__ __device__ __forceinline__ static void run(float2* v) {
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
    __host__ __device__ __forceinline__ static void run(float2* v) {
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
    __host__ __device__ __forceinline__ static void run(float2* v) {
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
    __host__ __device__ __forceinline__ static void run(float2* v) {
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

// ------------------------------------------------------------------ composite R-point DFTs
// Compile-time unrolling: f(integral_constant<int, i>) for i = B .. E-1.
template <int B, int E, class F>
__host__ __device__ __forceinline__ void static_for(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// cos / sin of 2 pi m / R by octant reduction and Taylor series in double; used only to
// initialise constexpr twiddle constants (evaluated by the compiler, never at run time).
__host__ __device__ constexpr double taylor_cos(double t) {
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 14; ++k) {
        term *= -t * t / ((2.0 * k - 1.0) * (2.0 * k));
        sum += term;
    }
    return sum;
}
__host__ __device__ constexpr double taylor_sin(double t) {
    double term = t, sum = t;
    for (int k = 1; k < 14; ++k) {
        term *= -t * t / ((2.0 * k) * (2.0 * k + 1.0));
        sum += term;
    }
    return sum;
}
// (cos, sin)(2 pi m / R): reduce m/R to [0, 1/8] with the symmetries of the circle
__host__ __device__ constexpr double unit_cos(int m, int R) {
    m %= R;
    if (m < 0) m += R;
    if (2 * m > R) m = R - m;                        // cos(2pi - a) = cos(a)
    if (4 * m > R) return -unit_cos(R - 2 * m, 2 * R);  // cos(pi - a) = -cos(a)
    const double PI = 3.14159265358979323846;
    if (8 * m > R) return taylor_sin(2.0 * PI * (double)(R - 4 * m) / (4.0 * R));  // cos(a) = sin(pi/2 - a)
    return taylor_cos(2.0 * PI * (double)m / (double)R);
}
__host__ __device__ constexpr double unit_sin(int m, int R) { return unit_cos(4 * m - R, 4 * R); }  // sin a = cos(a - pi/2)

// v * exp(-+ 2 pi i m / R) with m, R compile-time; trivial factors fold away.
template <int M, int R, bool INV>
__host__ __device__ __forceinline__ float2 ctw(float2 v) {
    constexpr int m = ((M % R) + R) % R;
    if constexpr (m == 0) {
        return v;
    } else if constexpr (4 * m == R) {
        return mul_mi<INV>(v);
    } else if constexpr (2 * m == R) {
        return make_float2(-v.x, -v.y);
    } else if constexpr (4 * m == 3 * R) {
        return mul_mi<!INV>(v);
    } else {
        constexpr float c = (float)unit_cos(m, R);
        constexpr float sn = INV ? (float)unit_sin(m, R) : -(float)unit_sin(m, R);
        return make_float2(c * v.x - sn * v.y, c * v.y + sn * v.x);
    }
}

template <int R>
struct DftSplit;  // R = R1 * R2 for the composite radices
template <> struct DftSplit<6> { static constexpr int R1 = 3, R2 = 2; };
template <> struct DftSplit<10> { static constexpr int R1 = 5, R2 = 2; };
template <> struct DftSplit<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct DftSplit<32> { static constexpr int R1 = 8, R2 = 4; };

// Composite R-point DFT in registers, natural order in and out: with j = j1 R2 + j2 and
// k = k1 + R1 k2, X_k = sum_j2 w_R2^(j2 k2) w_R^(j2 k1) sum_j1 w_R1^(j1 k1) x_j.
template <int R, bool INV>
struct DftComposite {
    __host__ __device__ __forceinline__ static void run(float2* v) {
        constexpr int R1 = DftSplit<R>::R1, R2 = DftSplit<R>::R2;
        float2 a[R];
        static_for<0, R2>([&](auto j2c) {
            constexpr int j2 = decltype(j2c)::value;
            float2 t[R1];
            static_for<0, R1>([&](auto j1c) { t[decltype(j1c)::value] = v[decltype(j1c)::value * R2 + j2]; });
            Dft<R1, INV>::run(t);
            static_for<0, R1>([&](auto k1c) {
                constexpr int k1 = decltype(k1c)::value;
                a[k1 * R2 + j2] = ctw<j2 * k1, R, INV>(t[k1]);
            });
        });
        static_for<0, R1>([&](auto k1c) {
            constexpr int k1 = decltype(k1c)::value;
            Dft<R2, INV>::run(a + k1 * R2);
            static_for<0, R2>([&](auto k2c) { v[k1 + R1 * decltype(k2c)::value] = a[k1 * R2 + decltype(k2c)::value]; });
        });
    }
};
template <bool INV> struct Dft<6, INV> : DftComposite<6, INV> {};
template <bool INV> struct Dft<10, INV> : DftComposite<10, INV> {};
template <bool INV> struct Dft<16, INV> : DftComposite<16, INV> {};
template <bool INV> struct Dft<32, INV> : DftComposite<32, INV> {};

// ------------------------------------------------------------------ one in-place stage
// OUT = false: results back to shared memory, then a block barrier.  OUT = true (the last
// stage of an inverse, st = 0, natural-order outputs e = q + r m of line w): results go to
// out(e, w, value) and there is no barrier (the caller synchronises before reusing s).
// PRE: each loaded value v of element e, line w becomes pre(e, w, v) first (a pointwise factor
// folded into the first stage an inverse executes).
struct NoOut {
    __device__ __forceinline__ void operator()(int, int, float2) const {}
};
struct NoPre {
    __device__ __forceinline__ float2 operator()(int, int, float2 v) const { return v; }
};
// Stage geometry: from the plan at run time (RtStage), or compile-time constants (CtStage: the
// strides become immediate offsets and the block division a constant one).  Both give the same
// butterflies in the same order, so the results are identical.
struct RtStage {
    int m, n, twoff;
    uint32_t magic;
    __device__ __forceinline__ RtStage(const FftPlan& pl, int st)
        : m(pl.m[st]), n(pl.n), twoff(pl.twoff[st]), magic(pl.magic[st]) {}
    __device__ __forceinline__ int div(int x) const { return m == 1 ? x : (int)__umulhi((unsigned)x, magic); }
};
template <int M, int N, int TWOFF>
struct CtStage {
    static constexpr int m = M, n = N, twoff = TWOFF;
    __device__ __forceinline__ static int div(int x) { return M == 1 ? x : x / M; }
};

// Row swizzle of a tile (SWR > 0, an even radix: the plan's stage with m = 1 has radix SWR and
// every other stage's m is a multiple of SWR): row e of the tile is stored at row
// e ^ ((e / SWR) & 1), so the m = 1 stage's butterflies of one warp (rows blk SWR + r of one
// parity before the swizzle) meet no bank twice.  Producers of such a tile write row e there.
template <int SWR>
__host__ __device__ __forceinline__ int tile_row(int e) { return SWR > 0 ? e ^ ((e / SWR) & 1) : e; }

// Butterflies [bf0, bf1) of the stage (bf1 < 0: all); SYNC: a block barrier at the end (in-place
// stages only); SWR > 0: rows in the tile_row<SWR> order (compile-time stages only).
template <int R, bool INV, int W, int SN, int T, bool OUT, bool PRE, class SP, class Out, class Pre,
          bool SYNC = true, int SWR = 0>
__device__ __forceinline__ void fft_stage_body(float2* __restrict__ s, const float2* __restrict__ tw, const SP& sp,
                                               Out&& out, Pre&& pre, const int bf0 = 0, const int bf1 = -1) {
    const int m = sp.m;
    const int nb = bf1 < 0 ? (sp.n / R) * W : bf1;
    const float2* tws = tw + sp.twoff - 1;
#pragma unroll(T >= 1024 ? 1 : 2)
    for (int bf = bf0 + threadIdx.x; bf < nb; bf += T) {
        const int j = bf / W, w = bf % W;
        const int blk = sp.div(j);
        const int q = j - blk * m;
        float2* p = s + (blk * R * m + q) * SN + w;
        float2 v[R];
        // element r at (r & 1 ? po : pe)[r m SN]
        float2 *pe = p, *po = p;
        if constexpr (SWR > 0) {
            // e = blk R m + q + r m: its row parity is q's (m even), and (e / SWR) & 1 is blk's for
            // m = 1, else (blk R K + q / SWR + r K) & 1 with K = m / SWR
            constexpr int M = SP::m;
            static_assert(SWR % 2 == 0 && (M == 1 ? R == SWR : M % SWR == 0), "row swizzle of another plan");
            if constexpr (M == 1) {
                const int f = (blk & 1) * SN;
                pe = p + f;
                po = p - f;
            } else {
                constexpr int K = M / SWR;
                const int A = (blk * R * K + q / SWR) & 1;
                const int d = (q & 1) ? -SN : SN;
                pe = p + (A ? d : 0);
                po = (K & 1) ? p + (A ? 0 : d) : pe;
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = (r & 1 ? po : pe)[r * m * SN];
        if constexpr (PRE) {
            const int e0 = blk * R * m + q;
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = pre(e0 + r * m, w, v[r]);
        }
        const float2* t = tws + q * (R - 1);   // t[r] = W_L^(r q), 1 <= r < R
        if (INV) {
            if (q != 0) {
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = cmulc(v[r], t[r]);
            }
            Dft<R, true>::run(v);
        } else {
            Dft<R, false>::run(v);
            if (q != 0) {
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = cmul(v[r], t[r]);
            }
        }
        if constexpr (OUT) {
#pragma unroll
            for (int r = 0; r < R; ++r) out(q + r * m, w, v[r]);
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) (r & 1 ? po : pe)[r * m * SN] = v[r];
        }
    }
    if constexpr (!OUT && SYNC) __syncthreads();
}

template <int R, bool INV, int W, int SN, int T, bool OUT = false, bool PRE = false, class Out = NoOut,
          class Pre = NoPre>
__device__ __forceinline__ void fft_stage(float2* __restrict__ s, const float2* __restrict__ tw,
                                          const FftPlan& pl, const int st, Out&& out = Out{}, Pre&& pre = Pre{}) {
    fft_stage_body<R, INV, W, SN, T, OUT, PRE>(s, tw, RtStage(pl, st), out, pre);
}

// Stage st of the compile-time plan of length NF.
template <int NF, int RMAX, int ST, bool INV, int W, int SN, int T, bool OUT = false, bool PRE = false,
          class Out = NoOut, class Pre = NoPre, int SWR = 0>
__device__ __forceinline__ void fft_stage_fixed(float2* __restrict__ s, const float2* __restrict__ tw,
                                                Out&& out = Out{}, Pre&& pre = Pre{}) {
    using FP = FixedPlan<NF, RMAX>;
    constexpr int R = FP::P.r[ST];
    static_assert(R <= RMAX, "fixed plan radix above the kernel's");
    using SP = CtStage<FP::P.m[ST], NF, FP::P.twoff[ST]>;
    fft_stage_body<R, INV, W, SN, T, OUT, PRE, SP, Out&, Pre&, true, SWR>(s, tw, SP{}, out, pre);
}

template <bool INV, int W, int SN, int T, int RMAX, bool OUT = false, bool PRE = false, class Out = NoOut,
          class Pre = NoPre>
__device__ __forceinline__ void fft_stage_any(float2* s, const float2* tw, const FftPlan& pl, int st,
                                              Out&& out = Out{}, Pre&& pre = Pre{}) {
    switch (pl.r[st]) {
        case 32:
            if constexpr (RMAX >= 32) fft_stage<32, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre);
            break;
        case 16:
            if constexpr (RMAX >= 16) fft_stage<16, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre);
            break;
        case 10:
            if constexpr (RMAX >= 16) fft_stage<10, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre);
            break;
        case 6:
            if constexpr (RMAX >= 16) fft_stage<6, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre);
            break;
        case 8: fft_stage<8, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre); break;
        case 4: fft_stage<4, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre); break;
        case 2: fft_stage<2, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre); break;
        case 3: fft_stage<3, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre); break;
        default: fft_stage<5, INV, W, SN, T, OUT, PRE>(s, tw, pl, st, out, pre); break;
    }
}

// Full transform of the W lines of the tile: forward natural -> digit-reversed, inverse
// digit-reversed -> natural (unnormalised).  tw holds the plan's per-stage twiddle tables
// (fill_stage_twiddles).  The caller synchronises after filling s; on
// return the block is synchronised.  The plan's radices must be <= RMAX (plan_fits; the
// launchers check it), larger radices are not compiled into the kernel.
template <bool INV, int W, int SN, int T, int RMAX = fft_max_radix(T), int NF = 0, int SWR = 0>
__device__ __forceinline__ void fft_tile(float2* __restrict__ s, const float2* __restrict__ tw,
                                         const FftPlan& pl) {
    static_assert(SWR == 0 || NF > 0, "row swizzle with compile-time plans only");
    if constexpr (NF > 0) {
        constexpr int NST = FixedPlan<NF, RMAX>::P.nst;
        static_for<0, NST>([&](auto c) {
            constexpr int st = INV ? NST - 1 - decltype(c)::value : decltype(c)::value;
            fft_stage_fixed<NF, RMAX, st, INV, W, SN, T, false, false, NoOut, NoPre, SWR>(s, tw);
        });
    } else if (!INV) {
        for (int st = 0; st < pl.nst; ++st) fft_stage_any<false, W, SN, T, RMAX>(s, tw, pl, st);
    } else {
        for (int st = pl.nst - 1; st >= 0; --st) fft_stage_any<true, W, SN, T, RMAX>(s, tw, pl, st);
    }
}

// Leading inverse stages (in execution order: NST-1, NST-2, ...) of the fixed plan whose groups of
// L = R m elements lie inside one of ns equal parts of the line (L divides NF / ns), at most
// NST - 1 (the last stage always runs on the whole line).
template <int NF, int RMAX>
__host__ __device__ constexpr int parts_depth(int ns) {
    using FP = FixedPlan<NF, RMAX>;
    int d = 0;
    for (int st = FP::P.nst - 1; st >= 1; --st) {
        const int L = FP::P.r[st] * FP::P.m[st];
        if ((NF / ns) % L != 0) break;
        ++d;
    }
    return d;
}

// Stage ST of the fixed plan on butterflies [bf0, bf1), no barrier.
template <int NF, int RMAX, int ST, bool INV, int W, int SN, int T>
__device__ __forceinline__ void fft_stage_fixed_range(float2* __restrict__ s, const float2* __restrict__ tw,
                                                      int bf0, int bf1) {
    using FP = FixedPlan<NF, RMAX>;
    constexpr int R = FP::P.r[ST];
    using SP = CtStage<FP::P.m[ST], NF, FP::P.twoff[ST]>;
    fft_stage_body<R, INV, W, SN, T, false, false, SP, NoOut, NoPre, false>(s, tw, SP{}, NoOut{}, NoPre{}, bf0, bf1);
}

// The inverse of ifft_tile_out for a fixed plan, with the elements in ns equal parts: the D
// leading stages whose groups lie inside one part (parts_depth) run part by part, wait(p) called
// before part p >= 1 (the caller has the first part), then after() once every part is done
// (after a block barrier), then the other stages.  Lets the later parts of a tile still be
// arriving while the first are transformed.  D must be 1 or 2 (the plans of the tile variants).
template <int W, int SN, int T, int RMAX, int NF, int D, class Wait, class After, class Out>
__device__ __forceinline__ void ifft_tile_out_parts(float2* __restrict__ s, const float2* __restrict__ tw,
                                                    const int ns, Wait&& wait, After&& after, Out&& out) {
    using FP = FixedPlan<NF, RMAX>;
    constexpr int NST = FP::P.nst;
    static_assert(D >= 1 && D <= 2 && D <= NST - 1, "parts need one or two leading part-local stages");
    constexpr int S0 = NST - 1, S1 = NST - 2;
    constexpr int NB0 = (NF / FP::P.r[S0]) * W, NB1 = (NF / FP::P.r[S1 >= 0 ? S1 : 0]) * W;
    for (int p = 0; p < ns; ++p) {
        if (p) wait(p);
        fft_stage_fixed_range<NF, RMAX, S0, true, W, SN, T>(s, tw, p * (NB0 / ns), (p + 1) * (NB0 / ns));
        if constexpr (D == 2) {
            __syncthreads();
            fft_stage_fixed_range<NF, RMAX, S1, true, W, SN, T>(s, tw, p * (NB1 / ns), (p + 1) * (NB1 / ns));
        }
    }
    __syncthreads();
    after();
    static_for<D, NST - 1>([&](auto c) {
        fft_stage_fixed<NF, RMAX, NST - 1 - decltype(c)::value, true, W, SN, T>(s, tw);
    });
    fft_stage_fixed<NF, RMAX, 0, true, W, SN, T, true>(s, tw, out);
}

// Inverse of the W lines with the last stage's natural-order results handed to out(e, w, v)
// (element e of line w) instead of written back: every stage but the last ends with a block
// barrier; the caller synchronises before it reuses s.
// SWR > 0 (compile-time plans): the tile's rows in the tile_row<SWR> order.
template <int W, int SN, int T, int RMAX, int NF = 0, int SWR = 0, class Out>
__device__ __forceinline__ void ifft_tile_out(float2* __restrict__ s, const float2* __restrict__ tw,
                                              const FftPlan& pl, Out&& out) {
    static_assert(SWR == 0 || NF > 0, "row swizzle with compile-time plans only");
    if constexpr (NF > 0) {
        constexpr int NST = FixedPlan<NF, RMAX>::P.nst;
        static_for<0, NST - 1>([&](auto c) {
            fft_stage_fixed<NF, RMAX, NST - 1 - decltype(c)::value, true, W, SN, T, false, false, NoOut, NoPre, SWR>(
                s, tw);
        });
        fft_stage_fixed<NF, RMAX, 0, true, W, SN, T, true, false, Out&, NoPre, SWR>(s, tw, out);
    } else {
        for (int st = pl.nst - 1; st >= 1; --st) fft_stage_any<true, W, SN, T, RMAX>(s, tw, pl, st);
        fft_stage_any<true, W, SN, T, RMAX, true>(s, tw, pl, 0, out);
    }
}

// Per-stage twiddle tables of the plan (FftPlan::twoff; fewer than n entries), filled by the
// block (no barrier).
__device__ __forceinline__ void fill_stage_twiddles(float2* stw, const FftPlan& pl) {
    for (int i = threadIdx.x; i < pl.twn; i += blockDim.x) {
        int st = 0;
        while (st + 1 < pl.nst && pl.twoff[st + 1] <= i) ++st;
        const int loc = i - pl.twoff[st];
        const int q = loc / (pl.r[st] - 1), r = loc - q * (pl.r[st] - 1) + 1;
        stw[i] = twiddle(r * q * pl.tstep[st], pl.n);
    }
}


}  // namespace smk
