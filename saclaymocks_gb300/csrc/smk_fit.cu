// The (a,b,c) fit on GB300: mean flux per redshift bin, binned 1D power spectrum of
// dF = F/<F> - 1, and the exact adjoint of the loss
//     L = sum_j (<F>_j - Fbar*_j)^2 + sum_b ((P_b - P*_b)/P*_b)^2
// with per-bin FGPA parameters theta_j = (a_j, b_j, c_j) (the fit of
// py/SaclayMocks/fit_az.py:194-279, with gradients instead of Migrad's finite differences).
//
// Pixels are never stored: every kernel recomputes F = exp(-a exp(b G (delta + c eta))) from
// the fixed fields (delta = delta_l + delta_s, eta_par, G, redshift bin) and the parameters.
//   fit_flux_kernel     F per pixel -> sum F per z bin and over all pixels (FP64)
//   fit_p1d_kernel      per pair of equal-length skewers: dF, length-N DFT by Bluestein's chirp
//                       transform on the FFT engine, |X_m|^2 dx/N binned in log-k (FP64)
//   fit_adjoint_kernel  per pair: X (read back from the forward's store, or recomputed),
//                       back-propagate the P1D weights through the inverse DFT (Bluestein
//                       again), then accumulate per bin
//                       A_j = sum (gM_j + gdF/<F>) dF/dtheta_j, B_j = sum dF/dtheta_j and
//                       S = sum gdF * F, so that dL/dtheta_j = A_j - S B_j / (n <F>^2)
//                       (the coupling through the global mean <F> needs no second pass).
#include <algorithm>
#include <vector>

#include "smk_fft.cuh"

namespace smk {

constexpr int FIT_T = 256;
constexpr int FIT_MAX_BINS = 64;

struct FitArgs {
    const float* delta;
    const float* eta;      // may be null (no RSD)
    const float* G;        // may be null (G = 1)
    const int16_t* zbin;   // [npix_total], 0..nzb-1
    const int64_t* offset;
    const int32_t* npix;
    const int32_t* order;  // pairs of equal length (-1: empty)
    int64_t n_items;
    int64_t n_total;       // pixels
    int nzb, nkb;
    const float* theta;    // [nzb][3]
    const double* kedges;  // [nkb + 1] log-k edges (h/Mpc)
    double dx;
    double* acc;           // accumulators, layout in smk_fit_acc_layout
    const double* gM;      // backward: dL/d<F>_j / n_j            [nzb]
    const double* gP;      // backward: dL/dP_b / count_b          [nkb]
    unsigned long long* counter;
    int mmax;              // largest Bluestein length of the problem: smem = s1 | s2 | tw of mmax each
    const float2* chirp;   // optional: FFT_M of the forward chirp of every length N, digit-reversed
    const int64_t* chirp_off;  // [FFT_MAX_N / 2 + 1]: offset (complex) of length N in chirp, or -1
    float2* spec;          // optional: the forward stores each pair's DFT at its first offset,
                           // the backward reads it back (no second forward transform)
};

// accumulator layout (doubles)
__host__ __device__ inline int acc_fsum(int) { return 0; }                       // [nzb]
__host__ __device__ inline int acc_ftot(int nzb) { return nzb; }                 // [1]
__host__ __device__ inline int acc_psum(int nzb) { return nzb + 1; }             // [nkb]
__host__ __device__ inline int acc_A(int nzb, int nkb) { return nzb + 1 + nkb; }  // [nzb][3]
__host__ __device__ inline int acc_B(int nzb, int nkb) { return 2 * nzb + 1 + nkb + 2 * nzb; }  // [nzb][3]
__host__ __device__ inline int acc_S(int nzb, int nkb) { return 7 * nzb + 1 + nkb; }  // [1]
__host__ __device__ inline int acc_psq(int nzb, int nkb) { return 7 * nzb + 2 + nkb; }  // [nkb]
__host__ __device__ inline int acc_len(int nzb, int nkb) { return 7 * nzb + 2 + 2 * nkb; }

__device__ __forceinline__ float flux_of(const FitArgs& a, int64_t o, const float* th, float* tau1, float* g) {
    const int j = a.zbin[o];
    const float pa = th[3 * j], pb = th[3 * j + 1], pc = th[3 * j + 2];
    const float e = a.eta ? __ldg(a.eta + o) : 0.f;
    const float G = a.G ? __ldg(a.G + o) : 1.f;
    const float gg = __ldg(a.delta + o) + pc * e;
    const float t = expf(pb * G * gg);
    *tau1 = t;
    *g = gg;
    return expf(-pa * t);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Warp-cooperative flush of per-lane FP32 partials v[0..K) that belong to redshift bin jw: the
// lanes with `flush` set (and jw >= 0) are grouped by bin, each group warp-summed and added by
// lane 0 to dst(bin, q) (FP64 shared memory) -- one atomic per distinct bin and value instead of
// one per lane, so the lanes of a block that all sit in one bin do not queue on one address.
// Those lanes leave with zeroed partials and jw = -1.  All 32 lanes must call it.
template <int K, class Dst>
__device__ __forceinline__ void warp_flush(bool flush, int& jw, float (&v)[K], Dst&& dst) {
    for (;;) {
        const unsigned act = __ballot_sync(0xffffffffu, flush && jw >= 0);
        if (!act) break;
        const int jl = __shfl_sync(0xffffffffu, jw, __ffs(act) - 1);
        const bool mine = flush && jw == jl;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float sum = warp_sum(mine ? v[q] : 0.f);
            if ((threadIdx.x & 31) == 0) atomicAdd(dst(jl, q), (double)sum);
        }
        if (mine) {
#pragma unroll
            for (int q = 0; q < K; ++q) v[q] = 0.f;
            jw = -1;
        }
    }
}

// ------------------------------------------------------------------ pass 1: mean flux
constexpr int FIT_RUN = 32 * 16;   // pixels per warp work run of the mean-flux pass

__global__ void __launch_bounds__(FIT_T) fit_flux_kernel(const FitArgs a) {
    __shared__ double sb[FIT_MAX_BINS + 1];
    __shared__ float th[3 * FIT_MAX_BINS];
    for (int i = threadIdx.x; i <= a.nzb; i += FIT_T) sb[i] = 0.0;
    for (int i = threadIdx.x; i < 3 * a.nzb; i += FIT_T) th[i] = a.theta[i];
    __syncthreads();
    // warps take runs of FIT_RUN consecutive pixels, lanes on consecutive pixels; each lane keeps
    // an FP32 partial of its current bin (16 pixels at most), flushed in FP64 per bin change
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (FIT_T / 32);
    for (int64_t base = (blockIdx.x * (int64_t)(FIT_T / 32) + (threadIdx.x >> 5)) * FIT_RUN; base < a.n_total;
         base += nw * FIT_RUN) {
        const int64_t end = min(base + (int64_t)FIT_RUN, a.n_total);
        float part[1] = {0.f}, tot[1] = {0.f};
        int jw = -1, jt = 0;
        for (int64_t o0 = base; o0 < end; o0 += 32) {   // warp-uniform trip count
            const int64_t o = o0 + lane;
            const bool ok = o < end;
            float F = 0.f;
            int j = -1;
            if (ok) {
                float t1, g;
                F = flux_of(a, o, th, &t1, &g);
                j = a.zbin[o];
            }
            const bool change = ok && jw >= 0 && j != jw;
            if (__any_sync(0xffffffffu, change)) warp_flush(change, jw, part, [&](int b, int) { return &sb[b]; });
            if (ok) {
                if (jw < 0) jw = j;
                part[0] += F;
                tot[0] += F;
            }
        }
        warp_flush(true, jw, part, [&](int b, int) { return &sb[b]; });
        warp_flush(true, jt, tot, [&](int, int) { return &sb[a.nzb]; });
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= a.nzb; i += FIT_T) atomicAdd(a.acc + i, sb[i]);
}

// ------------------------------------------------------------------ Bluestein DFT helpers
// chirp w_n = exp(-i pi n^2 / N) = exp(-2 pi i r / 2N), r = n^2 mod 2N (exact integers;
// n < N <= 2048, so n^2 fits 32 bits)
__device__ __forceinline__ float2 chirp(int n, int N) {
    const int r = (n * n) % (2 * N);
    return twiddle(r, 2 * N);
}

// Smallest M = 2^a 3^b 5^c >= 2N - 1 (N <= 2048, so M <= 4096): the cyclic convolution length
// of Bluestein's transform, a length the mixed-radix engine runs.
__host__ __device__ inline int bluestein_m(int N) {
    for (int M = 2 * N - 1;; ++M) {
        int m = M;
        while (m % 2 == 0) m /= 2;
        while (m % 3 == 0) m /= 3;
        while (m % 5 == 0) m /= 5;
        if (m == 1 && M >= 2) return M;
    }
}

// Forward chirp of length N wrapped into M slots: b_d = conj(w_d) at d and M - d, |d| < N.  It
// is even (b_d = b_{M-d}), so its DFT is even and the inverse transform's chirp spectrum
// FFT(conj b) is the elementwise conjugate of FFT(b).
__device__ __forceinline__ float2 chirp_b(int n, int N, int M) {
    const int d = n < N ? n : (n > M - N ? M - n : -1);
    if (d < 0) return make_float2(0.f, 0.f);
    const float2 w = chirp(d, N);
    return make_float2(w.x, -w.y);
}

// Unnormalised length-N DFTs of the W complex sequences held in s1 (element n of line w at
// s1[n W + w], natural order), forward (e^{-}) or inverse (e^{+}); results left in place in
// natural order.  s2 is scratch of M elements; tw the twiddle table of M.  Bc (may be null):
// FFT_M of the forward chirp in the engine's digit-reversed order, which saves one of the
// three transforms, followed by the chirp w_n itself for n < N (the same values chirp()
// computes).  Every line gets the same operations as a W = 1 call.  Block-synchronous.
template <bool INV, int W>
__device__ void bluestein(float2* s1, float2* s2, const float2* tw, int N, int M, const FftPlan& pl,
                          const float2* __restrict__ Bc) {
    const float2* __restrict__ Wt = Bc ? Bc + M : nullptr;
    // a_n = x_n w_n (INV: x_n conj(w_n)); b = the chirp (INV: its conjugate)
    for (int i = threadIdx.x; i < M * W; i += FIT_T) {
        const int n = i / W;
        if (n < N) {
            const float2 w = Wt ? __ldg(Wt + n) : chirp(n, N);
            s1[i] = INV ? cmulc(s1[i], w) : cmul(s1[i], w);
        } else {
            s1[i] = make_float2(0.f, 0.f);
        }
    }
    if (!Bc) {
        for (int n = threadIdx.x; n < M; n += FIT_T) {
            const float2 b = chirp_b(n, N, M);
            s2[n] = INV ? make_float2(b.x, -b.y) : b;
        }
    }
    __syncthreads();
    fft_tile<false, W, W, FIT_T, 16>(s1, tw, pl);
    if (Bc) {
        for (int i = threadIdx.x; i < M * W; i += FIT_T) {
            const float2 b = __ldg(Bc + i / W);
            s1[i] = cmul(s1[i], INV ? make_float2(b.x, -b.y) : b);   // digit-reversed, same order
        }
    } else {
        fft_tile<false, 1, 1, FIT_T, 16>(s2, tw, pl);
        for (int i = threadIdx.x; i < M * W; i += FIT_T) s1[i] = cmul(s1[i], s2[i / W]);  // digit-reversed
    }
    __syncthreads();
    fft_tile<true, W, W, FIT_T, 16>(s1, tw, pl);
    const float inv_m = 1.0f / (float)M;
    for (int i = threadIdx.x; i < N * W; i += FIT_T) {
        const int k = i / W;
        const float2 w = Wt ? __ldg(Wt + k) : chirp(k, N);
        const float2 c = cscale(s1[i], inv_m);
        s1[i] = INV ? cmulc(c, w) : cmul(c, w);
    }
    __syncthreads();
}

// Frequency k_m of mode m of a length-N spectrum: numpy's rfftfreq(N)*2*k_ny in FP64.  Its bin
// is searchsorted(edges, k_m, 'right') - 1 with the last edge inclusive, -1 outside the edges.
__device__ __forceinline__ double kfreq(int m, int N, double kfac) { return ((double)m * (1.0 / (double)N)) * kfac; }

// The bins as integer thresholds on m, once per length (k_m is nondecreasing in m):
// thr[b] (b < nkb) = the smallest m with k_m >= edges[b], thr[nkb] = the smallest m with
// k_m > edges[nkb] (m up to N/2 + 1).  Block-synchronous.
__device__ void kbin_thresholds(int N, double kfac, const double* edges, int nkb, int* thr) {
    const int half = N / 2;
    for (int b = threadIdx.x; b <= nkb; b += FIT_T) {
        const double e = edges[b];
        int m = (int)fmin(fmax(floor(e * (double)N / kfac), 0.0), (double)(half + 1));
        if (b < nkb) {
            while (m > 0 && kfreq(m - 1, N, kfac) >= e) --m;
            while (m <= half && kfreq(m, N, kfac) < e) ++m;
        } else {
            while (m > 0 && kfreq(m - 1, N, kfac) > e) --m;
            while (m <= half && kfreq(m, N, kfac) <= e) ++m;
        }
        thr[b] = m;
    }
    __syncthreads();
}

// The bin of mode m from the thresholds: the largest b < nkb with thr[b] <= m, -1 outside
// [thr[0], thr[nkb]).
__device__ __forceinline__ int kbin_thr(int m, const int* thr, int nkb) {
    if (m < thr[0] || m >= thr[nkb]) return -1;
    int lo = 0, hi = nkb;  // thr[lo] <= m, and hi == nkb or thr[hi] > m
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (thr[mid] <= m) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Work item of the fit kernels: two consecutive pairs of the schedule (pairs of equal-length
// skewers, longest first).  Pair p holds skewers sid[2p] (always present) and sid[2p + 1] (or
// -1); np = 1 when the schedule ended after the first pair.  Two pairs of one length run as the
// two lines of one tile (W = 2), else one after the other (W = 1).
struct Quad {
    int sid[4];
    int N[2];
    int np;
    int64_t off[4];
};

__device__ bool next_quad(const FitArgs& a, long long* item_sh, Quad* qd) {
    if (threadIdx.x == 0) *item_sh = (long long)atomicAdd(a.counter, 1ULL);
    __syncthreads();
    const long long q = *item_sh;
    if (q >= (a.n_items + 1) / 2) return false;
    if (threadIdx.x < 4) {
        const long long item = 2 * q + (threadIdx.x >> 1);
        const int sid = item < a.n_items ? a.order[2 * item + (threadIdx.x & 1)] : -1;
        qd->sid[threadIdx.x] = sid;
        qd->off[threadIdx.x] = sid >= 0 ? a.offset[sid] : 0;
        if ((threadIdx.x & 1) == 0) qd->N[threadIdx.x >> 1] = sid >= 0 ? a.npix[sid] : 0;
        if (threadIdx.x == 0) qd->np = 2 * q + 1 < a.n_items ? 2 : 1;
    }
    __syncthreads();
    return true;
}

// dF of the W pairs p0 .. p0 + W - 1 into s1: line w holds pair p0 + w's skewers as re / im
// (element n at s1[n W + w]); each line's pixels are read consecutively.
template <int W>
__device__ void load_pairs(const FitArgs& a, const float* th, float fbar_inv, const Quad& qd, int p0, float2* s1) {
    const int N = qd.N[p0];
    for (int i = threadIdx.x; i < N * W; i += FIT_T) {
        const int w = i / N, n = i - w * N;
        float v[2] = {0.f, 0.f};
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const int q = 2 * (p0 + w) + t;
            if (qd.sid[q] >= 0) {
                float t1, g;
                v[t] = flux_of(a, qd.off[q] + n, th, &t1, &g) * fbar_inv - 1.0f;
            }
        }
        s1[n * W + w] = make_float2(v[0], v[1]);
    }
    __syncthreads();
}

// Per-length state of a block: the plan and twiddles of M, the k-bin thresholds of N.
struct LengthState {
    int curM, curN;
};

// Prepares a group of length N (Bluestein length M): false (and a NaN in *nan_at) when M is above
// the shared memory's mmax or the chirp table lacks N and there is no room to transform it.
__device__ bool prepare_length(const FitArgs& a, int N, int M, FftPlan& pl, float2* tw, int* thr, const double* edges,
                               double kfac, float2* s2, LengthState& ls, double* nan_at, const float2** Bc) {
    if (N != ls.curN) {
        kbin_thresholds(N, kfac, edges, a.nkb, thr);
        ls.curN = N;
    }
    *Bc = a.chirp && a.chirp_off[N] >= 0 ? a.chirp + a.chirp_off[N] : nullptr;
    if (M > a.mmax || (!*Bc && !s2)) {
        // a skewer longer than SmkFitProblem.n_max (its Bluestein length does not fit the shared
        // memory), or a length missing from the chirp table: not transformed, the sums made NaN
        if (threadIdx.x == 0) *nan_at = __longlong_as_double(0x7ff8000000000000LL);
        __syncthreads();
        return false;
    }
    if (M != ls.curM) {
        if (threadIdx.x == 0) make_plan(M, &pl, 16);
        __syncthreads();
        fill_stage_twiddles(tw, pl);
        ls.curM = M;
    }
    return true;
}

// Add `v` to sbins[bin] for every lane: lanes hold consecutive frequencies so equal bins form
// contiguous runs; each run is summed by a segmented shuffle scan and its first lane issues
// one shared-memory FP64 atomic (bin < 0: nothing).
__device__ __forceinline__ void warp_bin_add(double* sbins, int bin, float v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float v2 = __shfl_down_sync(0xffffffffu, v, off);
        const int b2 = __shfl_down_sync(0xffffffffu, bin, off);
        if (lane + off < 32 && b2 == bin) v += v2;
    }
    const int bprev = __shfl_up_sync(0xffffffffu, bin, 1);
    if (bin >= 0 && (lane == 0 || bprev != bin)) atomicAdd(&sbins[bin], (double)v);
}


// ------------------------------------------------------------------ pass 2: binned P1D
// Shared memory of the fit kernels: s1 (two lines of mmax) | s2 (mmax, only without the chirp
// table) | tw (mmax).
struct FitSmem {
    float2 *s1, *s2, *tw;
    __device__ FitSmem(float2* smem, const FitArgs& a)
        : s1(smem), s2(a.chirp ? nullptr : smem + 2 * a.mmax), tw(smem + (a.chirp ? 2 : 3) * a.mmax) {}
};

// The P1D of the W pairs p0 .. p0 + W - 1 of qd (one length N): transform, store the packed
// spectra for the backward, bin |X_m|^2 dx/N of every skewer.
template <int W>
__device__ void p1d_group(const FitArgs& a, const Quad& qd, int p0, const FitSmem& sm, FftPlan& pl, int* thr,
                          const double* edges, double kfac, const float* th, float fbar_inv, double* psum,
                          double* psq, LengthState& ls) {
    const int N = qd.N[p0];
    const int M = bluestein_m(N);
    const float2* Bc;
    if (!prepare_length(a, N, M, pl, sm.tw, thr, edges, kfac, sm.s2, ls, &psum[0], &Bc)) return;
    load_pairs<W>(a, th, fbar_inv, qd, p0, sm.s1);
    bluestein<false, W>(sm.s1, sm.s2, sm.tw, N, M, pl, Bc);
    if (a.spec) {   // the packed spectra Z for the backward (s1 is only read below)
        for (int i = threadIdx.x; i < N * W; i += FIT_T) {
            const int w = i / N, m = i - w * N;
            a.spec[qd.off[2 * (p0 + w)] + m] = sm.s1[m * W + w];
        }
    }
    // X1_m = (Z_m + Z*_{N-m})/2, X2_m = (Z_m - Z*_{N-m})/(2i), m = 0..N/2; one bin for all lines
    const float norm = (float)(a.dx / (double)N);
    const int half = N / 2;
    for (int m0 = 0; m0 <= half; m0 += FIT_T) {    // block-uniform trip count
        const int m = m0 + (int)threadIdx.x;
        int b = -1;
        float p = 0.f, q = 0.f;
        if (m <= half) {
            b = kbin_thr(m, thr, a.nkb);
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const float2 zk = sm.s1[m * W + w], zm = sm.s1[(m == 0 ? 0 : N - m) * W + w];
                const float x1r = 0.5f * (zk.x + zm.x), x1i = 0.5f * (zk.y - zm.y);
                const float x2r = 0.5f * (zk.y + zm.y), x2i = -0.5f * (zk.x - zm.x);
                const float p1 = (x1r * x1r + x1i * x1i) * norm;
                const float p2 = qd.sid[2 * (p0 + w) + 1] >= 0 ? (x2r * x2r + x2i * x2i) * norm : 0.f;
                p += p1 + p2;
                q += p1 * p1 + p2 * p2;
            }
        }
        warp_bin_add(psum, b, p);
        warp_bin_add(psq, b, q);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(FIT_T, 3) fit_p1d_kernel(const FitArgs a) {
    extern __shared__ float2 smem[];
    const FitSmem sm(smem, a);
    __shared__ double psum[FIT_MAX_BINS];
    __shared__ double psq[FIT_MAX_BINS];
    __shared__ double edges[FIT_MAX_BINS + 1];
    __shared__ float th[3 * FIT_MAX_BINS];
    __shared__ long long item_sh;
    __shared__ Quad qd;
    for (int i = threadIdx.x; i < a.nkb; i += FIT_T) psum[i] = psq[i] = 0.0;
    for (int i = threadIdx.x; i <= a.nkb; i += FIT_T) edges[i] = a.kedges[i];
    for (int i = threadIdx.x; i < 3 * a.nzb; i += FIT_T) th[i] = a.theta[i];
    const float fbar_inv = (float)((double)a.n_total / a.acc[acc_ftot(a.nzb)]);
    const double kfac = 2.0 * (3.14159265358979323846 / a.dx);
    __shared__ FftPlan pl;
    __shared__ int thr[FIT_MAX_BINS + 1];
    LengthState ls{0, 0};
    while (next_quad(a, &item_sh, &qd)) {
        if (qd.np == 2 && qd.N[1] == qd.N[0]) {
            p1d_group<2>(a, qd, 0, sm, pl, thr, edges, kfac, th, fbar_inv, psum, psq, ls);
        } else {
            p1d_group<1>(a, qd, 0, sm, pl, thr, edges, kfac, th, fbar_inv, psum, psq, ls);
            if (qd.np == 2) p1d_group<1>(a, qd, 1, sm, pl, thr, edges, kfac, th, fbar_inv, psum, psq, ls);
        }
    }
    for (int i = threadIdx.x; i < a.nkb; i += FIT_T) {
        atomicAdd(a.acc + acc_psum(a.nzb) + i, psum[i]);
        atomicAdd(a.acc + acc_psq(a.nzb, a.nkb) + i, psq[i]);
    }
}

// ------------------------------------------------------------------ backward
// Shared state of the adjoint pass's blocks.
struct AdjShared {
    double* sA;
    double* sB;
    double* sS;
    const float* gP;
    const float* gM;
};

// The adjoint of the W pairs p0 .. p0 + W - 1 of qd (one length N): their spectra (read back or
// transformed again), the P1D weights applied, the inverse DFT (Bluestein), and the per-bin
// accumulation of every pixel of the 2 W skewers.
template <int W>
__device__ void adjoint_group(const FitArgs& a, const Quad& qd, int p0, const FitSmem& sm, FftPlan& pl, int* thr,
                              const double* edges, double kfac, const float* th, float fbar_inv,
                              const AdjShared& sh, LengthState& ls) {
    const int N = qd.N[p0];
    const int M = bluestein_m(N);
    const float2* Bc;
    if (!prepare_length(a, N, M, pl, sm.tw, thr, edges, kfac, sm.s2, ls, sh.sS, &Bc)) return;
    float2* s1 = sm.s1;
    if (a.spec) {   // Z as the forward pass with the same theta left it
        for (int i = threadIdx.x; i < N * W; i += FIT_T) {
            const int w = i / N, m = i - w * N;
            s1[m * W + w] = a.spec[qd.off[2 * (p0 + w)] + m];
        }
        __syncthreads();
    } else {
        load_pairs<W>(a, th, fbar_inv, qd, p0, s1);
        bluestein<false, W>(s1, sm.s2, sm.tw, N, M, pl, Bc);
    }
    // V_t (Hermitian): V_m = w_m X_m (0<m<N/2), V_{N-m} = conj; V_0, V_{N/2} = 2 Re(w X);
    // packed W = V_1 + i V_2; the unnormalised inverse DFT of W is gdF_1 + i gdF_2.
    const float norm = (float)(a.dx / (double)N);
    for (int m = threadIdx.x; m <= N / 2; m += FIT_T) {
        const int b = kbin_thr(m, thr, a.nkb);
        const float wgt = b >= 0 ? sh.gP[b] * norm : 0.f;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const float2 zk = s1[m * W + w], zm = s1[(m == 0 ? 0 : N - m) * W + w];
            float2 x1 = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            float2 x2 = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
            if (qd.sid[2 * (p0 + w) + 1] < 0) x2 = make_float2(0.f, 0.f);
            x1 = cscale(x1, wgt);
            x2 = cscale(x2, wgt);
            // in place: this thread alone reads and writes the slots m and N - m of the line
            if (m == 0 || 2 * m == N) {
                s1[m * W + w] = make_float2(2.f * x1.x, 2.f * x2.x);
            } else {
                s1[m * W + w] = make_float2(x1.x - x2.y, x1.y + x2.x);          // V1_m + i V2_m
                s1[(N - m) * W + w] = make_float2(x1.x + x2.y, x2.x - x1.y);    // conj(V1_m) + i conj(V2_m)
            }
        }
    }
    __syncthreads();
    bluestein<true, W>(s1, sm.s2, sm.tw, N, M, pl, Bc);
    // per pixel: gF~ = gM_j + gdF / <F>; dF/da = -tau1 F, dF/db = -a tau1 G g F,
    // dF/dc = -a tau1 b G eta F.  Each warp walks a contiguous run of the group's 2 W N pixel
    // slots (skewer by skewer, lanes on consecutive pixels); per-lane FP32 partials of the
    // current redshift bin are flushed to the block's FP64 accumulators when the bin changes
    // (warp_flush)
    {
        const int total = 2 * W * N;
        const int per_warp = ((total + FIT_T / 32 - 1) / (FIT_T / 32) + 31) & ~31;
        const int lane = threadIdx.x & 31;
        const int beg = (threadIdx.x >> 5) * per_warp, end = min(total, beg + per_warp);
        float acc6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, accS[1] = {0.f};
        int jw = -1, js = 0;
        auto dst6 = [&](int b, int q) { return q < 3 ? &sh.sA[3 * b + q] : &sh.sB[3 * b + q - 3]; };
        for (int i0 = beg; i0 < end; i0 += 32) {   // warp-uniform trip count
            const int i = i0 + lane;
            const int sk = i / N;                   // skewer 0 .. 2W - 1 of the group
            const int ii = i - sk * N;
            const int w = sk >> 1, t = sk & 1;
            const bool ok = i < end && qd.sid[2 * p0 + sk] >= 0;
            int j = -1;
            float v6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, vS = 0.f;
            if (ok) {
                const int64_t o = qd.off[2 * p0 + sk] + ii;
                float t1, g;
                const float F = flux_of(a, o, th, &t1, &g);
                const float2 z = s1[ii * W + w];
                const float gdF = t ? z.y : z.x;
                j = a.zbin[o];
                const float pa = th[3 * j], pb = th[3 * j + 1];
                const float e = a.eta ? __ldg(a.eta + o) : 0.f;
                const float G = a.G ? __ldg(a.G + o) : 1.f;
                const float dFa = -t1 * F;
                const float dFb = -pa * t1 * G * g * F;
                const float dFc = -pa * t1 * pb * G * e * F;
                const float gF = sh.gM[j] + gdF * fbar_inv;
                v6[0] = gF * dFa;
                v6[1] = gF * dFb;
                v6[2] = gF * dFc;
                v6[3] = dFa;
                v6[4] = dFb;
                v6[5] = dFc;
                vS = gdF * F;
            }
            const bool change = ok && jw >= 0 && j != jw;
            if (__any_sync(0xffffffffu, change)) warp_flush(change, jw, acc6, dst6);
            if (ok) {
                if (jw < 0) jw = j;
#pragma unroll
                for (int q = 0; q < 6; ++q) acc6[q] += v6[q];
                accS[0] += vS;
            }
        }
        warp_flush(true, jw, acc6, dst6);
        warp_flush(true, js, accS, [&](int, int) { return sh.sS; });
    }
    __syncthreads();
}

__global__ void __launch_bounds__(FIT_T, 3) fit_adjoint_kernel(const FitArgs a) {
    extern __shared__ float2 smem[];
    const FitSmem sm(smem, a);
    __shared__ double sA[3 * FIT_MAX_BINS], sB[3 * FIT_MAX_BINS], sS;
    __shared__ double edges[FIT_MAX_BINS + 1];
    __shared__ float gP[FIT_MAX_BINS], gM[FIT_MAX_BINS];   // the weights in FP32 (no FP64 per pixel)
    __shared__ float th[3 * FIT_MAX_BINS];
    __shared__ long long item_sh;
    __shared__ Quad qd;
    for (int i = threadIdx.x; i < 3 * a.nzb; i += FIT_T) {
        sA[i] = 0.0;
        sB[i] = 0.0;
        th[i] = a.theta[i];
    }
    for (int i = threadIdx.x; i <= a.nkb; i += FIT_T) edges[i] = a.kedges[i];
    for (int i = threadIdx.x; i < a.nkb; i += FIT_T) gP[i] = (float)a.gP[i];
    for (int i = threadIdx.x; i < a.nzb; i += FIT_T) gM[i] = (float)a.gM[i];
    if (threadIdx.x == 0) sS = 0.0;
    // the same FP32 1/<F> as the forward pass (the stored spectra were made with it)
    const float fbar_inv = (float)((double)a.n_total / a.acc[acc_ftot(a.nzb)]);
    const double kfac = 2.0 * (3.14159265358979323846 / a.dx);
    __shared__ FftPlan pl;
    __shared__ int thr[FIT_MAX_BINS + 1];
    const AdjShared sh{sA, sB, &sS, gP, gM};
    LengthState ls{0, 0};
    while (next_quad(a, &item_sh, &qd)) {
        if (qd.np == 2 && qd.N[1] == qd.N[0]) {
            adjoint_group<2>(a, qd, 0, sm, pl, thr, edges, kfac, th, fbar_inv, sh, ls);
        } else {
            adjoint_group<1>(a, qd, 0, sm, pl, thr, edges, kfac, th, fbar_inv, sh, ls);
            if (qd.np == 2) adjoint_group<1>(a, qd, 1, sm, pl, thr, edges, kfac, th, fbar_inv, sh, ls);
        }
    }
    double* A = a.acc + acc_A(a.nzb, a.nkb);
    double* B = a.acc + acc_B(a.nzb, a.nkb);
    for (int i = threadIdx.x; i < 3 * a.nzb; i += FIT_T) {
        atomicAdd(A + i, sA[i]);
        atomicAdd(B + i, sB[i]);
    }
    if (threadIdx.x == 0) atomicAdd(a.acc + acc_S(a.nzb, a.nkb), sS);
}

// FFT_M of the forward chirp of each length (one block per length), in the order the engine
// leaves a forward transform: the same arithmetic as bluestein() without a table; then the
// chirp w_n itself for n < N.
__global__ void __launch_bounds__(FIT_T) fit_chirp_kernel(const int32_t* lengths, const int64_t* offsets,
                                                          float2* out) {
    extern __shared__ float2 smem[];
    float2* s = smem;
    float2* tw = smem + FFT_MAX_N;
    __shared__ FftPlan pl;
    const int N = lengths[blockIdx.x];
    const int M = bluestein_m(N);
    if (threadIdx.x == 0) make_plan(M, &pl, 16);
    __syncthreads();
    fill_stage_twiddles(tw, pl);
    for (int n = threadIdx.x; n < M; n += FIT_T) s[n] = chirp_b(n, N, M);
    __syncthreads();
    fft_tile<false, 1, 1, FIT_T, 16>(s, tw, pl);
    float2* o = out + offsets[blockIdx.x];
    for (int n = threadIdx.x; n < M; n += FIT_T) o[n] = s[n];
    for (int n = threadIdx.x; n < N; n += FIT_T) o[M + n] = chirp(n, N);
}

static int fit_grid(const void* kernel, size_t smem, int64_t items, int* grid) {
    int dev = 0, nsm = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute(fit)");
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, FIT_T, smem) != cudaSuccess)
        return check_launch("occupancy(fit)");
    *grid = (int)std::max<int64_t>(1, std::min<int64_t>(items, (int64_t)std::max(per_sm, 1) * nsm));
    return SMK_OK;
}

}  // namespace smk

using namespace smk;

extern "C" {

int smk_fit_acc_len(int32_t nzb, int32_t nkb) { return acc_len(nzb, nkb); }

int smk_fit_bluestein_m(int32_t n) { return n >= 1 && n <= FFT_MAX_N / 2 ? bluestein_m(n) : 0; }

int smk_fit_chirps(int32_t n_lengths, const int32_t* lengths, const int64_t* offsets, float* out, void* stream) {
    if (n_lengths < 0 || (n_lengths > 0 && (!lengths || !offsets || !out)))
        return fail(SMK_EINVAL, "smk_fit_chirps: null argument");
    if (n_lengths == 0) return SMK_OK;
    if ((uintptr_t)out & 7) return fail(SMK_EINVAL, "smk_fit_chirps: out must be 8-byte aligned");
    const size_t smem = 2 * FFT_MAX_N * sizeof(float2);
    if (cudaFuncSetAttribute(fit_chirp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute(fit_chirp)");
    fit_chirp_kernel<<<n_lengths, FIT_T, smem, (cudaStream_t)stream>>>(lengths, offsets, reinterpret_cast<float2*>(out));
    return check_launch("fit_chirp_kernel");
}

int smk_fit_schedule(int64_t n, const int32_t* npix_host, int32_t* order_out, int64_t* n_slots_out) {
    if (n < 0 || (n > 0 && (!npix_host || !order_out)) || !n_slots_out)
        return fail(SMK_EINVAL, "smk_fit_schedule: null argument");
    std::vector<std::pair<int32_t, int32_t>> key((size_t)n);
    for (int64_t s = 0; s < n; ++s) {
        if (npix_host[s] < 1 || npix_host[s] > FFT_MAX_N / 2)
            return fail(SMK_ENOTSUPP, "smk_fit_schedule: skewer %lld has %d pixels (1..%d)", (long long)s,
                        npix_host[s], FFT_MAX_N / 2);
        key[(size_t)s] = {npix_host[s], (int32_t)s};
    }
    std::stable_sort(key.begin(), key.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
    int64_t k = 0;
    for (size_t i = 0; i < key.size();) {
        size_t j = i;
        while (j < key.size() && key[j].first == key[i].first) ++j;
        for (size_t q = i; q < j; ++q) order_out[k++] = key[q].second;
        if ((j - i) & 1) order_out[k++] = -1;
        i = j;
    }
    *n_slots_out = k;
    return SMK_OK;
}

static int fit_args(const SmkFitProblem* fp, const float* theta, double* acc, const double* gM, const double* gP,
                    unsigned long long* counter, FitArgs* a) {
    if (!fp || !theta || !acc || !counter) return fail(SMK_EINVAL, "smk_fit: null argument");
    if (!fp->delta || !fp->zbin || !fp->offset || !fp->npix || !fp->order || !fp->kedges)
        return fail(SMK_EINVAL, "smk_fit: null problem array");
    if (fp->nzb < 1 || fp->nzb > FIT_MAX_BINS || fp->nkb < 1 || fp->nkb > FIT_MAX_BINS || !(fp->dx > 0))
        return fail(SMK_EINVAL, "smk_fit: 1..%d redshift and k bins, dx > 0", FIT_MAX_BINS);
    a->delta = fp->delta;
    a->eta = fp->eta;
    a->G = fp->G;
    a->zbin = fp->zbin;
    a->offset = fp->offset;
    a->npix = fp->npix;
    a->order = fp->order;
    a->n_items = fp->n_slots / 2;
    a->n_total = fp->n_total;
    a->nzb = fp->nzb;
    a->nkb = fp->nkb;
    a->theta = theta;
    a->kedges = fp->kedges;
    a->dx = fp->dx;
    a->acc = acc;
    a->gM = gM;
    a->gP = gP;
    a->counter = counter;
    // Bluestein lengths of the problem's skewers (n_max = 0: any length up to 2048)
    const int nmax = fp->n_max > 0 ? std::min(fp->n_max, FFT_MAX_N / 2) : FFT_MAX_N / 2;
    a->mmax = (bluestein_m(nmax) + 15) / 16 * 16;
    a->chirp = reinterpret_cast<const float2*>(fp->chirp);
    a->chirp_off = fp->chirp_off;
    if (!a->chirp != !a->chirp_off) return fail(SMK_EINVAL, "smk_fit: give chirp and chirp_off together");
    a->spec = reinterpret_cast<float2*>(fp->spectrum);
    if ((uintptr_t)a->spec & 7) return fail(SMK_EINVAL, "smk_fit: spectrum must be 8-byte aligned");
    return SMK_OK;
}

int smk_fit_forward(const SmkFitProblem* fp, const float* theta, double* acc, void* workspace,
                    size_t workspace_bytes, void* stream) {
    if (!workspace || workspace_bytes < 256) return fail(SMK_EWORKSPACE, "smk_fit_forward: 256-byte workspace");
    FitArgs a;
    int rc = fit_args(fp, theta, acc, nullptr, nullptr, (unsigned long long*)workspace, &a);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(acc, 0, sizeof(double) * acc_len(a.nzb, a.nkb), st) != cudaSuccess ||
        cudaMemsetAsync(workspace, 0, 8, st) != cudaSuccess)
        return check_launch("smk_fit_forward: memset");
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int g1 = (int)std::min<int64_t>((a.n_total + FIT_T * 16 - 1) / (FIT_T * 16), 8LL * nsm);
    fit_flux_kernel<<<std::max(g1, 1), FIT_T, 0, st>>>(a);
    if ((rc = check_launch("fit_flux_kernel"))) return rc;
    const size_t smem = (a.chirp ? 3 : 4) * (size_t)a.mmax * sizeof(float2);   // two lines, tw (, s2)
    int grid = 0;
    if ((rc = fit_grid((const void*)fit_p1d_kernel, smem, (a.n_items + 1) / 2, &grid))) return rc;
    fit_p1d_kernel<<<grid, FIT_T, smem, st>>>(a);
    return check_launch("fit_p1d_kernel");
}

int smk_fit_backward(const SmkFitProblem* fp, const float* theta, double* acc, const double* gM,
                     const double* gP, void* workspace, size_t workspace_bytes, void* stream) {
    if (!workspace || workspace_bytes < 256) return fail(SMK_EWORKSPACE, "smk_fit_backward: 256-byte workspace");
    if (!gM || !gP) return fail(SMK_EINVAL, "smk_fit_backward: null weights");
    FitArgs a;
    int rc = fit_args(fp, theta, acc, gM, gP, (unsigned long long*)workspace, &a);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int off = acc_A(a.nzb, a.nkb);
    if (cudaMemsetAsync(acc + off, 0, sizeof(double) * (acc_psq(a.nzb, a.nkb) - off), st) != cudaSuccess ||
        cudaMemsetAsync(workspace, 0, 8, st) != cudaSuccess)
        return check_launch("smk_fit_backward: memset");
    const size_t smem = (a.chirp ? 3 : 4) * (size_t)a.mmax * sizeof(float2);   // two lines, tw (, s2)
    int grid = 0;
    if ((rc = fit_grid((const void*)fit_adjoint_kernel, smem, (a.n_items + 1) / 2, &grid))) return rc;
    fit_adjoint_kernel<<<grid, FIT_T, smem, st>>>(a);
    return check_launch("fit_adjoint_kernel");
}

}  // extern "C"
