// GRF box generation (make_boxes) on GB300: white noise -> r2c -> x sqrt(P/Vcell) ->
// delta_k and eta_k = kz^2/k^2 delta_k -> c2r, as five kinds of HBM passes over padded
// [batch][nx][ny][pitch] float32 boxes:
//
//   zfwd   r2c along z of row pairs (Philox noise drawn in the kernel, or read densely)
//   line   c2c along y (forward)
//   xpass  c2c along x forward, multiply by sqrt(P/Vcell) and split eta_k, c2c along x
//          inverse for both fields (one read of the noise spectrum, two writes)
//   line   c2c along y (inverse) over delta and eta in one launch
//   zinv   c2r along z of row pairs over delta and eta, x 1/N, FP64 sum/sum^2/non-finite
//
// Every pass is a persistent kernel over tiles of W lines (see smk_fft.cuh), sized to the
// resident-block count of the GPU.
#include <algorithm>

#include "smk_fft.cuh"

namespace smk {

template <int W_, int T_>
struct TileCfg {
    static constexpr int W = W_, T = T_;
};
using CfgA = TileCfg<16, 256>;  // n <= 512
using CfgB = TileCfg<16, 512>;  // n <= 1024
using CfgC = TileCfg<8, 512>;   // n <= 2560
using CfgD = TileCfg<4, 512>;   // n <= 4096

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ------------------------------------------------------------------ shared tiling of z passes
// Rows of one box are tiled by pairs, W pairs (2W rows) per tile; tiles never straddle boxes.
struct ZTiling {
    int64_t rows_per_box;  // nx*ny
    int64_t tiles_per_box;
    __host__ __device__ void init(int64_t rpb, int W) {
        rows_per_box = rpb;
        tiles_per_box = ceil_div(ceil_div(rpb, 2), W);
    }
};

// Strided tile load: element e (0..n-1) of column w (0..W-1) from base[e*estride + w] into
// s[e*W + w] with 16-byte cp.async (columns >= cols are zero-filled).  W is even, base,
// estride and s are 16-byte aligned.  The caller waits (cp_async_wait_all + barrier).
template <int W, int T>
__device__ __forceinline__ void load_cols_async(float2* s, const float2* base, int n, int64_t estride, int cols) {
    constexpr int G = W / 2;
    for (int idx = threadIdx.x; idx < n * G; idx += T) {
        const int e = idx / G, w = 2 * (idx % G);
        const int bytes = w < cols ? (w + 1 < cols ? 16 : 8) : 0;
        cp_async<16>(s + e * W + w, bytes ? base + e * estride + w : base, bytes);
    }
}

template <int W, int T>
__device__ __forceinline__ void store_cols(const float2* s, float2* base, int n, int64_t estride, int cols) {
    for (int idx = threadIdx.x; idx < n * W; idx += T) {
        const int e = idx / W, w = idx % W;
        if (w < cols) base[e * estride + w] = s[e * W + w];
    }
}

struct ZFwdArgs {
    FftPlan pl;
    ZTiling zt;
    int batch;
    int64_t pitch;
    const float* noise;  // dense [batch][rows_per_box][nz]
    float* out;
};

// r2c along z of the caller's white noise (two rows per complex line).
// smem: s[n*SN] | tw[n] | sof[n] (slot of each frequency)
template <class C>
__global__ void __launch_bounds__(C::T, 1) zfwd_kernel(const ZFwdArgs a) {
    constexpr int W = C::W, SN = W + 1, T = C::T;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;
    float2* s = smem;
    float2* tw = s + n * SN;
    int* sof = reinterpret_cast<int*>(tw + n);
    float* sf = reinterpret_cast<float*>(s);
    fill_twiddles<T>(tw, n);
    for (int k = threadIdx.x; k < n; k += T) sof[k] = slot_of_freq(a.pl, k);
    const int nh = n / 2 + 1;
    const int64_t ntiles = a.zt.tiles_per_box * a.batch;
    const int64_t cp = a.pitch / 2;
    float2* out2 = reinterpret_cast<float2*>(a.out);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t b = tile / a.zt.tiles_per_box;
        const int64_t lrow0 = (tile - b * a.zt.tiles_per_box) * (2 * W);  // row inside box b
        const int64_t grow0 = b * a.zt.rows_per_box + lrow0;               // global row
        const int rows_here = (int)min((int64_t)(2 * W), a.zt.rows_per_box - lrow0);
        const float* src = a.noise + grow0 * n;
        for (int rl = 0; rl < 2 * W; ++rl) {
            const bool ok = rl < rows_here;
            float* dst = sf + 2 * (rl >> 1) + (rl & 1);
            for (int e = threadIdx.x; e < n; e += T)
                cp_async<4>(dst + 2 * e * SN, ok ? src + (int64_t)rl * n + e : a.noise, ok ? 4 : 0);
        }
        cp_async_wait_all();
        __syncthreads();
        fft_tile<false, W, SN, T>(s, tw, a.pl);
        // split the two real transforms packed as re/im and store the half spectra
        for (int idx = threadIdx.x; idx < W * nh; idx += T) {
            const int k = idx / W, w = idx % W;
            const float2 zk = s[sof[k] * SN + w];
            const float2 zm = s[sof[k == 0 ? 0 : n - k] * SN + w];
            if (2 * w < rows_here)
                out2[(grow0 + 2 * w) * cp + k] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            if (2 * w + 1 < rows_here)
                out2[(grow0 + 2 * w + 1) * cp + k] = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ c2c along a strided axis
struct LineArgs {
    FftPlan pl;
    float2* base[2];
    int nbuf;
    int64_t n_outer, ostride, estride;
    int ncol;
};

// Forward: natural -> digit-reversed order along the axis (kept in HBM); inverse: back.
// smem: s[n*W] | tw[n]
template <class C, bool INV>
__global__ void __launch_bounds__(C::T, 1) line_kernel(const LineArgs a) {
    constexpr int W = C::W, T = C::T;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;
    float2* s = smem;
    float2* tw = s + n * W;
    fill_twiddles<T>(tw, n);
    const int64_t ncolt = ceil_div(a.ncol, W);
    const int64_t tpb = a.n_outer * ncolt;
    const int64_t ntiles = tpb * a.nbuf;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int buf = (int)(tile / tpb);
        const int64_t t = tile - buf * tpb;
        const int64_t o = t / ncolt;
        const int cb = (int)(t - o * ncolt);
        float2* base = a.base[buf] + o * a.ostride + (int64_t)cb * W;
        const int cols = min(W, a.ncol - cb * W);
        load_cols_async<W, T>(s, base, n, a.estride, cols);
        cp_async_wait_all();
        __syncthreads();
        fft_tile<INV, W, W, T>(s, tw, a.pl);
        store_cols<W, T>(s, base, n, a.estride, cols);
        __syncthreads();
    }
}

// ------------------------------------------------------------------ fused x pass
struct XArgs {
    FftPlan pl;            // x axis
    FftPlan ply;           // y axis (the y spectrum is in digit-reversed order)
    float2* A;             // noise spectrum in, delta (x-inverse) out
    float2* B;             // eta (x-inverse) out, or null
    int nx, ny, nzh, batch;
    int64_t cp;
    int pk_mode;
    const float* grid;     // SMK_PK_GRID: [nx][ny][nzh] in natural order
    const double* amp_dev; // device A (analytic, if amp_host <= 0)
    double amp_host;
    double kfac;           // 2 * pi / dcell (2 k_Nyquist)
    float inv_k0, inv_vcell;
};

__device__ __forceinline__ float kaxis(int i, int n, double kfac, bool full) {
    // numpy fftfreq / rfftfreq times 2 k_ny, rounded to float32 (bin/make_boxes.py:299-302)
    const int ii = (full && i >= (n + 1) / 2) ? i - n : i;
    return (float)(((double)ii * (1.0 / (double)n)) * kfac);
}

// smem: s[n*W] | tw[n] | kx[n] (k_x of each slot) | ix[n] (frequency index of each slot) |
//       kt[W+1] (k_y of the tile, k_z of its columns)
template <class C>
__global__ void __launch_bounds__(C::T, 1) xpass_kernel(const XArgs a) {
    constexpr int W = C::W, T = C::T;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;  // == nx
    float2* s = smem;
    float2* tw = s + n * W;
    float* kx = reinterpret_cast<float*>(tw + n);
    int* ix = reinterpret_cast<int*>(kx + n);
    float* kt = reinterpret_cast<float*>(ix + n);
    fill_twiddles<T>(tw, n);
    for (int e = threadIdx.x; e < n; e += T) {
        const int f = freq_of_slot(a.pl, e);
        ix[e] = f;
        kx[e] = kaxis(f, n, a.kfac, true);
    }
    float amp = 0.f;
    if (a.pk_mode == SMK_PK_ANALYTIC) amp = (float)(a.amp_host > 0.0 ? a.amp_host : *a.amp_dev);
    const int64_t ncolt = ceil_div(a.nzh, W);
    const int64_t ntiles = (int64_t)a.batch * a.ny * ncolt;
    const int64_t estride = (int64_t)a.ny * a.cp;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t o = tile / ncolt;  // b*ny + y slot
        const int cb = (int)(tile - o * ncolt);
        const int64_t b = o / a.ny;
        const int yslot = (int)(o - b * a.ny);
        const int64_t off = b * (int64_t)a.nx * estride + (int64_t)yslot * a.cp + (int64_t)cb * W;
        float2* pa = a.A + off;
        float2* pb = a.B ? a.B + off : nullptr;
        const int cols = min(W, a.nzh - cb * W);
        load_cols_async<W, T>(s, pa, n, estride, cols);
        const int iy = freq_of_slot(a.ply, yslot);
        if (threadIdx.x == 0) kt[0] = kaxis(iy, a.ny, a.kfac, true);
        if (threadIdx.x < W) kt[1 + threadIdx.x] = kaxis(cb * W + threadIdx.x, 2 * (a.nzh - 1), a.kfac, false);
        cp_async_wait_all();
        __syncthreads();
        fft_tile<false, W, W, T>(s, tw, a.pl);
        const float ky = kt[0];
        for (int idx = threadIdx.x; idx < n * W; idx += T) {
            const int e = idx / W, w = idx % W;
            const float kxv = kx[e], kz = kt[1 + w];
            // k^2 in float32 without contraction, as numpy evaluates kx*kx + ky*ky + kz*kz
            const float kk = __fadd_rn(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
            float sc;
            if (a.pk_mode == SMK_PK_GRID) {
                sc = w < cols ? __ldg(a.grid + ((int64_t)ix[e] * a.ny + iy) * a.nzh + cb * W + w) : 0.f;
            } else {
                const float k = __fsqrt_rn(kk);
                const float kr = k * a.inv_k0;
                const float den = fmaf(kr, kr, 1.0f);
                sc = sqrtf(amp * k / (den * den) * a.inv_vcell);
            }
            const float2 d = cscale(s[idx], sc);
            s[idx] = d;
            if (pb && w < cols) {
                const float kk1 = (kk == 0.0f) ? 1.0f : kk;  // k^2[0,0,0] = 1 (bin/make_boxes.py:306)
                pb[e * estride + w] = cscale(d, __fdiv_rn(__fmul_rn(kz, kz), kk1));
            }
        }
        __syncthreads();
        fft_tile<true, W, W, T>(s, tw, a.pl);
        store_cols<W, T>(s, pa, n, estride, cols);
        __syncthreads();
        if (pb) {
            // each thread reads back (plain loads, L2) exactly the eta_k elements it wrote above
            for (int idx = threadIdx.x; idx < n * W; idx += T) {
                const int e = idx / W, w = idx % W;
                s[idx] = w < cols ? __ldcg(pb + e * estride + w) : make_float2(0.f, 0.f);
            }
            __syncthreads();
            fft_tile<true, W, W, T>(s, tw, a.pl);
            store_cols<W, T>(s, pb, n, estride, cols);
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------ Fourier-space noise pass
// GPU noise mode: the x pass draws the Fourier modes of white noise directly (the forward
// r2c of N(0,1) noise has independent Re/Im ~ N(0, N/2) per mode, real N(0, N) on
// self-conjugate modes, and X(-kx,-ky,kz) = X(kx,ky,kz)* on the kz = 0 and kz = nz/2 planes),
// multiplies by sqrt(P/Vcell), forms eta_k = kz^2/k^2 delta_k, and takes the inverse x
// transform of both fields as 2*WC lines of one tile.  No forward z / y passes are needed.
struct XGenArgs {
    FftPlan pl;            // x axis
    FftPlan ply;           // y axis (output stays in the y-digit-reversed order of the y inverse)
    float2* A;             // delta out
    float2* B;             // eta out, or null
    int nx, ny, nz, nzh, batch;
    int64_t cp;
    int pk_mode;
    const float* grid;
    const double* amp_dev;
    double amp_host;
    double kfac;
    float inv_k0, inv_vcell;
    float sig_c, sig_r;    // sqrt(N/2), sqrt(N)
    uint64_t seed;
};

template <int W_, int T_>
struct XGenCfg {
    static constexpr int W = W_, T = T_;   // W lines = W/2 delta columns + W/2 eta columns
};
using XGenA = XGenCfg<32, 256>;  // n <= 512
using XGenB = XGenCfg<16, 512>;  // n <= 1024
using XGenC = XGenCfg<8, 512>;   // n <= 2560
using XGenD = XGenCfg<4, 512>;   // n <= 4096

// smem: s[n*W] | tw[n] | kx[n] | ix[n]
template <class C>
__global__ void __launch_bounds__(C::T, 1) xgen_kernel(const XGenArgs a) {
    constexpr int W = C::W, WC = W / 2, NP = WC / 2, T = C::T;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;  // == nx
    float2* s = smem;
    float2* tw = s + n * W;
    float* kx = reinterpret_cast<float*>(tw + n);
    int* ix = reinterpret_cast<int*>(kx + n);
    fill_twiddles<T>(tw, n);
    for (int e = threadIdx.x; e < n; e += T) {
        const int f = freq_of_slot(a.pl, e);
        ix[e] = f;
        kx[e] = kaxis(f, n, a.kfac, true);
    }
    __syncthreads();
    float amp = 0.f;
    if (a.pk_mode == SMK_PK_ANALYTIC) amp = (float)(a.amp_host > 0.0 ? a.amp_host : *a.amp_dev);
    const int64_t ncolt = ceil_div(a.nzh, WC);
    const int64_t ntiles = (int64_t)a.batch * a.ny * ncolt;
    const int64_t estride = (int64_t)a.ny * a.cp;
    const int half = a.nz / 2;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t o = tile / ncolt;  // b*ny + y slot
        const int cb = (int)(tile - o * ncolt);
        const int64_t b = o / a.ny;
        const int yslot = (int)(o - b * a.ny);
        const int iy = freq_of_slot(a.ply, yslot);
        const int iym = iy == 0 ? 0 : a.ny - iy;
        const float ky = kaxis(iy, a.ny, a.kfac, true);
        const uint64_t seed = a.seed + (uint64_t)b;
        for (int idx = threadIdx.x; idx < n * NP; idx += T) {
            const int e = idx / NP, pr = idx % NP;
            const int c0 = 2 * pr, kz0 = cb * WC + c0;
            const int ixe = ix[e];
            float g[4];
            {
                u32x4 ctr;
                ctr.v[0] = (uint32_t)(kz0 >> 1);
                ctr.v[1] = (uint32_t)ixe;
                ctr.v[2] = (uint32_t)iy;
                ctr.v[3] = STREAM_KMODE;
                gauss4(philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32)), g);
            }
            const float kxv = kx[e];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int kz = kz0 + h;
                float2 d = make_float2(0.f, 0.f), et = make_float2(0.f, 0.f);
                if (kz < a.nzh) {
                    float2 X = make_float2(a.sig_c * g[2 * h], a.sig_c * g[2 * h + 1]);
                    if (kz == 0 || kz == half) {
                        const int ixm = ixe == 0 ? 0 : a.nx - ixe;
                        if (ixm == ixe && iym == iy) {
                            X = make_float2(a.sig_r * g[2 * h], 0.f);
                        } else if ((int64_t)ixe * a.ny + iy > (int64_t)ixm * a.ny + iym) {
                            // the partner (-kx, -ky) owns the draw: take its conjugate
                            u32x4 ctr;
                            ctr.v[0] = (uint32_t)(kz0 >> 1);
                            ctr.v[1] = (uint32_t)ixm;
                            ctr.v[2] = (uint32_t)iym;
                            ctr.v[3] = STREAM_KMODE;
                            float gm[4];
                            gauss4(philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32)), gm);
                            X = make_float2(a.sig_c * gm[2 * h], -a.sig_c * gm[2 * h + 1]);
                        }
                    }
                    const float kz_ = kaxis(kz, a.nz, a.kfac, false);
                    const float kk = __fadd_rn(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(ky, ky)), __fmul_rn(kz_, kz_));
                    float sc;
                    if (a.pk_mode == SMK_PK_GRID) {
                        sc = __ldg(a.grid + ((int64_t)ixe * a.ny + iy) * a.nzh + kz);
                    } else {
                        const float k = __fsqrt_rn(kk);
                        const float kr = k * a.inv_k0;
                        const float den = fmaf(kr, kr, 1.0f);
                        sc = sqrtf(amp * k / (den * den) * a.inv_vcell);
                    }
                    d = cscale(X, sc);
                    const float kk1 = (kk == 0.0f) ? 1.0f : kk;
                    et = cscale(d, __fdiv_rn(__fmul_rn(kz_, kz_), kk1));
                }
                s[e * W + c0 + h] = d;
                s[e * W + WC + c0 + h] = et;
            }
        }
        __syncthreads();
        fft_tile<true, W, W, T>(s, tw, a.pl);
        const int cols = min(WC, a.nzh - cb * WC);
        const int64_t off = b * (int64_t)a.nx * estride + (int64_t)yslot * a.cp + (int64_t)cb * WC;
        for (int idx = threadIdx.x; idx < n * W; idx += T) {
            const int e = idx / W, l = idx % W;
            const int c = l % WC;
            if (c < cols) {
                float2* dst = l < WC ? a.A : a.B;
                if (dst) dst[off + e * estride + c] = s[idx];
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ z inverse (c2r) + stats
struct ZInvArgs {
    FftPlan pl;
    ZTiling zt;
    int batch;
    float* buf[2];
    int nbuf;
    int64_t pitch;
    float scale;
    double* stats;  // [batch][2][4] or null
};

template <int T>
__device__ __forceinline__ void flush_stats(double s1, double s2, double bad, double* red, double* dst) {
    // block sum of three doubles, then one atomic per quantity
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s1 += __shfl_down_sync(0xffffffffu, s1, off);
        s2 += __shfl_down_sync(0xffffffffu, s2, off);
        bad += __shfl_down_sync(0xffffffffu, bad, off);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        red[3 * wid] = s1;
        red[3 * wid + 1] = s2;
        red[3 * wid + 2] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t1 = 0, t2 = 0, t3 = 0;
        for (int i = 0; i < T / 32; ++i) {
            t1 += red[3 * i];
            t2 += red[3 * i + 1];
            t3 += red[3 * i + 2];
        }
        atomicAdd(dst, t1);
        atomicAdd(dst + 1, t2);
        atomicAdd(dst + 2, t3);
    }
    __syncthreads();
}

// smem: s[n*SN] | tw[n] | sof[n] | red[3*T/32] (doubles)
template <class C>
__global__ void __launch_bounds__(C::T, 1) zinv_kernel(const ZInvArgs a) {
    constexpr int W = C::W, SN = W + 1, T = C::T;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;
    float2* s = smem;
    float2* tw = s + n * SN;
    int* sof = reinterpret_cast<int*>(tw + n);
    double* red = reinterpret_cast<double*>(sof + n + (n & 1));
    float* sf = reinterpret_cast<float*>(s);
    fill_twiddles<T>(tw, n);
    for (int k = threadIdx.x; k < n; k += T) sof[k] = slot_of_freq(a.pl, k);
    __syncthreads();
    const int nh = n / 2 + 1, half = n / 2;
    const int64_t tpbuf = a.zt.tiles_per_box * a.batch;
    const int64_t ntiles = tpbuf * a.nbuf;
    const int64_t cp = a.pitch / 2;
    double acc1 = 0.0, acc2 = 0.0, accb = 0.0;
    int64_t cur = -1;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int buf = (int)(tile / tpbuf);
        const int64_t t = tile - buf * tpbuf;
        const int64_t b = t / a.zt.tiles_per_box;
        const int64_t lrow0 = (t - b * a.zt.tiles_per_box) * (2 * W);
        const int64_t grow0 = b * a.zt.rows_per_box + lrow0;
        const int rows_here = (int)min((int64_t)(2 * W), a.zt.rows_per_box - lrow0);
        const int64_t key = (int64_t)buf * a.batch + b;
        if (a.stats && key != cur) {
            if (cur >= 0) {
                const int64_t cb = cur % a.batch, cf = cur / a.batch;
                flush_stats<T>(acc1, acc2, accb, red, a.stats + 8 * cb + 4 * cf);
            }
            acc1 = acc2 = accb = 0.0;
            cur = key;
        }
        const float2* in2 = reinterpret_cast<const float2*>(a.buf[buf]) + grow0 * cp;
        // X1_k (even row) to the slot of frequency k, X2_k (odd row) to the slot of n-k;
        // DC and Nyquist keep their real parts (re: X1, im: X2).  Rows are the fast index of
        // the thread mapping so the permuted shared-memory slots are written W-contiguous.
        for (int idx = threadIdx.x; idx < 2 * W * nh; idx += T) {
            const int k = idx / (2 * W), rl = idx % (2 * W);
            const int w = rl >> 1, odd = rl & 1;
            const bool ok = rl < rows_here;
            const float2* src = ok ? in2 + (int64_t)rl * cp + k : in2;
            if (k == 0 || k == half) {
                cp_async<4>(sf + 2 * (sof[k] * SN + w) + odd, src, ok ? 4 : 0);
            } else {
                cp_async<8>(s + sof[odd ? n - k : k] * SN + w, src, ok ? 8 : 0);
            }
        }
        cp_async_wait_all();
        __syncthreads();
        for (int idx = threadIdx.x; idx < W * (half - 1); idx += T) {
            const int k = 1 + idx / W, w = idx % W;
            const int i1 = sof[k] * SN + w, i2 = sof[n - k] * SN + w;
            const float2 x1 = s[i1], x2 = s[i2];
            s[i1] = make_float2(x1.x - x2.y, x1.y + x2.x);   // Z_k = X1_k + i X2_k
            s[i2] = make_float2(x1.x + x2.y, x2.x - x1.y);   // Z_{n-k} = X1_k* + i X2_k*
        }
        __syncthreads();
        fft_tile<true, W, SN, T>(s, tw, a.pl);
        float p1 = 0.f, p2 = 0.f, pb = 0.f;
        float* out = a.buf[buf] + grow0 * a.pitch;
        for (int rl = 0; rl < rows_here; ++rl) {
            const float* srow = sf + 2 * (rl >> 1) + (rl & 1);
            float* orow = out + (int64_t)rl * a.pitch;
            for (int e = threadIdx.x; e < n; e += T) {
                const float v = srow[2 * e * SN] * a.scale;
                orow[e] = v;
                if (isfinite(v)) {
                    p1 += v;
                    p2 = fmaf(v, v, p2);
                } else {
                    pb += 1.f;
                }
            }
        }
        acc1 += p1;
        acc2 += p2;
        accb += pb;
        __syncthreads();
    }
    if (a.stats && cur >= 0) {
        const int64_t cb = cur % a.batch, cf = cur / a.batch;
        flush_stats<T>(acc1, acc2, accb, red, a.stats + 8 * cb + 4 * cf);
    }
}

// ------------------------------------------------------------------ P(k) normalisation
__global__ void pk_norm_kernel(int nx, int ny, int nz, double kfac, float inv_k0, double* acc) {
    const int nzh = nz / 2 + 1;
    const int nchunk = (nzh + 63) / 64;
    const int64_t items = (int64_t)nx * ny * nchunk;
    double tsum = 0.0;
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < items;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = it / nchunk;
        const int ch = (int)(it - row * nchunk);
        const int x = (int)(row / ny), y = (int)(row - (int64_t)x * ny);
        const float kx = kaxis(x, nx, kfac, true), ky = kaxis(y, ny, kfac, true);
        const float kxy = __fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky));
        float part = 0.f;
        const int z1 = min(nzh, 64 * ch + 64);
        for (int z = 64 * ch; z < z1; ++z) {
            const float kz = kaxis(z, nz, kfac, false);
            const float k = __fsqrt_rn(__fadd_rn(kxy, __fmul_rn(kz, kz)));
            const float kr = k * inv_k0;
            const float den = fmaf(kr, kr, 1.0f);
            const float w = (z == 0 || (2 * z == nz)) ? 1.f : 2.f;
            part += w * (k / (den * den));
        }
        tsum += part;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) tsum += __shfl_down_sync(0xffffffffu, tsum, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, tsum);
}

__global__ void pk_amp_kernel(const double* acc, double ncell_vcell, double* amp) {
    if (threadIdx.x == 0 && blockIdx.x == 0) amp[0] = ncell_vcell / acc[0];
}

// ------------------------------------------------------------------ launch helpers
static int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

template <typename K>
static int persistent_grid(K kernel, int threads, size_t smem, int64_t ntiles, int* grid) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess)
        return check_launch("cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (per_sm < 1) return fail(SMK_ENOTSUPP, "kernel does not fit on an SM (smem %zu B)", smem);
    *grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)per_sm * sm_count()));
    return SMK_OK;
}

template <class C>
static size_t zpass_smem(int n) {
    return (size_t)n * (C::W + 1) * sizeof(float2) + (size_t)n * sizeof(float2) + (size_t)(n + 1) * sizeof(int) +
           3 * (C::T / 32) * sizeof(double) + 8;
}

template <class C>
static int launch_zfwd(const ZFwdArgs& a, cudaStream_t st) {
    const size_t smem = zpass_smem<C>(a.pl.n);
    const int64_t ntiles = a.zt.tiles_per_box * a.batch;
    int grid = 0, rc;
    if ((rc = persistent_grid(zfwd_kernel<C>, C::T, smem, ntiles, &grid))) return rc;
    zfwd_kernel<C><<<grid, C::T, smem, st>>>(a);
    return check_launch("zfwd_kernel");
}

template <class C>
static int launch_xgen(const XGenArgs& a, cudaStream_t st) {
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2) + (size_t)a.pl.n * 8;
    const int64_t ntiles = (int64_t)a.batch * a.ny * ceil_div(a.nzh, C::W / 2);
    int grid = 0, rc;
    if ((rc = persistent_grid(xgen_kernel<C>, C::T, smem, ntiles, &grid))) return rc;
    xgen_kernel<C><<<grid, C::T, smem, st>>>(a);
    return check_launch("xgen_kernel");
}

template <class C>
static int launch_line(const LineArgs& a, bool inv, cudaStream_t st) {
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2);
    const int64_t ntiles = a.n_outer * ceil_div(a.ncol, C::W) * a.nbuf;
    int grid = 0, rc;
    if (inv) {
        if ((rc = persistent_grid(line_kernel<C, true>, C::T, smem, ntiles, &grid))) return rc;
        line_kernel<C, true><<<grid, C::T, smem, st>>>(a);
    } else {
        if ((rc = persistent_grid(line_kernel<C, false>, C::T, smem, ntiles, &grid))) return rc;
        line_kernel<C, false><<<grid, C::T, smem, st>>>(a);
    }
    return check_launch("line_kernel");
}

template <class C>
static int launch_xpass(const XArgs& a, cudaStream_t st) {
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2) + (size_t)a.pl.n * 8 + (C::W + 1) * 4;
    const int64_t ntiles = (int64_t)a.batch * a.ny * ceil_div(a.nzh, C::W);
    int grid = 0, rc;
    if ((rc = persistent_grid(xpass_kernel<C>, C::T, smem, ntiles, &grid))) return rc;
    xpass_kernel<C><<<grid, C::T, smem, st>>>(a);
    return check_launch("xpass_kernel");
}

template <class C>
static int launch_zinv(const ZInvArgs& a, cudaStream_t st) {
    const size_t smem = zpass_smem<C>(a.pl.n);
    const int64_t ntiles = a.zt.tiles_per_box * a.batch * a.nbuf;
    int grid = 0, rc;
    if ((rc = persistent_grid(zinv_kernel<C>, C::T, smem, ntiles, &grid))) return rc;
    zinv_kernel<C><<<grid, C::T, smem, st>>>(a);
    return check_launch("zinv_kernel");
}

// n -> tile class; the dispatch macro instantiates every pass for the four classes
#define SMK_DISPATCH_X(n, FN, ...)                                \
    ((n) <= 512 ? FN<XGenA>(__VA_ARGS__)                          \
                : (n) <= 1024 ? FN<XGenB>(__VA_ARGS__)            \
                              : (n) <= 2560 ? FN<XGenC>(__VA_ARGS__) : FN<XGenD>(__VA_ARGS__))

#define SMK_DISPATCH(n, FN, ...)                                  \
    ((n) <= 512 ? FN<CfgA>(__VA_ARGS__)                           \
                : (n) <= 1024 ? FN<CfgB>(__VA_ARGS__)             \
                              : (n) <= 2560 ? FN<CfgC>(__VA_ARGS__) : FN<CfgD>(__VA_ARGS__))

static int zfwd_w(int n) { return n <= 512 ? CfgA::W : n <= 1024 ? CfgB::W : n <= 2560 ? CfgC::W : CfgD::W; }

}  // namespace smk

using namespace smk;

extern "C" {

int64_t smk_grf_pitch(int32_t nz) {
    if (nz < 2) return 0;
    const int64_t p = 2 * (int64_t)(nz / 2 + 1);
    return (p + 7) / 8 * 8;
}

int64_t smk_grf_box_floats(const SmkGrfParams* p) {
    if (!p || p->nx < 1 || p->ny < 1 || p->nz < 2 || p->batch < 1) return 0;
    return (int64_t)p->batch * p->nx * p->ny * smk_grf_pitch(p->nz);
}

size_t smk_grf_workspace_size(const SmkGrfParams* p) {
    (void)p;
    return 256;  // [0] FP64 mode sum, [1] amplitude A
}

int smk_pk_normalisation(int32_t nx, int32_t ny, int32_t nz, double dcell, double k0, double* amp_dev,
                         void* stream) {
    if (nx < 1 || ny < 1 || nz < 2 || !(dcell > 0) || !(k0 > 0) || !amp_dev)
        return fail(SMK_EINVAL, "smk_pk_normalisation: invalid argument");
    cudaStream_t st = (cudaStream_t)stream;
    // amp_dev[0] is used as the accumulator first, then overwritten by A
    if (cudaMemsetAsync(amp_dev, 0, sizeof(double), st) != cudaSuccess) return check_launch("cudaMemsetAsync");
    const double kfac = 2.0 * (3.14159265358979323846 / dcell);
    const int64_t items = (int64_t)nx * ny * ((nz / 2 + 1 + 63) / 64);
    const int grid = (int)std::min<int64_t>(ceil_div(items, 256), 8LL * sm_count());
    pk_norm_kernel<<<grid, 256, 0, st>>>(nx, ny, nz, kfac, (float)(1.0 / k0), amp_dev);
    int rc = check_launch("pk_norm_kernel");
    if (rc) return rc;
    const double vcell = (double)(float)(dcell * dcell * dcell);
    pk_amp_kernel<<<1, 32, 0, st>>>(amp_dev, (double)nx * ny * nz * vcell, amp_dev);
    return check_launch("pk_amp_kernel");
}

int smk_grf_check(const double* st, int64_t ncells, double* sigma_out) {
    if (!st || ncells <= 0) return fail(SMK_EINVAL, "smk_grf_check: invalid argument");
    const double mean = st[0] / (double)ncells;
    const double var = std::max(0.0, st[1] / (double)ncells - mean * mean);
    if (sigma_out) *sigma_out = sqrt(var);
    if (st[2] > 0) return fail(SMK_ENULLBOX, "box holds %.0f non-finite cells", st[2]);
    if (st[1] == 0.0) return fail(SMK_ENULLBOX, "box is all zero");
    return SMK_OK;
}

int smk_grf_boxes(const SmkGrfParams* p, float* delta, float* eta, double* stats, void* workspace,
                  size_t workspace_bytes, void* stream) {
    if (!p || !delta) return fail(SMK_EINVAL, "smk_grf_boxes: null params or delta");
    if (p->batch < 1 || p->nx < 2 || p->ny < 2 || p->nz < 2 || (p->nz & 1))
        return fail(SMK_EINVAL, "smk_grf_boxes: need nx, ny >= 2, nz >= 2 even, batch >= 1");
    if (!(p->dcell > 0)) return fail(SMK_EINVAL, "smk_grf_boxes: dcell must be > 0");
    if (p->want_eta && !eta) return fail(SMK_EINVAL, "smk_grf_boxes: want_eta needs an eta box");
    if (p->noise_mode != SMK_NOISE_HOST && p->noise_mode != SMK_NOISE_PHILOX)
        return fail(SMK_EINVAL, "smk_grf_boxes: unknown noise_mode");
    if (p->noise_mode == SMK_NOISE_HOST && !p->noise) return fail(SMK_EINVAL, "smk_grf_boxes: null noise");
    if (p->pk_mode == SMK_PK_GRID) {
        if (!p->pk_grid) return fail(SMK_EINVAL, "smk_grf_boxes: SMK_PK_GRID needs pk_grid");
    } else if (p->pk_mode == SMK_PK_ANALYTIC) {
        if (!(p->k0 > 0)) return fail(SMK_EINVAL, "smk_grf_boxes: k0 must be > 0");
        if (!(p->amp > 0) && (!workspace || workspace_bytes < smk_grf_workspace_size(p)))
            return fail(SMK_EWORKSPACE, "smk_grf_boxes: normalisation needs %zu workspace bytes",
                        smk_grf_workspace_size(p));
    } else {
        return fail(SMK_EINVAL, "smk_grf_boxes: unknown pk_mode");
    }
    FftPlan plx, ply, plz;
    if (!make_plan(p->nx, &plx) || !make_plan(p->ny, &ply) || !make_plan(p->nz, &plz))
        return fail(SMK_ENOTSUPP, "smk_grf_boxes: %dx%dx%d has an axis outside 2..4096 or not 2^a3^b5^c",
                    p->nx, p->ny, p->nz);
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t pitch = smk_grf_pitch(p->nz);
    const int64_t cp = pitch / 2;
    const int nzh = p->nz / 2 + 1;
    const double kfac = 2.0 * (3.14159265358979323846 / p->dcell);
    int rc;

    double* amp_dev = nullptr;
    if (p->pk_mode == SMK_PK_ANALYTIC && !(p->amp > 0)) {
        amp_dev = reinterpret_cast<double*>(workspace);
        if ((rc = smk_pk_normalisation(p->nx, p->ny, p->nz, p->dcell, p->k0, amp_dev, stream))) return rc;
    }
    if (stats && cudaMemsetAsync(stats, 0, sizeof(double) * 8 * p->batch, st) != cudaSuccess)
        return check_launch("cudaMemsetAsync(stats)");

    cudaEvent_t* ev = p->n_pass_events >= 6 ? (cudaEvent_t*)p->pass_events : nullptr;
    auto mark = [&](int i) {
        if (ev && cudaEventRecord(ev[i], st) != cudaSuccess) return check_launch("cudaEventRecord");
        return SMK_OK;
    };
    if ((rc = mark(0))) return rc;
    float2* d2 = reinterpret_cast<float2*>(delta);
    float2* e2 = reinterpret_cast<float2*>(eta);
    LineArgs ya;
    ya.pl = ply;
    ya.base[0] = d2;
    ya.base[1] = e2;
    ya.nbuf = 1;
    ya.n_outer = (int64_t)p->batch * p->nx;
    ya.ostride = (int64_t)p->ny * cp;
    ya.estride = cp;
    ya.ncol = nzh;
    ZTiling zt;
    zt.init((int64_t)p->nx * p->ny, zfwd_w(p->nz));
    const float inv_vcell = 1.0f / (float)(p->dcell * p->dcell * p->dcell);
    if (p->noise_mode == SMK_NOISE_PHILOX) {
        // Fourier modes drawn in the x pass: no forward z / y passes
        if ((rc = mark(1)) || (rc = mark(2))) return rc;
        XGenArgs ga;
        ga.pl = plx;
        ga.ply = ply;
        ga.A = d2;
        ga.B = p->want_eta ? e2 : nullptr;
        ga.nx = p->nx;
        ga.ny = p->ny;
        ga.nz = p->nz;
        ga.nzh = nzh;
        ga.batch = p->batch;
        ga.cp = cp;
        ga.pk_mode = p->pk_mode;
        ga.grid = p->pk_grid;
        ga.amp_dev = amp_dev;
        ga.amp_host = amp_dev ? 0.0 : p->amp;
        ga.kfac = kfac;
        ga.inv_k0 = p->pk_mode == SMK_PK_ANALYTIC ? (float)(1.0 / p->k0) : 0.f;
        ga.inv_vcell = inv_vcell;
        const double ncell = (double)p->nx * p->ny * p->nz;
        ga.sig_c = (float)sqrt(0.5 * ncell);
        ga.sig_r = (float)sqrt(ncell);
        ga.seed = p->seed;
        if ((rc = SMK_DISPATCH_X(p->nx, launch_xgen, ga, st))) return rc;
        if ((rc = mark(3))) return rc;
    } else {
        // 1. r2c along z of the caller's noise
        ZFwdArgs za;
        za.pl = plz;
        za.zt = zt;
        za.batch = p->batch;
        za.pitch = pitch;
        za.noise = p->noise;
        za.out = delta;
        if ((rc = SMK_DISPATCH(p->nz, launch_zfwd, za, st))) return rc;
        if ((rc = mark(1))) return rc;
        // 2. c2c along y, forward (the y spectrum stays in digit-reversed order)
        if ((rc = SMK_DISPATCH(p->ny, launch_line, ya, false, st))) return rc;
        if ((rc = mark(2))) return rc;
        // 3. x: forward, P(k) scaling + eta split, inverse
        XArgs xa;
        xa.pl = plx;
        xa.ply = ply;
        xa.A = d2;
        xa.B = p->want_eta ? e2 : nullptr;
        xa.nx = p->nx;
        xa.ny = p->ny;
        xa.nzh = nzh;
        xa.batch = p->batch;
        xa.cp = cp;
        xa.pk_mode = p->pk_mode;
        xa.grid = p->pk_grid;
        xa.amp_dev = amp_dev;
        xa.amp_host = amp_dev ? 0.0 : p->amp;
        xa.kfac = kfac;
        xa.inv_k0 = p->pk_mode == SMK_PK_ANALYTIC ? (float)(1.0 / p->k0) : 0.f;
        xa.inv_vcell = inv_vcell;
        if ((rc = SMK_DISPATCH(p->nx, launch_xpass, xa, st))) return rc;
        if ((rc = mark(3))) return rc;
    }

    // 4. c2c along y, inverse, on delta (and eta)
    ya.nbuf = p->want_eta ? 2 : 1;
    if ((rc = SMK_DISPATCH(p->ny, launch_line, ya, true, st))) return rc;
    if ((rc = mark(4))) return rc;

    // 5. c2r along z, / N, statistics
    ZInvArgs ia;
    ia.pl = plz;
    ia.zt = zt;
    ia.batch = p->batch;
    ia.buf[0] = delta;
    ia.buf[1] = eta;
    ia.nbuf = p->want_eta ? 2 : 1;
    ia.pitch = pitch;
    ia.scale = (float)(1.0 / ((double)p->nx * p->ny * p->nz));
    ia.stats = stats;
    if ((rc = SMK_DISPATCH(p->nz, launch_zinv, ia, st))) return rc;
    return mark(5);
}

}  // extern "C"
