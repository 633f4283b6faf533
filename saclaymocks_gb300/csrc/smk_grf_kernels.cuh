// GRF pass kernels of libsmk (make_boxes on GB300), shared by the translation units that
// instantiate their tile variants:
//
//   zfwd   r2c along z of the caller's white noise, two rows per complex line (zfwdw: one
//          warp per row pair, the built-in form; zfwd_kernel: block tiles)
//   line   c2c along y (forward: natural -> digit-reversed, inverse: back), in place, from the
//          blocked x-pass intermediate, or (forward) into it
//   xpass  x forward, x sqrt(P/Vcell), eta_k = kz^2/k^2 delta_k, x inverse of both fields
//          (xpi_kernel: read from and written to the blocked intermediate)
//   xgen   GPU noise: Fourier modes of white noise drawn in place, x sqrt(P/Vcell), eta split,
//          x inverse of both fields (replaces zfwd + line forward + xpass; xgi_kernel: into the
//          blocked intermediate)
//   zinv   c2r along z of row pairs of delta and eta, x 1/N, FP64 sum/sum^2/non-finite (zinvw:
//          one warp per row pair)
//
// Every pass is a persistent kernel over tiles of W lines (see smk_fft.cuh) or warps sized to
// the resident-block count of the GPU; the tile variant (W, threads) of each pass is chosen per
// line length from the tables below (smk_tune_set overrides the default).
#pragma once

#include <algorithm>
#include <atomic>

#include <cooperative_groups.h>

#include "smk_fft.cuh"

namespace smk {

namespace cg = cooperative_groups;

// W lines (or row pairs) per tile, T threads, largest FFT radix R in registers, at least B
// resident blocks per SM requested from the register allocator; F > 0: the line length is F and
// the FFT plan is a compile-time constant (FixedPlan<F, R>), else the plan is read at run time.
template <int W_, int T_, int R_ = fft_max_radix(T_), int B_ = 1, int F_ = 0, int D_ = -1>
struct TileCfg {
    // D: y-pass direction compiled in (1 inverse, 0 forward, -1 both)
    static constexpr int W = W_, T = T_, RMAX = R_, MINB = B_, NF = F_, DIR = D_;
};

// The launch's plan is the one a fixed-length variant was compiled for (always true otherwise).
template <class C>
inline bool fixed_plan_ok(const FftPlan& pl) {
    if constexpr (C::NF > 0) return same_plan(pl, FixedPlan<C::NF, C::RMAX>::P);
    else return true;
}

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

// The tile's W columns (column block cb of the launch, line o) into the blocked layout
// dst[((c / kb) * n_outer + o) * n + e][c % kb], c = cb W + w: each of the W / kb blocks is one
// contiguous run of n * kb values, written as 16-byte pieces (kb even, dst 16-byte aligned).
// Columns past the launch's count carry the zeros the load put there.
template <int W, int T, int KB>
__device__ __forceinline__ void store_blocked(const float2* s, float2* dst, int n, int64_t n_outer, int64_t o,
                                              int cb) {
    constexpr int HK = KB / 2;
    for (int q = 0; q < W / KB; ++q) {
        float2* run = dst + (((int64_t)cb * (W / KB) + q) * n_outer + o) * n * KB;
        for (int idx = threadIdx.x; idx < n * HK; idx += T) {
            const int e = idx / HK, w2 = 2 * (idx % HK);
            const float2 v0 = s[e * W + q * KB + w2], v1 = s[e * W + q * KB + w2 + 1];
            *reinterpret_cast<float4*>(run + (int64_t)e * KB + w2) = make_float4(v0.x, v0.y, v1.x, v1.y);
        }
    }
}
template <int W, int T>
__device__ __forceinline__ void store_blocked(const float2* s, float2* dst, int n, int kb, int64_t n_outer,
                                              int64_t o, int cb) {
    if constexpr (W >= 2) { if (kb == W) { store_blocked<W, T, W>(s, dst, n, n_outer, o, cb); return; } }
    if constexpr (W >= 4) { if (kb == W / 2) { store_blocked<W, T, W / 2>(s, dst, n, n_outer, o, cb); return; } }
    if constexpr (W >= 8) { if (kb == W / 4) { store_blocked<W, T, W / 4>(s, dst, n, n_outer, o, cb); return; } }
    if constexpr (W >= 16) { if (kb == W / 8) { store_blocked<W, T, W / 8>(s, dst, n, n_outer, o, cb); return; } }
}

struct ZFwdArgs {
    FftPlan pl;
    ZTiling zt;             // set by the launcher from its tile width
    int batch;
    int64_t pitch;
    const float* noise;  // dense [batch][rows_per_box][nz]
    float* out;
    int prefetch;        // one-warp-per-row-pair form: pull the next pair's rows into L2
};

// r2c along z of the caller's white noise (two rows per complex line).
// smem: s[n*SN] | tw[n] | sof[n] (slot of each frequency)
template <class C>
__global__ void __launch_bounds__(C::T, C::MINB) zfwd_kernel(const ZFwdArgs a) {
    constexpr int W = C::W, SN = W + 1, T = C::T;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;
    float2* s = smem;
    float2* tw = s + n * SN;
    int* sof = reinterpret_cast<int*>(tw + n);
    float* sf = reinterpret_cast<float*>(s);
    fill_stage_twiddles(tw, a.pl);
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
        fft_tile<false, W, SN, T, C::RMAX, C::NF>(s, tw, a.pl);
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
    int prefetch;   // pull the next tile into L2 during the transform
    // TMA tile loads (tma = 1): one 3D tensor map per buffer over (column, element, outer) of
    // 8-byte complex values, boxes of W columns x box_rows elements (box_rows divides n)
    int tma, box_rows;
    // wait test (SMK_TUNE_TMA_WAIT_TEST): extra bytes the barrier expects beyond the copies, so
    // the phase never completes, and the wait limit in clock cycles
    int tma_extra_tx;
    long long tma_wait_limit;
    CUtensorMap tmap[2];
    // Source of the tiles: in place (src[0] null) or the blocked intermediate of the x pass
    // (xgi_kernel): column c of the launch (0 <= c < ncol) of line o, element e at
    // src[buf] + (((c / src_kb) * n_outer + o) * n + e) * src_kb + c % src_kb.  With TMA, tmap is
    // a 5D map (src_kb, W / src_kb, n, n_outer, column tiles) over the source.  Output columns
    // start at col0 in every row.
    const float2* src[2];
    int src_kb;
    int col0;
    // Destination of a forward launch (one buffer): in place (null) or the blocked layout above
    // with dst_kb columns per block (the host-noise x pass reads it as contiguous rows)
    float2* dst;
    int dst_kb;
};

constexpr int LINE_PARTS = 2;   // most parts a y tile's TMA load is split into

// Forward: natural -> digit-reversed order along the axis (kept in HBM); inverse: back.
// smem: s[n*W] | tw[n]
template <class C, bool INV>
__global__ void __launch_bounds__(C::T, C::MINB) line_kernel(const __grid_constant__ LineArgs a) {
    constexpr int W = C::W, T = C::T;
    extern __shared__ __align__(128) float2 smem[];
    __shared__ __align__(8) uint64_t bar[LINE_PARTS];   // TMA completion of the tile (of each of its parts)
    __shared__ int timed_out;
    const int n = a.pl.n;
    float2* s = smem;
    float2* tw = s + n * W;
    fill_stage_twiddles(tw, a.pl);
    if (threadIdx.x == 0) {
        timed_out = 0;
        if (a.tma) {
            for (int p = 0; p < LINE_PARTS; ++p) mbar_init(&bar[p], 1);
            mbar_fence_init();
        }
    }
    __syncthreads();
    unsigned parity = 0;
    // Tile in two halves (inverse with a compile-time plan whose first stages work on groups that
    // stay inside a half, TMA loads into shared memory): half p of the rows completes on bar[p],
    // and those stages run on the first half while the second is still in flight.  The halves
    // are whole boxes (ns = 1 otherwise; four parts with 128-row boxes measured slower).
    int ns = 1;
    if constexpr (INV && C::NF > 0) {
        constexpr int d2 = parts_depth<C::NF, C::RMAX>(2);
        if (d2 >= 1 && a.tma == 1 && n % 2 == 0 && (n / 2) % a.box_rows == 0) ns = 2;
    }
    const int64_t ncolt = ceil_div(a.ncol, W);
    const int64_t tpb = a.n_outer * ncolt;
    const int64_t ntiles = tpb * a.nbuf;
    // the source runs of this block's next tile into L2 (intermediate source)
    auto prefetch_src = [&](int64_t tile) {
        if (tile + gridDim.x >= ntiles) return;
        const int64_t tn = tile + gridDim.x;
        const int bn = (int)(tn / tpb);
        const int64_t un = tn - bn * tpb;
        const int64_t on = un / ncolt;
        const int cbn = (int)(un - on * ncolt);
        for (int q = 0; q < W / a.src_kb; ++q)
            prefetch_l2_bulk(a.src[bn] + (((int64_t)cbn * (W / a.src_kb) + q) * a.n_outer + on) * n * a.src_kb,
                             (uint32_t)(n * a.src_kb * sizeof(float2)));
    };
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int buf = (int)(tile / tpb);
        const int64_t t = tile - buf * tpb;
        const int64_t o = t / ncolt;
        const int cb = (int)(t - o * ncolt);
        float2* base = a.base[buf] + o * a.ostride + a.col0 + (int64_t)cb * W;
        const int cols = min(W, a.ncol - cb * W);
        const float2* src = a.src[buf];
        if (a.tma) {
            // n / box_rows tensor boxes of W columns (columns past ncol read as zeros)
            if (threadIdx.x == 0) {
                if (a.tma == 2) bulk_wait_read_all();   // the previous tile's stores have read s
                const int pr = n / ns;
                for (int part = 0; part < ns; ++part) {
                    uint64_t* b = &bar[part];
                    const int e_lo = part * pr, e_hi = e_lo + pr;
                    mbar_arrive_expect_tx(b, (unsigned)((e_hi - e_lo) * W * sizeof(float2)) +
                                                 (part ? 0u : (unsigned)a.tma_extra_tx));
                    for (int e0 = e_lo; e0 < e_hi; e0 += a.box_rows) {
                        if (src)
                            tma_load_5d(s + e0 * W, &a.tmap[buf], b, 0, 0, e0, (int)o, cb);
                        else
                            tma_load_3d(s + e0 * W, &a.tmap[buf], b, a.col0 + cb * W, e0, (int)o);
                    }
                }
            }
            // bounded wait (~1 s at 2 GHz): on time-out the tile is poisoned with NaN, which the
            // z pass counts as non-finite cells (SMK_ENULLBOX from smk_grf_check), and the
            // block stops after a last bounded wait for its copies (in parts: the later parts' waits
            // and the poisoning happen inside the transform, after its first stage)
            if (!mbar_wait_bounded(&bar[0], parity, a.tma_wait_limit)) timed_out = 1;
            if (ns == 1) {
                parity ^= 1u;
                __syncthreads();
                if (timed_out) {
                    if (threadIdx.x == 0) mbar_wait_bounded(&bar[0], parity ^ 1u, a.tma_wait_limit);
                    __syncthreads();
                    for (int i = threadIdx.x; i < n * W; i += T) s[i] = make_float2(__int_as_float(0x7fc00000), 0.f);
                    __syncthreads();
                }
            }
        } else if (src) {
            // W / src_kb contiguous runs of n * src_kb complex values, 16 bytes per copy
            const int kb = a.src_kb, G = W / 2;
            for (int idx = threadIdx.x; idx < n * G; idx += T) {
                const int e = idx / G, w = 2 * (idx % G);
                const int c = cb * W + w;
                cp_async<16>(s + e * W + w, src + (((int64_t)(c / kb) * a.n_outer + o) * n + e) * kb + c % kb, 16);
            }
            cp_async_wait_all();
            __syncthreads();
        } else {
            load_cols_async<W, T>(s, base, n, a.estride, cols);
            cp_async_wait_all();
            __syncthreads();
        }
        if (src) {
            // the next tile's source runs into L2, once the current tile's (first part) has
            // arrived (issued with the current tile's loads, or two tiles ahead, measured slower)
            if (a.prefetch && threadIdx.x == 0) prefetch_src(tile);
        } else if (a.prefetch && tile + gridDim.x < ntiles) {
            // the next tile of this block: one line per row segment of its W columns
            const int64_t tn = tile + gridDim.x;
            const int bn = (int)(tn / tpb);
            const int64_t un = tn - bn * tpb;
            const int64_t on = un / ncolt;
            const float2* nb = a.base[bn] + on * a.ostride + a.col0 + (un - on * ncolt) * W;
            for (int e = threadIdx.x; e < n; e += T) prefetch_l2(nb + (int64_t)e * a.estride);
        }
        if (INV && a.tma == 2) {
            // transform in shared memory, then TMA tensor stores of the tile (columns past ncol
            // are not written); the next load waits until these stores have read s
            fft_tile<true, W, W, T, C::RMAX, C::NF>(s, tw, a.pl);
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int e0 = 0; e0 < n; e0 += a.box_rows) tma_store_3d(&a.tmap[buf], s + e0 * W, cb * W, e0, (int)o);
                bulk_commit();
            }
        } else if constexpr (INV) {
            // the last stage stores straight from registers
            const int64_t es = a.estride;
            auto store = [&](int e, int w, float2 v) {
                if (w < cols) base[e * es + w] = v;
            };
            if constexpr (C::NF > 0) {
                // the leading stages whose groups stay inside a half run half by half (two for
                // the plan 16,16,10 at 2560: groups of 10 and of 160 rows)
                constexpr int D2 = parts_depth<C::NF, C::RMAX>(2) >= 2 ? 2 : 1;
                if (ns > 1) {
                    ifft_tile_out_parts<W, W, T, C::RMAX, C::NF, D2>(s, tw, ns, [&](int p) {
                        if (!mbar_wait_bounded(&bar[p], parity, a.tma_wait_limit)) timed_out = 1;
                    }, [&]() {
                        parity ^= 1u;
                        if (timed_out) {
                            if (threadIdx.x == 0)
                                for (int p = 0; p < ns; ++p) mbar_wait_bounded(&bar[p], parity ^ 1u, a.tma_wait_limit);
                            __syncthreads();
                            for (int i = threadIdx.x; i < n * W; i += T) s[i] = make_float2(__int_as_float(0x7fc00000), 0.f);
                            __syncthreads();
                        }
                    }, store);
                } else {
                    ifft_tile_out<W, W, T, C::RMAX, C::NF>(s, tw, a.pl, store);
                }
            } else {
                ifft_tile_out<W, W, T, C::RMAX, C::NF>(s, tw, a.pl, store);
            }
        } else {
            fft_tile<INV, W, W, T, C::RMAX, C::NF>(s, tw, a.pl);
            if (a.dst)
                store_blocked<W, T>(s, a.dst, n, a.dst_kb, a.n_outer, o, cb);
            else
                store_cols<W, T>(s, base, n, a.estride, cols);
        }
        if (a.tma) fence_proxy_async_smem();   // this tile's shared accesses before the next TMA writes
        __syncthreads();
        if (timed_out) break;
    }
    if (a.tma == 2 && threadIdx.x == 0) bulk_wait_all();
}

// Row swizzle of an x-pass tile (tile_row): the compile-time plan's last radix when it is even,
// the other stages' strides are multiples of it and the tile has 64-byte rows (W = 8), else none.
template <class C>
constexpr int xpass_row_swizzle() {
    if constexpr (C::NF > 0 && C::W == 8) {
        constexpr FftPlan P = FixedPlan<C::NF, C::RMAX>::P;
        constexpr int RL = P.r[P.nst - 1];
        bool ok = RL % 2 == 0;
        for (int st = 0; st + 1 < P.nst; ++st) ok = ok && P.m[st] % RL == 0;
        return ok ? RL : 0;
    } else {
        return 0;
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
    int eta_comp;          // SMK_ETA_*: eta_ij = k_i k_j / k^2 delta_k, or a velocity component
    float vfac;            // velocity: H0 * dD/dz(0)
    // xpi_kernel: the blocked intermediate of XGenArgs (I[0] delta, I[1] eta or null) and the
    // k_z column blocks [cb0, cb0 + ncb) of this chunk; prefetch: pull the next tile's rows into
    // L2 while transforming the current one
    float2* I[2];
    int cb0, ncb;
    int prefetch;
    // xpi_kernel source: the boxes (null) or the blocked layout of I[0] that the y forward wrote
    // (the tile's rows ny * WC * 8 bytes apart instead of ny * pitch * 4; read, then overwritten
    // by the tile itself)
    int src_blocked;
};

// k_i k_j of the eta component (SMK_ETA_*), float32 product as numpy forms kx*ky
__device__ __forceinline__ float eta_num(int comp, float kx, float ky, float kz) {
    switch (comp) {
        case SMK_ETA_XX: return __fmul_rn(kx, kx);
        case SMK_ETA_YY: return __fmul_rn(ky, ky);
        case SMK_ETA_XY: return __fmul_rn(kx, ky);
        case SMK_ETA_XZ: return __fmul_rn(kx, kz);
        case SMK_ETA_YZ: return __fmul_rn(ky, kz);
        default: return __fmul_rn(kz, kz);
    }
}

// The second output of the x pass from delta_k: eta_ij = k_i k_j / k^2 delta_k (components 0..5)
// or velocity v_i = -i k_i / k^2 * vfac * delta_k (SMK_ETA_VX/VY/VZ); kk1 = k^2 with k^2(0) = 1.
// EXACT: correctly rounded quotient (the host-noise path, compared with the reference's arrays).
template <bool EXACT>
__device__ __forceinline__ float2 eta_apply(int comp, float2 d, float kx, float ky, float kz, float kk1,
                                            float vfac) {
    if (comp >= SMK_ETA_VX) {
        const float ki = comp == SMK_ETA_VX ? kx : (comp == SMK_ETA_VY ? ky : kz);
        const float f = (EXACT ? __fdiv_rn(ki, kk1) : __fdividef(ki, kk1)) * vfac;
        return make_float2(d.y * f, -d.x * f);
    }
    const float num = eta_num(comp, kx, ky, kz);
    return cscale(d, EXACT ? __fdiv_rn(num, kk1) : __fdividef(num, kk1));
}

__device__ __forceinline__ float kaxis(int i, int n, double kfac, bool full) {
    // numpy fftfreq / rfftfreq times 2 k_ny, rounded to float32 (bin/make_boxes.py:299-302)
    const int ii = (full && i >= (n + 1) / 2) ? i - n : i;
    return (float)(((double)ii * (1.0 / (double)n)) * kfac);
}

// smem: s[n*W] | tw[n] | kx[n] (k_x of each slot) | ix[n] (frequency index of each slot) |
//       kt[W+1] (k_y of the tile, k_z of its columns)
template <class C>
__global__ void __launch_bounds__(C::T, C::MINB) xpass_kernel(const XArgs a) {
    constexpr int W = C::W, T = C::T;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;  // == nx
    float2* s = smem;
    float2* tw = s + n * W;
    float* kx = reinterpret_cast<float*>(tw + n);
    int* ix = reinterpret_cast<int*>(kx + n);
    float* kt = reinterpret_cast<float*>(ix + n);
    fill_stage_twiddles(tw, a.pl);
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
        fft_tile<false, W, W, T, C::RMAX, C::NF>(s, tw, a.pl);
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
                pb[e * estride + w] = eta_apply<true>(a.eta_comp, d, kxv, ky, kz, kk1, a.vfac);
            }
        }
        __syncthreads();
        fft_tile<true, W, W, T, C::RMAX, C::NF>(s, tw, a.pl);
        store_cols<W, T>(s, pa, n, estride, cols);
        __syncthreads();
        if (pb) {
            // each thread reads back (plain loads, L2) exactly the eta_k elements it wrote above
            for (int idx = threadIdx.x; idx < n * W; idx += T) {
                const int e = idx / W, w = idx % W;
                s[idx] = w < cols ? __ldcg(pb + e * estride + w) : make_float2(0.f, 0.f);
            }
            __syncthreads();
            fft_tile<true, W, W, T, C::RMAX, C::NF>(s, tw, a.pl);
            store_cols<W, T>(s, pb, n, estride, cols);
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------ host-noise x pass into the
// blocked intermediate
// Tiles (box b, column block kb, y slot), y slot fastest, of KB = W/2 k_z columns (W with delta
// only): load the KB columns of the noise spectrum (after the y forward pass) for every x,
// forward x FFT of those KB lines (tile pitch W), x sqrt(P/Vcell) and the eta split into lines
// KB..W-1 of the same tile, inverse x FFT of the W lines, last stage stored from registers into
// the intermediate (layout of XGenArgs::I).  Same arithmetic as xpass_kernel per line.
// smem: s[n*W] | tw[n] | kx[n] | ix[n] | kt[W+1]
template <class C, bool BOTH>
__global__ void __launch_bounds__(C::T, C::MINB) xpi_kernel(const XArgs a) {
    constexpr int W = C::W, T = C::T;
    constexpr int KB = W / 2;
    constexpr int SWR = xpass_row_swizzle<C>();   // rows of the tile in the tile_row order
    extern __shared__ __align__(128) float2 smem[];
    const int n = a.pl.n;  // == nx
    float2* s = smem;
    float2* tw = s + n * W;
    float* kx = reinterpret_cast<float*>(tw + n);
    int* ix = reinterpret_cast<int*>(kx + n);
    float* kt = reinterpret_cast<float*>(ix + n);
    fill_stage_twiddles(tw, a.pl);
    for (int e = threadIdx.x; e < n; e += T) {
        const int f = freq_of_slot(a.pl, e);
        ix[e] = f;
        kx[e] = kaxis(f, n, a.kfac, true);
    }
    float amp = 0.f;
    if (a.pk_mode == SMK_PK_ANALYTIC) amp = (float)(a.amp_host > 0.0 ? a.amp_host : *a.amp_dev);
    constexpr bool both = BOTH;       // both fields (I[1] set): the launcher's choice of instance
    constexpr int WC = BOTH ? KB : W;  // k_z columns per tile
    const int64_t ntiles = (int64_t)a.batch * a.ncb * a.ny;
    const int64_t nouter = (int64_t)a.batch * a.nx;
    const int64_t estride = (int64_t)a.ny * a.cp;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int yslot = (int)(tile % a.ny);
        const int64_t r = tile / a.ny;
        const int kbl = (int)(r % a.ncb);
        const int64_t b = r / a.ncb;
        const int cb = a.cb0 + kbl;
        const int cols = min(WC, a.nzh - cb * WC);
        const int64_t row0 = ((int64_t)kbl * nouter + b * a.nx) * a.ny + yslot;
        const int64_t es = (int64_t)a.ny * WC;
        // WC columns (16-byte copies of column pairs, zero past nzh) into lines 0..WC-1 of the tile
        const float2* pa = a.src_blocked ? a.I[0] + row0 * WC
                                         : a.A + b * (int64_t)a.nx * estride + (int64_t)yslot * a.cp + (int64_t)cb * WC;
        const int64_t rs = a.src_blocked ? es : estride;
        for (int idx = threadIdx.x; idx < n * (WC / 2); idx += T) {
            const int e = idx / (WC / 2), w = 2 * (idx % (WC / 2));
            const int bytes = w < cols ? (w + 1 < cols ? 16 : 8) : 0;
            cp_async<16>(s + tile_row<SWR>(e) * W + w, bytes ? pa + e * rs + w : pa, bytes);
        }
        const int iy = freq_of_slot(a.ply, yslot);
        if (threadIdx.x == 0) kt[0] = kaxis(iy, a.ny, a.kfac, true);
        if (threadIdx.x < WC) kt[1 + threadIdx.x] = kaxis(cb * WC + threadIdx.x, 2 * (a.nzh - 1), a.kfac, false);
        cp_async_wait_all();
        __syncthreads();
        if (a.prefetch && tile + gridDim.x < ntiles) {
            // the next tile's nx row pieces (one line each) into L2
            const int64_t tn = tile + gridDim.x;
            const int64_t rn = tn / a.ny;
            const float2* pn = a.src_blocked
                ? a.I[0] + (((int64_t)(rn % a.ncb) * nouter + (rn / a.ncb) * a.nx) * a.ny + tn % a.ny) * WC
                : a.A + (rn / a.ncb) * (int64_t)a.nx * estride + (int64_t)(tn % a.ny) * a.cp +
                      (int64_t)(a.cb0 + (int)(rn % a.ncb)) * WC;
            for (int e = threadIdx.x; e < n; e += T) prefetch_l2(pn + e * rs);
        }
        if (both)
            fft_tile<false, KB, W, T, C::RMAX, C::NF, SWR>(s, tw, a.pl);
        else
            fft_tile<false, W, W, T, C::RMAX, C::NF, SWR>(s, tw, a.pl);
        const float ky = kt[0];
        // two adjacent columns per thread, read and written as 16-byte pieces (rows are 64 B
        // apart, so 8-byte accesses of lanes on rows e and e + 2 met on the same banks)
        for (int idx = threadIdx.x; idx < n * (WC / 2); idx += T) {
            const int e = idx / (WC / 2), w0 = 2 * (idx % (WC / 2));
            const float kxv = kx[e];
            float2* row = s + tile_row<SWR>(e) * W;
            const float4 in = *reinterpret_cast<const float4*>(row + w0);
            float2 d[2] = {make_float2(in.x, in.y), make_float2(in.z, in.w)}, et[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int w = w0 + h;
                const float kz = kt[1 + w];
                // k^2 in float32 without contraction, as numpy evaluates kx*kx + ky*ky + kz*kz
                const float kk = __fadd_rn(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
                float sc;
                if (a.pk_mode == SMK_PK_GRID) {
                    sc = w < cols ? __ldg(a.grid + ((int64_t)ix[e] * a.ny + iy) * a.nzh + cb * WC + w) : 0.f;
                } else {
                    const float k = __fsqrt_rn(kk);
                    const float kr = k * a.inv_k0;
                    const float den = fmaf(kr, kr, 1.0f);
                    sc = sqrtf(amp * k / (den * den) * a.inv_vcell);
                }
                d[h] = cscale(d[h], sc);
                if (both) {
                    const float kk1 = (kk == 0.0f) ? 1.0f : kk;  // k^2[0,0,0] = 1 (bin/make_boxes.py:306)
                    et[h] = eta_apply<true>(a.eta_comp, d[h], kxv, ky, kz, kk1, a.vfac);
                }
            }
            *reinterpret_cast<float4*>(row + w0) = make_float4(d[0].x, d[0].y, d[1].x, d[1].y);
            if (both)
                *reinterpret_cast<float4*>(row + KB + w0) = make_float4(et[0].x, et[0].y, et[1].x, et[1].y);
        }
        __syncthreads();
        float2* d0 = a.I[0] + row0 * WC;
        float2* d1 = both ? a.I[1] + row0 * WC : nullptr;
        // I holds whole column blocks, so every column of the tile is stored (those past nzh
        // were loaded as zeros and stay zero)
        ifft_tile_out<W, W, T, C::RMAX, C::NF, SWR>(s, tw, a.pl, [&](int e, int w, float2 v) {
            const int f = both && w >= WC;
            const int c = w - f * WC;
            (f ? d1 : d0)[e * es + c] = v;
        });
        __syncthreads();
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
    uint32_t rk0[10], rk1[10];  // Philox round keys of seed (box 0; batch 1 uses them directly)
    int eta_comp;
    float vfac;
    int fields;            // XGEN_BOTH: W/2 delta + W/2 eta lines per tile; XGEN_DELTA / XGEN_ETA:
                           // W lines of one field (two launches; see xgen_split)
    // Intermediate output (xgi_kernel): field f of k_z column block kb (kb - cb0 within this
    // chunk; blocks of KB = W / fields columns) at I[f] + (((kb - cb0) * batch * nx + b * nx + x)
    // * ny + yslot) * KB + kz % KB: the x rows of a tile lie ny * KB * 8 bytes apart, and the y
    // line of one column block is one contiguous run for the y pass
    float2* I[2];
    int cb0, ncb;          // column blocks of this chunk
};

// GPU-noise mode arithmetic (no bit-level reference: the FP64 oracle restates the drawn modes
// and the boxes are compared within the FP32 tolerance).  k^2 is formed as numpy does it
// (kx*kx + ky*ky + kz*kz, no contraction); r = 1/k from the hardware reciprocal square root;
// 1/k^2 = r*r (1 at k = 0, where the reference sets k^2[0,0,0] = 1).
__device__ __forceinline__ float mode_k2(float kxv, float ky, float kz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
}
__device__ __forceinline__ float mode_inv_k2(float kk) {
    const float r = hw_rsqrt(kk);
    return kk > 0.0f ? r * r : 1.0f;
}

// Second output of the GPU-noise x pass from delta_k and 1/k^2: eta_ij = k_i k_j / k^2 delta_k,
// or velocity v_i = -i k_i / k^2 * vfac * delta_k (SMK_ETA_VX/VY/VZ).
template <int COMP = -1>   // COMP >= 0: the component fixed at compile time (no per-mode switch)
__device__ __forceinline__ float2 eta_from_inv_k2(int comp_rt, float2 d, float kx, float ky, float kz, float ikk,
                                                  float vfac) {
    const int comp = COMP >= 0 ? COMP : comp_rt;
    if (comp >= SMK_ETA_VX) {
        const float ki = comp == SMK_ETA_VX ? kx : (comp == SMK_ETA_VY ? ky : kz);
        const float f = ki * ikk * vfac;
        return make_float2(d.y * f, -d.x * f);
    }
    return cscale(d, eta_num(comp, kx, ky, kz) * ikk);
}

// Per-launch constant of the analytic P(k) scale: sqrt(N/2) * sqrt(A / Vcell), so that
// sqrt(N/2) * sqrt(P(k)/Vcell) = scale_c / sqrt((1 + k^2/k0^2)^2 / k) for P = A k/(1+(k/k0)^2)^2.
__device__ __forceinline__ float pk_scale_c(const XGenArgs& a) {
    if (a.pk_mode != SMK_PK_ANALYTIC) return a.sig_c;
    const float amp = (float)(a.amp_host > 0.0 ? a.amp_host : *a.amp_dev);
    return a.sig_c * sqrtf(amp * a.inv_vcell);
}

// delta_k of the modes (ix, iy, kz0) and (ix, iy, kz0 + 1) of one box (GPU noise):
// Philox4x32-10 block (kz0/2, ix, iy, STREAM_KMODE) keyed by seed, Box-Muller, Re/Im ~ N(0, N/2),
// times sqrt(P/Vcell).  CHECK (tiles holding the kz = 0 or nz/2 plane, or columns past nzh):
// on the kz = 0 and nz/2 planes the lower flat index of (ix, iy) and (-ix, -iy) owns the draw
// and self-conjugate modes are real with variance N; kz >= nzh gives 0.  Also returns k_z and
// 1/k^2 per mode for the eta split.
struct ModePair {
    float2 d[2];
    float kz[2], ikk[2];
};
template <bool CHECK, int PKM = -1>   // PKM >= 0: the P(k) mode fixed at compile time
__device__ __forceinline__ ModePair draw_pair(const XGenArgs& a, uint64_t seed, int ixe, int iy, int iym,
                                              float kxv, float ky, int kz0, const float* kzt, float scale_c) {
    ModePair mp;
    float g[4];
    {
        u32x4 ctr;
        ctr.v[0] = (uint32_t)(kz0 >> 1);
        ctr.v[1] = (uint32_t)ixe;
        ctr.v[2] = (uint32_t)iy;
        ctr.v[3] = STREAM_KMODE;
        gauss4(philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32)), g);
    }
    const float inv_k0sq = a.inv_k0 * a.inv_k0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int kz = kz0 + h;
        float2 X = make_float2(g[2 * h], g[2 * h + 1]);
        float sc = scale_c;
        if (CHECK) {
            mp.d[h] = make_float2(0.f, 0.f);
            mp.kz[h] = 0.f;
            mp.ikk[h] = 1.f;
            if (kz >= a.nzh) continue;
            if (kz == 0 || kz == a.nz / 2) {
                const int ixm = ixe == 0 ? 0 : a.nx - ixe;
                if (ixm == ixe && iym == iy) {
                    X = make_float2(g[2 * h], 0.f);
                    sc *= a.sig_r / a.sig_c;
                } else if ((int64_t)ixe * a.ny + iy > (int64_t)ixm * a.ny + iym) {
                    // the partner (-kx, -ky) owns the draw: take its conjugate
                    u32x4 ctr;
                    ctr.v[0] = (uint32_t)(kz0 >> 1);
                    ctr.v[1] = (uint32_t)ixm;
                    ctr.v[2] = (uint32_t)iym;
                    ctr.v[3] = STREAM_KMODE;
                    float gm[4];
                    gauss4(philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32)), gm);
                    X = make_float2(gm[2 * h], -gm[2 * h + 1]);
                }
            }
        }
        const float kz_ = kzt[kz];
        const float kk = mode_k2(kxv, ky, kz_);
        const float r = hw_rsqrt(kk);   // 1/k (+inf at k = 0)
        if ((PKM >= 0 ? PKM : a.pk_mode) == SMK_PK_GRID) {
            sc *= __ldg(a.grid + ((int64_t)ixe * a.ny + iy) * a.nzh + kz);
        } else {
            // sqrt(k)/den = 1/sqrt(den^2/k): one reciprocal square root (0 at k = 0)
            const float den = fmaf(kk, inv_k0sq, 1.0f);
            sc *= hw_rsqrt(den * den * r);
        }
        mp.d[h] = cscale(X, sc);
        mp.kz[h] = kz_;
        mp.ikk[h] = kk > 0.0f ? r * r : 1.0f;
    }
    return mp;
}
enum { XGEN_BOTH = 0, XGEN_DELTA = 1, XGEN_ETA = 2 };

// True when the k_z columns [c0, c0 + w) include the kz = 0 or nz/2 plane or run past nzh.
__device__ __forceinline__ bool tile_needs_check(const XGenArgs& a, int c0, int w) {
    return c0 == 0 || (c0 <= a.nz / 2 && a.nz / 2 < c0 + w) || c0 + w > a.nzh;
}

// smem: s[n*W] | tw[n] | kx[n] | ix[n] | kzt[nzh]
// ONE: one field per launch (a.fields = XGEN_DELTA or XGEN_ETA, W columns per tile), else
// XGEN_BOTH (W/2 columns, each drawn once for both fields).
template <class C, bool ONE>
__global__ void __launch_bounds__(C::T, C::MINB) xgen_kernel(const XGenArgs a) {
    constexpr int W = C::W, T = C::T;
    constexpr int WC = ONE ? W : W / 2;   // k_z columns per tile
    constexpr int NP = WC / 2;
    extern __shared__ float2 smem[];
    const int n = a.pl.n;  // == nx
    float2* s = smem;
    float2* tw = s + n * W;
    float* kx = reinterpret_cast<float*>(tw + n);
    int* ix = reinterpret_cast<int*>(kx + n);
    float* kzt = reinterpret_cast<float*>(ix + n);
    fill_stage_twiddles(tw, a.pl);
    for (int e = threadIdx.x; e < n; e += T) {
        const int f = freq_of_slot(a.pl, e);
        ix[e] = f;
        kx[e] = kaxis(f, n, a.kfac, true);
    }
    for (int z = threadIdx.x; z < a.nzh; z += T) kzt[z] = kaxis(z, a.nz, a.kfac, false);
    __syncthreads();
    const float scale_c = pk_scale_c(a);
    const int64_t ncolt = ceil_div(a.nzh, WC);
    const int64_t nouter = (int64_t)a.batch * a.ny;
    const int64_t ntiles = nouter * ncolt;
    const int64_t estride = (int64_t)a.ny * a.cp;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t o = tile / ncolt;   // b*ny + y slot
        const int cb = (int)(tile - o * ncolt);
        const int64_t b = o / a.ny;
        const int yslot = (int)(o - b * a.ny);
        const int iy = freq_of_slot(a.ply, yslot);
        const int iym = iy == 0 ? 0 : a.ny - iy;
        const float ky = kaxis(iy, a.ny, a.kfac, true);
        const uint64_t seed = a.seed + (uint64_t)b;
        auto draw = [&](auto chk) {
#pragma unroll 2
            for (int idx = threadIdx.x; idx < n * NP; idx += T) {
                const int e = idx / NP, pr = idx % NP;
                const int c0 = 2 * pr, kz0 = cb * WC + c0;
                const float kxv = kx[e];
                const ModePair mp = draw_pair<decltype(chk)::value>(a, seed, ix[e], iy, iym, kxv, ky, kz0, kzt, scale_c);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float2 et = make_float2(0.f, 0.f);
                    if (!ONE || a.fields == XGEN_ETA) et = eta_from_inv_k2(a.eta_comp, mp.d[h], kxv, ky, mp.kz[h], mp.ikk[h], a.vfac);
                    if (!ONE) {
                        s[e * W + c0 + h] = mp.d[h];
                        s[e * W + WC + c0 + h] = et;
                    } else {
                        s[e * W + c0 + h] = a.fields == XGEN_DELTA ? mp.d[h] : et;
                    }
                }
            }
        };
        if (tile_needs_check(a, cb * WC, WC))
            draw(std::true_type{});
        else
            draw(std::false_type{});
        __syncthreads();
        const int cols = min(WC, a.nzh - cb * WC);
        const int64_t off = b * (int64_t)a.nx * estride + (int64_t)yslot * a.cp + (int64_t)cb * WC;
        if constexpr (ONE) {
            // the last stage stores straight from registers
            float2* dst = (a.fields == XGEN_DELTA ? a.A : a.B) + off;
            ifft_tile_out<W, W, T, C::RMAX, C::NF>(s, tw, a.pl, [&](int e, int w, float2 v) {
                if (w < cols) dst[e * estride + w] = v;
            });
        } else {
            fft_tile<true, W, W, T, C::RMAX, C::NF>(s, tw, a.pl);
            for (int idx = threadIdx.x; idx < n * W; idx += T) {
                const int e = idx / W, l = idx % W;
                const int c = l < WC ? l : l - WC;
                if (c < cols) {
                    float2* dst = l < WC ? a.A : a.B;
                    if (dst) dst[off + e * estride + c] = s[idx];
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ GPU-noise x pass into the
// blocked intermediate
// Tiles (box b, column block kb, y slot), y slot fastest: a tile draws the modes of its WC k_z
// columns for every x slot once, forms delta_k (and eta_k with XGEN_BOTH), takes the x inverse
// of its W lines and stores the last stage from registers into I (see XGenArgs).  Tiles that
// run together hold neighbouring y slots, so their 8 * KB-byte pieces of a row of I are
// assembled into whole lines in L2.
// smem: s[n*W] | tw[n] | kxi[n] (k_x, frequency index) | kzt[nzh]
template <class C>
__global__ void __launch_bounds__(C::T, C::MINB) xgi_kernel(const XGenArgs a) {
    constexpr int W = C::W, T = C::T;
    // compile-time plan with an even last radix on 64-byte rows: rows in the tile_row order
    constexpr int SWR = xpass_row_swizzle<C>();
    extern __shared__ __align__(128) float2 smem[];
    const bool both = a.fields == XGEN_BOTH;
    const int WC = both ? W / 2 : W;          // k_z columns per tile (= KB)
    const int n = a.pl.n;  // == nx
    float2* s = smem;
    float2* tw = s + n * W;
    float2* kxi = tw + n;                     // slot e: (k_x, frequency index as int bits)
    float* kzt = reinterpret_cast<float*>(kxi + n);
    fill_stage_twiddles(tw, a.pl);
    for (int e = threadIdx.x; e < n; e += T) {
        const int f = freq_of_slot(a.pl, e);
        kxi[e] = make_float2(kaxis(f, n, a.kfac, true), __int_as_float(f));
    }
    for (int z = threadIdx.x; z < a.nzh; z += T) kzt[z] = kaxis(z, a.nz, a.kfac, false);
    __syncthreads();
    const float scale_c = pk_scale_c(a);
    const int64_t ntiles = (int64_t)a.batch * a.ncb * a.ny;
    const int64_t nouter = (int64_t)a.batch * a.nx;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int yslot = (int)(tile % a.ny);
        const int64_t r = tile / a.ny;
        const int kbl = (int)(r % a.ncb);      // block within the chunk
        const int64_t b = r / a.ncb;
        const int cb = a.cb0 + kbl;
        const int iy = freq_of_slot(a.ply, yslot);
        const int iym = iy == 0 ? 0 : a.ny - iy;
        const float ky = kaxis(iy, a.ny, a.kfac, true);
        const uint64_t seed = a.seed + (uint64_t)b;
        // the column count per tile as a constant (BOTH: W/2 columns of each field, else W of one);
        // FAST: analytic P(k) and eta_zz fixed at compile time (no per-mode switches)
        auto draw = [&](auto chk, auto both_c, auto fast_c, auto rk_c) {
            constexpr bool BOTH = decltype(both_c)::value, FAST = decltype(fast_c)::value;
            constexpr bool RK = decltype(rk_c)::value;   // one box: the round keys from the parameters
            constexpr int WCC = BOTH ? W / 2 : W, NPC = WCC / 2;
            constexpr int PKM = FAST ? SMK_PK_ANALYTIC : -1, COMP = FAST ? SMK_ETA_ZZ : -1;
            if constexpr (FAST && BOTH && !decltype(chk)::value) {
                // the same arithmetic as draw_pair + eta_from_inv_k2, with the column pair fixed per
                // thread (T is a multiple of NPC): its k_z and k_z^2 and the tile's k_y^2 stay in
                // registers across the rows
                static_assert(T % NPC == 0, "a thread keeps one column pair");
                const int pr = threadIdx.x % NPC, c0 = 2 * pr, kz0 = cb * WCC + c0;
                const float kzz[2] = {__fmul_rn(kzt[kz0], kzt[kz0]), __fmul_rn(kzt[kz0 + 1], kzt[kz0 + 1])};
                const float kyy = __fmul_rn(ky, ky);
                const float inv_k0sq = a.inv_k0 * a.inv_k0;
#pragma unroll 2
                for (int e = threadIdx.x / NPC; e < n; e += T / NPC) {
                    const float2 kq = kxi[e];
                    float g[4];
                    u32x4 ctr;
                    ctr.v[0] = (uint32_t)(kz0 >> 1);
                    ctr.v[1] = (uint32_t)__float_as_int(kq.y);
                    ctr.v[2] = (uint32_t)iy;
                    ctr.v[3] = STREAM_KMODE;
                    if constexpr (RK)
                        gauss4(philox4x32_10_rk(ctr, a.rk0, a.rk1), g);
                    else
                        gauss4(philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32)), g);
                    const float kxy = __fadd_rn(__fmul_rn(kq.x, kq.x), kyy);
                    float2 v[2][2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const float kk = __fadd_rn(kxy, kzz[h]);
                        const float r = hw_rsqrt(kk);
                        const float den = fmaf(kk, inv_k0sq, 1.0f);
                        const float2 d = cscale(make_float2(g[2 * h], g[2 * h + 1]), scale_c * hw_rsqrt(den * den * r));
                        v[0][h] = d;
                        v[1][h] = cscale(d, kzz[h] * (kk > 0.0f ? r * r : 1.0f));
                    }
                    float2* row = s + tile_row<SWR>(e) * W;
                    *reinterpret_cast<float4*>(row + c0) = make_float4(v[0][0].x, v[0][0].y, v[0][1].x, v[0][1].y);
                    *reinterpret_cast<float4*>(row + WCC + c0) = make_float4(v[1][0].x, v[1][0].y, v[1][1].x, v[1][1].y);
                }
                return;
            }
#pragma unroll 2
            for (int idx = threadIdx.x; idx < n * NPC; idx += T) {
                const int e = idx / NPC, pr = idx % NPC;
                const int c0 = 2 * pr, kz0 = cb * WCC + c0;
                const float2 kq = kxi[e];
                const float kxv = kq.x;
                const ModePair mp = draw_pair<decltype(chk)::value, PKM>(a, seed, __float_as_int(kq.y), iy, iym, kxv, ky, kz0, kzt, scale_c);
                // the two modes of a field as one 16-byte store (rows are 64 B apart, so 8-byte stores
                // of lanes on rows e and e + 2 met on the same banks)
                float2 v[2][2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float2 et = eta_from_inv_k2<COMP>(a.eta_comp, mp.d[h], kxv, ky, mp.kz[h], mp.ikk[h], a.vfac);
                    if constexpr (BOTH) {
                        v[0][h] = mp.d[h];
                        v[1][h] = et;
                    } else {
                        v[0][h] = a.fields == XGEN_DELTA ? mp.d[h] : et;
                    }
                }
                float2* row = s + tile_row<SWR>(e) * W;
                *reinterpret_cast<float4*>(row + c0) = make_float4(v[0][0].x, v[0][0].y, v[0][1].x, v[0][1].y);
                if constexpr (BOTH)
                    *reinterpret_cast<float4*>(row + WCC + c0) = make_float4(v[1][0].x, v[1][0].y, v[1][1].x, v[1][1].y);
            }
        };
        const bool fast = a.pk_mode == SMK_PK_ANALYTIC && a.eta_comp == SMK_ETA_ZZ;
        using F_ = std::false_type;
        using T_ = std::true_type;
        if (tile_needs_check(a, cb * WC, WC)) {
            if (both) draw(T_{}, T_{}, F_{}, F_{});
            else draw(T_{}, F_{}, F_{}, F_{});
        } else {
            if (both && fast && a.batch == 1) draw(F_{}, T_{}, T_{}, T_{});
            else if (both && fast) draw(F_{}, T_{}, T_{}, F_{});
            else if (both) draw(F_{}, T_{}, F_{}, F_{});
            else draw(F_{}, F_{}, F_{}, F_{});
        }
        __syncthreads();
        const int64_t row0 = ((int64_t)kbl * nouter + b * a.nx) * a.ny + yslot;
        float2* d0 = a.I[0] + row0 * WC;
        float2* d1 = both ? a.I[1] + row0 * WC : nullptr;
        const int64_t es = (int64_t)a.ny * WC;
        // I holds whole column blocks (a chunk is a multiple of 16 columns), so every column of the
        // tile is stored: those past nzh carry the zero modes the draw gives there
        ifft_tile_out<W, W, T, C::RMAX, C::NF, SWR>(s, tw, a.pl, [&](int e, int w, float2 v) {
            const int f = both && w >= WC;
            const int c = w - f * WC;
            (f ? d1 : d0)[e * es + c] = v;
        });
        __syncthreads();
    }
}

// ------------------------------------------------------------------ z inverse (c2r) + stats
struct ZInvArgs {
    FftPlan pl;
    ZTiling zt;             // set by the launcher from its tile width
    int batch;
    float* buf[2];
    int nbuf;
    int64_t pitch;
    float scale;
    double* stats;  // [batch][2][4] or null
    int prefetch;   // pull the next tile into L2 during the transform
};

// ------------------------------------------------------------------ z inverse, one warp per row pair
// c2r of row pairs + 1/N + FP64 statistics: every warp transforms its own row pair in
// a private region of shared memory and synchronises only with __syncwarp: the warps of an SM
// run out of phase, so one warp's loads, another's transform and a third's stores overlap.
// Slot p of a warp's line sits at zslot<SWZ>(p).  SWZ = 1: p ^ ((p >> 4) & 15), an XOR swizzle
// inside blocks of 16 slots that, with the odd radix in the middle of the plan ((16, 6, 16) for
// 1536, (16, 10, 16) for 2560), makes every stage's accesses conflict-free and spreads the
// digit-reversed scatter of the half spectrum over the banks.  SWZ = 0: p + (p >> 5), one pad
// per 32 slots (power-of-two lengths >= 2048, whose scatter the swizzle does not spread).
// SWZ = 2: p + (p >> 4), one pad per 16 slots (compile-time plans (16, x, 16) whose strides m are 1
// or multiples of 16: the R elements of a butterfly then lie a constant stride apart, and every
// stage and the scatter are conflict-free).
template <int SWZ>
__host__ __device__ __forceinline__ int zslot(int p) {
    return SWZ == 2 ? p + (p >> 4) : SWZ ? (p ^ ((p >> 4) & 15)) : p + (p >> 5);
}
__host__ __device__ __forceinline__ int zpad(int p) { return zslot<0>(p); }

// One stage of a warp's line (slots padded by zpad) with the plan's per-stage twiddles.
// LAST (the final stage of the inverse, m = n / R, natural-order outputs e = q + r m): the
// outputs go to out(e, v) instead of back to shared memory.
template <int R, bool INV, bool LAST, int SWZ, class Out>
__device__ __forceinline__ void warp_fft_stage(float2* __restrict__ s, const float2* __restrict__ stw,
                                               const FftPlan& pl, const int st, const int lane, Out&& out) {
    const int m = pl.m[st];
    const int nb = pl.n / R;
    const float2* tws = stw + pl.twoff[st];
    for (int j = lane; j < nb; j += 32) {
        const int blk = div_m(pl, st, j);
        const int q = j - blk * m;
        const int p0 = blk * R * m + q;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = s[zslot<SWZ>(p0 + r * m)];
        const float2* t = tws + q * (R - 1) - 1;
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
        if constexpr (LAST) {
#pragma unroll
            for (int r = 0; r < R; ++r) out(p0 + r * m, v[r]);
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) s[zslot<SWZ>(p0 + r * m)] = v[r];
        }
    }
    __syncwarp();
}

// Stage ST of the compile-time mid-ordered plan of length NF on a warp's line in the SWZ = 2
// layout: element r of butterfly (blk, q) sits at slot(blk R m + q) + r ES, ES = m + m/16 (m a
// multiple of 16) or 1 (m = 1, R = 16), so the loads and stores are immediate offsets from one
// base.  Same butterflies and twiddles as warp_fft_stage (bit-identical results).
template <int NF, int ST, bool LAST, class Out, bool INV = true>
__device__ __forceinline__ void warp_fft_stage_fixed(float2* __restrict__ s, const float2* __restrict__ stw,
                                                     const int lane, Out&& out) {
    using FP = FixedPlan<NF, 16, true>;
    constexpr int R = FP::P.r[ST], m = FP::P.m[ST];
    static_assert(m == 1 ? R == 16 : m % 16 == 0, "one-pad-per-16 layout needs strides 1 (R = 16) or 16k");
    constexpr int ES = m == 1 ? 1 : m + m / 16;
    constexpr int nb = NF / R;
    const float2* tws = stw + FP::P.twoff[ST];
    for (int j = lane; j < nb; j += 32) {
        const int blk = j / m;
        const int q = j - blk * m;
        const int p0 = blk * R * m + q;
        float2* b = s + zslot<2>(p0);
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = b[r * ES];
        const float2* t = tws + q * (R - 1) - 1;
        if constexpr (INV) {
            if constexpr (m > 1) {
                if (q != 0) {
#pragma unroll
                    for (int r = 1; r < R; ++r) v[r] = cmulc(v[r], t[r]);
                }
            }
            Dft<R, true>::run(v);
        } else {
            // forward: every butterfly of a stage with m > 1 multiplies (the q = 0 entries are 1,
            // exact), with no divergent branch around the twiddles (z forward 19.1 -> 18.6 ms; the
            // same in the inverse measured 0.3 ms slower)
            Dft<R, false>::run(v);
            if constexpr (m > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = cmul(v[r], t[r]);
            }
        }
        if constexpr (LAST) {
#pragma unroll
            for (int r = 0; r < R; ++r) out(p0 + r * m, v[r]);
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) b[r * ES] = v[r];
        }
    }
    __syncwarp();
}

// Inverse transform of a warp's line (digit-reversed slots in, natural order out): every stage
// but the last in place, the last one's outputs handed to out(e, value).  NF > 0: the compile-time
// mid-ordered plan of that length on the SWZ = 2 layout (the run-time plan on the XOR swizzle
// measured 38.8 ms at 1536 and its compile-time form 39.2 ms).
template <int RMAX, int SWZ, class Out, int NF = 0>
__device__ __forceinline__ void warp_ifft_out(float2* s, const float2* stw, const FftPlan& pl, const int lane,
                                              Out&& out) {
    auto none = [](int, float2) {};
    if constexpr (NF > 0) {
        static_assert(SWZ == 2, "compile-time warp plans use the one-pad-per-16 layout");
        constexpr int NST = FixedPlan<NF, 16, true>::P.nst;
        static_for<0, NST - 1>([&](auto c) {
            warp_fft_stage_fixed<NF, NST - 1 - decltype(c)::value, false>(s, stw, lane, none);
        });
        warp_fft_stage_fixed<NF, 0, true>(s, stw, lane, out);
        return;
    }
    for (int st = pl.nst - 1; st >= 0; --st) {
        const bool last = st == 0;
#define SMK_WSTAGE(RR)                                                              \
    if (last)                                                                       \
        warp_fft_stage<RR, true, true, SWZ>(s, stw, pl, st, lane, out);             \
    else                                                                            \
        warp_fft_stage<RR, true, false, SWZ>(s, stw, pl, st, lane, none);
        switch (pl.r[st]) {
            case 32:
                if constexpr (RMAX >= 32) { SMK_WSTAGE(32) }
                break;
            case 16:
                if constexpr (RMAX >= 16) { SMK_WSTAGE(16) }
                break;
            case 10:
                if constexpr (RMAX >= 16) { SMK_WSTAGE(10) }
                break;
            case 6:
                if constexpr (RMAX >= 16) { SMK_WSTAGE(6) }
                break;
            case 8: SMK_WSTAGE(8) break;
            case 4: SMK_WSTAGE(4) break;
            case 2: SMK_WSTAGE(2) break;
            case 3: SMK_WSTAGE(3) break;
            default: SMK_WSTAGE(5) break;
        }
#undef SMK_WSTAGE
    }
}

// The output positions e that warp_ifft_out hands to a lane (its final-stage butterflies).
template <class F>
__device__ __forceinline__ void warp_out_positions(const FftPlan& pl, const int lane, F&& f) {
    const int R = pl.r[0], m = pl.m[0];
    for (int j = lane; j < m; j += 32)
        for (int r = 0; r < R; ++r) f(j + r * m);
}

// Warp-level sums of three doubles; lane 0 adds them to dst[0..2].
__device__ __forceinline__ void warp_flush_stats(double s1, double s2, double bad, double* dst) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s1 += __shfl_down_sync(0xffffffffu, s1, off);
        s2 += __shfl_down_sync(0xffffffffu, s2, off);
        bad += __shfl_down_sync(0xffffffffu, bad, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(dst, s1);
        atomicAdd(dst + 1, s2);
        atomicAdd(dst + 2, bad);
    }
}

// Forward transform of a warp's line (natural-order slots in, digit-reversed out), in place.
template <int RMAX, int SWZ, int NF = 0>
__device__ __forceinline__ void warp_fft_fwd(float2* s, const float2* stw, const FftPlan& pl, const int lane) {
    auto none = [](int, float2) {};
    if constexpr (NF > 0) {
        // the compile-time mid-ordered plan on the SWZ = 2 layout (same butterflies and twiddles)
        static_assert(SWZ == 2, "compile-time warp plans use the one-pad-per-16 layout");
        constexpr int NST = FixedPlan<NF, 16, true>::P.nst;
        static_for<0, NST>([&](auto c) {
            warp_fft_stage_fixed<NF, decltype(c)::value, false, decltype(none)&, false>(s, stw, lane, none);
        });
        return;
    }
    for (int st = 0; st < pl.nst; ++st) {
        switch (pl.r[st]) {
            case 32:
                if constexpr (RMAX >= 32) warp_fft_stage<32, false, false, SWZ>(s, stw, pl, st, lane, none);
                break;
            case 16:
                if constexpr (RMAX >= 16) warp_fft_stage<16, false, false, SWZ>(s, stw, pl, st, lane, none);
                break;
            case 10:
                if constexpr (RMAX >= 16) warp_fft_stage<10, false, false, SWZ>(s, stw, pl, st, lane, none);
                break;
            case 6:
                if constexpr (RMAX >= 16) warp_fft_stage<6, false, false, SWZ>(s, stw, pl, st, lane, none);
                break;
            case 8: warp_fft_stage<8, false, false, SWZ>(s, stw, pl, st, lane, none); break;
            case 4: warp_fft_stage<4, false, false, SWZ>(s, stw, pl, st, lane, none); break;
            case 2: warp_fft_stage<2, false, false, SWZ>(s, stw, pl, st, lane, none); break;
            case 3: warp_fft_stage<3, false, false, SWZ>(s, stw, pl, st, lane, none); break;
            default: warp_fft_stage<5, false, false, SWZ>(s, stw, pl, st, lane, none); break;
        }
    }
}

// Shared memory of zinvw_kernel for `warps` warps: stw[twn] | sof[n] | per-warp lines.
__host__ __device__ inline size_t zinvw_line_slots(int n, int swz) {
    return swz == 2 ? (size_t)zslot<2>(n - 1) + 1 : swz ? (size_t)(n + 15) / 16 * 16 : (size_t)zpad(n - 1) + 1;
}
inline size_t zinvw_smem(const FftPlan& pl, int warps, int swz) {
    return (size_t)pl.twn * sizeof(float2) + (size_t)(pl.n + (pl.n & 1)) * sizeof(int) +
           (size_t)warps * zinvw_line_slots(pl.n, swz) * sizeof(float2);
}

// smem: stw[twn] | sof[n] | line[warp][zinvw_line_slots(n, SWZ)]
template <class C, int SWZ>
__global__ void __launch_bounds__(C::T, C::MINB) zinvw_kernel(const ZInvArgs a) {
    extern __shared__ float2 smem[];
    const int n = a.pl.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    float2* stw = smem;
    int* sof = reinterpret_cast<int*>(stw + a.pl.twn);
    float2* sw = reinterpret_cast<float2*>(sof + n + (n & 1)) + (size_t)warp * zinvw_line_slots(n, SWZ);
    fill_stage_twiddles(stw, a.pl);
    for (int m = threadIdx.x; m < n; m += blockDim.x) sof[m] = zslot<SWZ>(slot_of_freq(a.pl, m));
    __syncthreads();
    const int nh = n / 2 + 1, half = n / 2;
    const int64_t rpb = a.zt.rows_per_box;
    const int64_t ppb = (rpb + 1) / 2;                  // row pairs per box
    const int64_t per_buf = ppb * a.batch;
    const int64_t npairs = per_buf * a.nbuf;
    const int64_t cp = a.pitch / 2;
    const int64_t gw = (int64_t)blockIdx.x * nwarp + warp, nw = (int64_t)gridDim.x * nwarp;
    double acc1 = 0.0, acc2 = 0.0, accb = 0.0;
    int64_t cur = -1;
    for (int64_t pi = gw; pi < npairs; pi += nw) {
        const int buf = (int)(pi / per_buf);
        const int64_t t = pi - buf * per_buf;
        const int64_t b = t / ppb;
        const int64_t lrow = 2 * (t - b * ppb);         // first row of the pair inside box b
        const bool two = lrow + 1 < rpb;
        const int64_t row0 = b * rpb + lrow;
        const int64_t key = (int64_t)buf * a.batch + b;
        if (a.stats && key != cur) {
            if (cur >= 0) warp_flush_stats(acc1, acc2, accb, a.stats + 8 * (cur % a.batch) + 4 * (cur / a.batch));
            acc1 = acc2 = accb = 0.0;
            cur = key;
        }
        const float2* in1 = reinterpret_cast<const float2*>(a.buf[buf]) + row0 * cp;
        const float2* in2 = in1 + cp;
        if (a.prefetch && lane < 2 && pi + nw < npairs) {
            // the next pair of this warp: one bulk L2 prefetch per row
            const int64_t tn = pi + nw;
            const int bn = (int)(tn / per_buf);
            const int64_t un = tn - bn * per_buf;
            const int64_t bbn = un / ppb;
            const int64_t rn = bbn * rpb + 2 * (un - bbn * ppb) + lane;
            if (rn < (bbn + 1) * rpb) prefetch_l2_bulk(a.buf[bn] + rn * a.pitch, (uint32_t)(a.pitch * 4));
        }
        // Z_k = X1_k + i X2_k (k <= n/2), Z_{n-k} = X1_k* + i X2_k*; DC and Nyquist real parts.
        // Lanes take consecutive k (the scatter to slot_of_freq(k) then spreads over the banks),
        // U loads per row in flight; a compile-time length takes the U that covers the n/2 + 1
        // modes in two rounds (13 at 1536: 36.6 -> 34.3 ms against 12, whose third round loads
        // the Nyquist mode alone).
        constexpr int U = (C::NF > 0 && (C::NF / 2 + 64) / 64 <= 16) ? (C::NF / 2 + 64) / 64 : 12;
        for (int k0 = lane; k0 < nh; k0 += 32 * U) {
            float2 x1[U], x2[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int k = k0 + 32 * u;
                x1[u] = x2[u] = make_float2(0.f, 0.f);
                if (k < nh) {
                    x1[u] = __ldcs(in1 + k);
                    if (two) x2[u] = __ldcs(in2 + k);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int k = k0 + 32 * u;
                if (k >= nh) break;
                if (k == 0 || k == half) {
                    sw[sof[k]] = make_float2(x1[u].x, x2[u].x);
                } else {
                    sw[sof[k]] = make_float2(x1[u].x - x2[u].y, x1[u].y + x2[u].x);
                    sw[sof[n - k]] = make_float2(x1[u].x + x2[u].y, x2[u].x - x1[u].y);
                }
            }
        }
        __syncwarp();
        // the last stage writes z_e = x1_e + i x2_e, x 1/N, straight from registers
        float* o1 = a.buf[buf] + row0 * a.pitch;
        float* o2 = o1 + a.pitch;
        float p1 = 0.f, p2 = 0.f;
        const float sc = a.scale;
        auto out_fn = [&](int e, float2 z) {
            const float v0 = z.x * sc;
            __stcs(o1 + e, v0);
            p1 += v0;
            p2 = fmaf(v0, v0, p2);
            if (two) {
                const float v1 = z.y * sc;
                __stcs(o2 + e, v1);
                p1 += v1;
                p2 = fmaf(v1, v1, p2);
            }
        };
        warp_ifft_out<C::RMAX, SWZ, decltype(out_fn)&, SWZ == 2 ? C::NF : 0>(sw, stw, a.pl, lane, out_fn);
        if (!(fabsf(p2) < INFINITY)) {
            // a non-finite value in this lane's share: recount it exactly (finite values only)
            // from the outputs this lane wrote (rows of this pair, read back from global)
            p1 = p2 = 0.f;
            float pb = 0.f;
            warp_out_positions(a.pl, lane, [&](int e) {
                const float v[2] = {o1[e], two ? o2[e] : 0.0f};
                for (int r = 0; r < (two ? 2 : 1); ++r) {
                    if (isfinite(v[r])) {
                        p1 += v[r];
                        p2 = fmaf(v[r], v[r], p2);
                    } else {
                        pb += 1.f;
                    }
                }
            });
            accb += pb;
        }
        acc1 += p1;
        acc2 += p2;
        __syncwarp();
    }
    if (a.stats && cur >= 0) warp_flush_stats(acc1, acc2, accb, a.stats + 8 * (cur % a.batch) + 4 * (cur / a.batch));
}

// ------------------------------------------------------------------ launch helpers
int sm_count();

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

// r2c along z of the caller's noise, one warp per row pair (variants with W = 0): the two real
// rows packed as z = x1 + i x2 in the warp's private (swizzled) line, forward transform, the two
// half spectra split out of Z_k and Z*_{n-k} and stored row by row.  Same shared-memory layout
// as zinvw_kernel: stw[twn] | sof[n] | line[warp][zinvw_line_slots(n, SWZ)].
template <class C, int SWZ>
__global__ void __launch_bounds__(C::T, C::MINB) zfwdw_kernel(const ZFwdArgs a) {
    extern __shared__ float2 smem[];
    const int n = a.pl.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    float2* stw = smem;
    int* sof = reinterpret_cast<int*>(stw + a.pl.twn);
    float2* sw = reinterpret_cast<float2*>(sof + n + (n & 1)) + (size_t)warp * zinvw_line_slots(n, SWZ);
    fill_stage_twiddles(stw, a.pl);
    for (int m = threadIdx.x; m < n; m += blockDim.x) sof[m] = zslot<SWZ>(slot_of_freq(a.pl, m));
    __syncthreads();
    const int nh = n / 2 + 1;
    const int64_t rpb = a.zt.rows_per_box;
    const int64_t ppb = (rpb + 1) / 2;                  // row pairs per box
    const int64_t npairs = ppb * a.batch;
    const int64_t cp = a.pitch / 2;
    float2* out2 = reinterpret_cast<float2*>(a.out);
    const bool pf = a.prefetch && (n & 3) == 0 && ((uintptr_t)a.noise & 15) == 0;
    const int64_t gw = (int64_t)blockIdx.x * nwarp + warp, nw = (int64_t)gridDim.x * nwarp;
    for (int64_t pi = gw; pi < npairs; pi += nw) {
        const int64_t b = pi / ppb;
        const int64_t lrow = 2 * (pi - b * ppb);        // first row of the pair inside box b
        const bool two = lrow + 1 < rpb;
        const int64_t row0 = b * rpb + lrow;
        const float* in1 = a.noise + row0 * n;
        const float* in2 = in1 + n;
        if (pf && lane < 2 && pi + nw < npairs) {
            // the next pair of this warp: one bulk L2 prefetch per row
            const int64_t tn = pi + nw;
            const int64_t bn = tn / ppb;
            const int64_t rn = bn * rpb + 2 * (tn - bn * ppb) + lane;
            if (rn < (bn + 1) * rpb) prefetch_l2_bulk(a.noise + rn * n, (uint32_t)(n * 4));
        }
        constexpr int U = 12;
        for (int e0 = lane; e0 < n; e0 += 32 * U) {
            float x1[U], x2[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = e0 + 32 * u;
                x1[u] = x2[u] = 0.f;
                if (e < n) {
                    x1[u] = __ldcs(in1 + e);
                    if (two) x2[u] = __ldcs(in2 + e);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = e0 + 32 * u;
                if (e < n) sw[zslot<SWZ>(e)] = make_float2(x1[u], x2[u]);
            }
        }
        __syncwarp();
        warp_fft_fwd<C::RMAX, SWZ, SWZ == 2 ? C::NF : 0>(sw, stw, a.pl, lane);
        // X1_k = (Z_k + Z*_{n-k})/2, X2_k = (Z_k - Z*_{n-k})/(2i)
        float2* o1 = out2 + row0 * cp;
        float2* o2 = o1 + cp;
        for (int k = lane; k < nh; k += 32) {
            const float2 zk = sw[sof[k]];
            const float2 zm = sw[sof[k == 0 ? 0 : n - k]];
            __stcs(o1 + k, make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y)));
            if (two) __stcs(o2 + k, make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x)));
        }
        __syncwarp();
    }
}

template <class C>
static size_t zpass_smem(int n) {
    return (size_t)n * (C::W + 1) * sizeof(float2) + (size_t)n * sizeof(float2) + (size_t)(n + 1) * sizeof(int) +
           3 * (C::T / 32) * sizeof(double) + 8;
}

// One warp per row pair (variants with W = 0): as many warps per block as fit in shared
// memory, up to C::T / 32; the plan and swizzle rule of zinvw_kernel.
template <class C>
static int launch_zfwdw(ZFwdArgs a, int64_t rows_per_box, cudaStream_t st) {
    a.zt.rows_per_box = rows_per_box;
    a.zt.tiles_per_box = 0;
    const int n = a.pl.n;
    const int swz = C::NF > 0 ? 2 : ((n & (n - 1)) != 0 || n < 2048) ? 1 : 0;
    if (swz && !make_plan(n, &a.pl, C::RMAX, true)) return fail(SMK_ENOTSUPP, "zfwdw_kernel: no plan for %d", n);
    if constexpr (C::NF > 0) {
        if (!same_plan(a.pl, FixedPlan<C::NF, 16, true>::P))
            return fail(SMK_EINVAL, "zfwdw_kernel: length %d is not the variant's fixed length", n);
    }
    int dev = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    int warps = C::T / 32;
    while (warps > 1 && zinvw_smem(a.pl, warps, swz) > (size_t)smem_max) --warps;
    const size_t smem = zinvw_smem(a.pl, warps, swz);
    if (smem > (size_t)smem_max) return fail(SMK_ENOTSUPP, "zfwdw_kernel: line of %d does not fit", n);
    void (*kern)(const ZFwdArgs) = nullptr;
    if constexpr (C::NF > 0) kern = zfwdw_kernel<C, 2>;
    else kern = swz ? zfwdw_kernel<C, 1> : zfwdw_kernel<C, 0>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute(zfwdw)");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * warps, smem) != cudaSuccess)
        return check_launch("cudaOccupancyMaxActiveBlocksPerMultiprocessor(zfwdw)");
    if (per_sm < 1) return fail(SMK_ENOTSUPP, "zfwdw_kernel does not fit on an SM (smem %zu B)", smem);
    const int64_t npairs = (rows_per_box + 1) / 2 * a.batch;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(npairs, warps), (int64_t)per_sm * sm_count()));
    kern<<<grid, 32 * warps, smem, st>>>(a);
    return check_launch("zfwdw_kernel");
}

template <class C>
static int launch_zfwd(ZFwdArgs a, int64_t rows_per_box, cudaStream_t st) {
    if (!plan_fits(a.pl, C::RMAX)) return fail(SMK_EINVAL, "%s: plan radix above the variant's", "zfwd_kernel");
    if constexpr (C::W == 0) {
        return launch_zfwdw<C>(a, rows_per_box, st);
    } else {
        if (!fixed_plan_ok<C>(a.pl)) return fail(SMK_EINVAL, "%s: length %d is not the variant's fixed length", "zfwd_kernel", a.pl.n);
        a.zt.init(rows_per_box, C::W);
        const size_t smem = zpass_smem<C>(a.pl.n);
        const int64_t ntiles = a.zt.tiles_per_box * a.batch;
        int grid = 0, rc;
        if ((rc = persistent_grid(zfwd_kernel<C>, C::T, smem, ntiles, &grid))) return rc;
        zfwd_kernel<C><<<grid, C::T, smem, st>>>(a);
        return check_launch("zfwd_kernel");
    }
}

// One warp per row pair (variants with W = 0): as many warps per block as fit in shared
// memory, up to C::T / 32.
template <class C>
static int launch_zinvw(ZInvArgs a, int64_t rows_per_box, cudaStream_t st) {
    if (!plan_fits(a.pl, C::RMAX)) return fail(SMK_EINVAL, "%s: plan radix above the variant's", "zinvw_kernel");
    if (!fixed_plan_ok<C>(a.pl)) return fail(SMK_EINVAL, "%s: length %d is not the variant's fixed length", "zinvw_kernel", a.pl.n);
    a.zt.rows_per_box = rows_per_box;
    a.zt.tiles_per_box = 0;
    // layout: a compile-time plan on one pad per 16 slots; else the XOR swizzle with the odd radix
    // mid-plan, except power-of-two lengths >= 2048
    const int n = a.pl.n;
    const int swz = C::NF > 0 ? 2 : ((n & (n - 1)) != 0 || n < 2048) ? 1 : 0;
    if (swz && !make_plan(n, &a.pl, C::RMAX, true)) return fail(SMK_ENOTSUPP, "zinvw_kernel: no plan for %d", n);
    if constexpr (C::NF > 0) {
        if (!same_plan(a.pl, FixedPlan<C::NF, 16, true>::P))
            return fail(SMK_EINVAL, "zinvw_kernel: length %d is not the variant's fixed length", n);
    }
    int dev = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    int warps = C::T / 32;
    while (warps > 1 && zinvw_smem(a.pl, warps, swz) > (size_t)smem_max) --warps;
    const size_t smem = zinvw_smem(a.pl, warps, swz);
    if (smem > (size_t)smem_max) return fail(SMK_ENOTSUPP, "zinvw_kernel: line of %d does not fit", n);
    void (*kern)(const ZInvArgs) = nullptr;
    if constexpr (C::NF > 0) kern = zinvw_kernel<C, 2>;
    else kern = swz ? zinvw_kernel<C, 1> : zinvw_kernel<C, 0>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute(zinvw)");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * warps, smem) != cudaSuccess)
        return check_launch("cudaOccupancyMaxActiveBlocksPerMultiprocessor(zinvw)");
    if (per_sm < 1) return fail(SMK_ENOTSUPP, "zinvw_kernel does not fit on an SM (smem %zu B)", smem);
    const int64_t npairs = (rows_per_box + 1) / 2 * a.batch * a.nbuf;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(npairs, warps), (int64_t)per_sm * sm_count()));
    kern<<<grid, 32 * warps, smem, st>>>(a);
    return check_launch("zinvw_kernel");
}

template <class C>
static int launch_zinv(ZInvArgs a, int64_t rows_per_box, cudaStream_t st) {
    return launch_zinvw<C>(a, rows_per_box, st);
}

template <class C>
static int launch_line(const LineArgs& a, bool inv, cudaStream_t st) {
    if (!plan_fits(a.pl, C::RMAX)) return fail(SMK_EINVAL, "%s: plan radix above the variant's", "line_kernel");
    if (!fixed_plan_ok<C>(a.pl)) return fail(SMK_EINVAL, "%s: length %d is not the variant's fixed length", "line_kernel", a.pl.n);
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2);
    const int64_t ntiles = a.n_outer * ceil_div(a.ncol, C::W) * a.nbuf;
    int grid = 0, rc;
    // one direction per instantiation (the two are compiled in separate translation units)
    if constexpr (C::DIR >= 0) {
        if (inv != (C::DIR == 1)) return fail(SMK_EINVAL, "line: direction of another unit");
    }
    if (inv) {
        if constexpr (C::DIR != 0) {
            if ((rc = persistent_grid(line_kernel<C, true>, C::T, smem, ntiles, &grid))) return rc;
            line_kernel<C, true><<<grid, C::T, smem, st>>>(a);
        }
    } else {
        if constexpr (C::DIR != 1) {
            if ((rc = persistent_grid(line_kernel<C, false>, C::T, smem, ntiles, &grid))) return rc;
            line_kernel<C, false><<<grid, C::T, smem, st>>>(a);
        }
    }
    return check_launch("line_kernel");
}

template <class C>
static int launch_xpass(const XArgs& a, cudaStream_t st) {
    if (!plan_fits(a.pl, C::RMAX)) return fail(SMK_EINVAL, "%s: plan radix above the variant's", "xpass_kernel");
    if (!fixed_plan_ok<C>(a.pl)) return fail(SMK_EINVAL, "%s: length %d is not the variant's fixed length", "xpass_kernel", a.pl.n);
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2) + (size_t)a.pl.n * 8 + (C::W + 1) * 4;
    const int64_t ntiles = (int64_t)a.batch * a.ny * ceil_div(a.nzh, C::W);
    int grid = 0, rc;
    if ((rc = persistent_grid(xpass_kernel<C>, C::T, smem, ntiles, &grid))) return rc;
    xpass_kernel<C><<<grid, C::T, smem, st>>>(a);
    return check_launch("xpass_kernel");
}

template <class C>
static int launch_xpi(const XArgs& a, cudaStream_t st) {
    if (!plan_fits(a.pl, C::RMAX)) return fail(SMK_EINVAL, "%s: plan radix above the variant's", "xpi_kernel");
    if (!fixed_plan_ok<C>(a.pl)) return fail(SMK_EINVAL, "%s: length %d is not the variant's fixed length", "xpi_kernel", a.pl.n);
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2) + (size_t)a.pl.n * 8 + (C::W + 1) * 4;
    const int64_t ntiles = (int64_t)a.batch * a.ncb * a.ny;
    int grid = 0, rc;
    if (a.I[1]) {
        if ((rc = persistent_grid(xpi_kernel<C, true>, C::T, smem, ntiles, &grid))) return rc;
        xpi_kernel<C, true><<<grid, C::T, smem, st>>>(a);
    } else {
        if ((rc = persistent_grid(xpi_kernel<C, false>, C::T, smem, ntiles, &grid))) return rc;
        xpi_kernel<C, false><<<grid, C::T, smem, st>>>(a);
    }
    return check_launch("xpi_kernel");
}

template <class C>
static int launch_xgi(const XGenArgs& a, cudaStream_t st) {
    if (!plan_fits(a.pl, C::RMAX)) return fail(SMK_EINVAL, "%s: plan radix above the variant's", "xgi_kernel");
    if (!fixed_plan_ok<C>(a.pl)) return fail(SMK_EINVAL, "%s: length %d is not the variant's fixed length", "xgi_kernel", a.pl.n);
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2) + (size_t)a.pl.n * 8 +
                        (size_t)a.nzh * 4 + 16;
    const int64_t ntiles = (int64_t)a.batch * a.ncb * a.ny;
    int grid = 0, rc;
    if ((rc = persistent_grid(xgi_kernel<C>, C::T, smem, ntiles, &grid))) return rc;
    xgi_kernel<C><<<grid, C::T, smem, st>>>(a);
    return check_launch("xgi_kernel");
}

template <class C>
static int launch_xgen(const XGenArgs& a, cudaStream_t st) {
    if (!plan_fits(a.pl, C::RMAX)) return fail(SMK_EINVAL, "%s: plan radix above the variant's", "xgen_kernel");
    if (!fixed_plan_ok<C>(a.pl)) return fail(SMK_EINVAL, "%s: length %d is not the variant's fixed length", "xgen_kernel", a.pl.n);
    const size_t smem = (size_t)(a.pl.n * C::W + a.pl.n) * sizeof(float2) + (size_t)a.pl.n * 8 +
                        (size_t)a.nzh * 4 + 16;
    const bool one = a.fields != XGEN_BOTH;
    const int64_t ntiles = (int64_t)a.batch * a.ny * ceil_div(a.nzh, one ? C::W : C::W / 2);
    int grid = 0, rc;
    if (one) {
        if ((rc = persistent_grid(xgen_kernel<C, true>, C::T, smem, ntiles, &grid))) return rc;
        xgen_kernel<C, true><<<grid, C::T, smem, st>>>(a);
    } else {
        if ((rc = persistent_grid(xgen_kernel<C, false>, C::T, smem, ntiles, &grid))) return rc;
        xgen_kernel<C, false><<<grid, C::T, smem, st>>>(a);
    }
    return check_launch("xgen_kernel");
}

// ------------------------------------------------------------------ tile variants
struct TileVariant {
    int w, t, nmax;  // columns (line pairs for z passes, lines for xgen) per tile, threads, max length
                     // (nmax < 0: the length -nmax only, with its FFT plan fixed at compile time)
    int rmax, minb;  // largest FFT radix, requested resident blocks per SM
};
// TileCfg's fixed length of a table entry
#define SMK_NFIX(N) ((N) < 0 ? -(N) : 0)
inline bool variant_fits(const TileVariant& v, int n) { return v.nmax < 0 ? n == -v.nmax : v.nmax >= n; }
// r2c along z of host noise (zfwd): W = row pairs per tile; W = 0: one warp per row pair (built-in)
#define SMK_Z_VARIANTS(X) X(16, 256, 512, 32, 1) X(16, 512, 1024, 16, 1) X(8, 512, 2560, 16, 1) X(4, 512, 2560, 16, 1) \
    X(2, 128, 2560, 16, 4) X(4, 512, 4096, 16, 1) X(0, 512, 2560, 16, 1) X(0, 512, 4096, 16, 1) \
    X(0, 512, -1536, 16, 1) X(0, 512, -1024, 16, 1)
// z inverse: one warp per row pair (W = 0; as many warps per block as fit, up to T / 32)
#define SMK_ZINV_VARIANTS(X) X(0, 512, 2560, 16, 1) X(0, 512, 1024, 16, 1) X(0, 256, 1024, 16, 2) \
    X(0, 512, 4096, 16, 1) X(0, 256, 2560, 32, 1) X(0, 512, -1536, 16, 1) X(0, 512, -1024, 16, 1)
// y pass (line): W = columns per tile
#define SMK_LINE_VARIANTS(X) X(16, 256, 512, 32, 1) X(16, 512, 1024, 16, 1) X(8, 512, 2560, 16, 1) X(8, 1024, 2560, 8, 1) \
    X(4, 512, 4096, 16, 1) X(8, 256, 2560, 16, 1) X(8, 512, -2560, 16, 1) X(8, 256, -1024, 16, 2) \
    X(16, 256, -128, 16, 2)
// x pass of host noise: W = columns per tile
#define SMK_X_VARIANTS(X) X(16, 256, 512, 32, 1) X(16, 512, 1024, 16, 1) X(8, 512, 2560, 16, 1) X(4, 512, 4096, 16, 1) \
    X(8, 512, -2560, 16, 1) X(16, 512, -1024, 16, 1)
// x pass of GPU noise: W = lines per tile (one field per launch: W columns; both fields: W/2 + W/2).
// At 1024 the x and y tiles of 8 lines fit two blocks per SM (measured 6-8 % faster than one block
// of 16 lines); at 2560 two 8-line tiles do not fit the shared memory.
#define SMK_XGEN_VARIANTS(X) X(16, 256, 512, 32, 1) X(16, 512, 1024, 16, 1) X(8, 512, 2560, 16, 1) \
    X(8, 1024, 2560, 8, 1) X(4, 512, 4096, 16, 1) X(8, 512, -2560, 16, 1) X(8, 256, -1024, 16, 2) \
    X(16, 256, -128, 16, 2)

enum { PASS_ZFWD = 0, PASS_LINE = 1, PASS_XPASS = 2, PASS_XGEN = 3, PASS_ZINV = 4, NPASS = 5 };

int variant_count(int pass);
const TileVariant* variant_table(int pass);
// Variant used for a line of length n (tuned choice if valid, else the first that fits).
int variant_for(int pass, int n);

int run_zfwd(int v, const ZFwdArgs& a, int64_t rows_per_box, cudaStream_t st);
int run_zinv(int v, const ZInvArgs& a, int64_t rows_per_box, cudaStream_t st);
int run_line(int v, const LineArgs& a, bool inv, cudaStream_t st);
int run_line_inv(int v, const LineArgs& a, cudaStream_t st);
int run_line_fwd(int v, const LineArgs& a, cudaStream_t st);
int run_xpass(int v, const XArgs& a, cudaStream_t st);
int run_xgen(int v, const XGenArgs& a, cudaStream_t st);
int run_xgi(int v, const XGenArgs& a, cudaStream_t st);
int run_xpi(int v, const XArgs& a, cudaStream_t st);

}  // namespace smk
