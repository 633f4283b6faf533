// Fused skewer stage on GB300: trilinear read of the delta / eta_par boxes along each
// skewer + missing small-scale 1D power (one complex FFT carries the Gaussian fields of two
// skewers) + FGPA flux, in one persistent launch.
//
// Work items are pairs of skewers with the same small-scale FFT length (host schedule,
// longest first); blocks take items from an atomic counter.  Per item:
//   1. delta_s of both skewers in shared memory (SMK_SS_HOST: noise -> FFT -> x S_k -> IFFT;
//      SMK_SS_PHILOX: Gaussian modes drawn directly in Fourier space -> IFFT),
//   2. every pixel: position -> 8-corner trilinear read of delta (and eta), redshift,
//      a(z), b, c, G(z), F = exp(-a exp(b G (delta_l + delta_s + c eta))).
#include <algorithm>
#include <mutex>
#include <vector>

#include "smk_fft.cuh"

namespace smk {

std::atomic<int> g_skewer_blocks{0};

constexpr int SK_T = 256;
constexpr int SK_NCLASS = 5;  // small-scale FFT lengths 256 << j

struct SkArgs {
    const float* start;
    const float* dir;
    const double* start64;    // optional FP64 start / direction (override start / dir)
    const double* dir64;
    const int32_t* npix;
    const int64_t* offset;
    double dpix;
    const int32_t* order;
    int64_t n_items;
    int interp;
    const float* eta6[6];     // SMK_INTERP_GAUSS343: eta_xx, yy, zz, xy, xz, yz boxes (or null)
    double obs[3];            // SMK_INTERP_GAUSS343: observer, box-corner frame (Mpc/h)
    const float* pix_delta;
    const float* pix_eta;
    const float* pix_z;
    const float* delta;
    const float* eta;
    int nx, ny, nz;
    int64_t pitch;
    double dcell;
    int ss_mode, ss_nz;
    const float* ss_scale;
    const float* ss_noise;
    const int64_t* ss_noise_offset;
    uint64_t seed;
    const int32_t* forest;    // [n][2] forest pixel range [f0, f1) of each skewer, or null (all)
    int ss_nztab;             // 0: one table set; > 0: one set per redshift ss_ztab[j]
    const float* ss_ztab;     // [ss_nztab] ascending redshifts of the table sets
    const float* ss_zsigma;   // [ss_nztab] sigma_s at ss_ztab, or null: no sigma_s(z)/sigma_s(zeff)
    FftPlan plans[SK_NCLASS];
    int abc_mode;
    float a, b, c, a_zref1, a_power;
    const float* abc_tab;
    int n_tab;
    float z_tab0, dz_tab;
    float z_lo, z_hi;
    int growth_mode;
    float growth24;
    float* flux;
    float* delta_out;
    float* eta_out;
    float* z_out;
    unsigned long long* counter;
    int ss_nmax;              // longest small-scale FFT of the launch (shared-memory sizing)
};

__device__ __forceinline__ int ss_class(int nzz) {
    int j = 0;
    while ((256 << j) < nzz) ++j;
    return j;
}

__device__ __forceinline__ int ss_table_offset(int j) {
    int off = 0;
    for (int i = 0; i < j; ++i) off += (256 << i) / 2 + 1;
    return off;
}

__device__ __forceinline__ int wrap(int64_t c, int n) {
    int64_t r = c % n;
    return (int)(r < 0 ? r + n : r);
}

// The same for a 32-bit cell index (a wrapped start cell plus the cells a skewer advances, or a
// neighbour offset): one 32-bit remainder instead of the emulated 64-bit one.
__device__ __forceinline__ int wrap32(int c, int n) {
    const int r = c % n;
    return r < 0 ? r + n : r;
}

// c mod n for c in [-n, 2n): one compare each way (a skewer whose advance stays within the box,
// SkewerGeo::near).
__device__ __forceinline__ int wrap_near(int c, int n) {
    if (c < 0) c += n;
    else if (c >= n) c -= n;
    return c;
}

// Pixel positions in cells along each axis as 32.32 fixed point: q_i = f0 + i * step exactly
// in int64, cell = i0 + (q_i >> 32), fraction = low 32 bits (error < 2e-7 cells at 1e3 pixels,
// where float32 i*step would lose ~1e-5 cells).
struct SkewerGeo {
    int i0[3];        // cell index of the first pixel's lower corner, wrapped
    long long f0[3];  // fraction of the first pixel above i0, 2^-32 units
    long long step[3];// pixel step, 2^-32 cell units
    long long i0u[3]; // i0 before wrapping (unwrapped line of sight, for the eta projection)
    int near;         // every axis: n >= 16 and the skewer advances fewer than n - 8 cells
                      // either way, so cell indices (and +-4 neighbours) lie in [-n, 2n)
};

// Floats of one small-scale table set: sqrt(P1Dmiss/pix) for nz = 256 << j, j = 0..4.
constexpr int SK_SS_SET = 129 + 257 + 513 + 1025 + 2049;

// Redshift of pixel i of a skewer read from the boxes: z_lo..z_hi mapped linearly on the
// wrapped x coordinate x/dcell (the trilinear read's rule).
__device__ __forceinline__ float pixel_z_box(const SkArgs& a, const SkewerGeo& g, int i) {
    const long long q = g.f0[0] + (long long)i * g.step[0];
    const float fr = (float)(unsigned)(q & 0xffffffffLL) * 2.3283064365386963e-10f;
    const int c = g.i0[0] + (int)(q >> 32);
    float xc = (float)(g.near ? wrap_near(c, a.nx) : wrap32(c, a.nx)) + fr + 0.5f;
    if (xc >= (float)a.nx) xc -= (float)a.nx;
    return a.z_lo + (a.z_hi - a.z_lo) * (xc / (float)a.nx);
}

// sigma_s(z) by linear interpolation on (ss_ztab, ss_zsigma), clamped to the table's ends.
__device__ __forceinline__ float zsigma_at(const SkArgs& a, float z) {
    const int n = a.ss_nztab;
    if (n == 1 || z <= a.ss_ztab[0]) return a.ss_zsigma[0];
    if (z >= a.ss_ztab[n - 1]) return a.ss_zsigma[n - 1];
    int j = 0;
    while (j < n - 2 && z > a.ss_ztab[j + 1]) ++j;
    const float z0 = a.ss_ztab[j], z1 = a.ss_ztab[j + 1];
    const float t = (z - z0) / (z1 - z0);
    return fmaf(t, a.ss_zsigma[j + 1] - a.ss_zsigma[j], a.ss_zsigma[j]);
}

// Gaussian-weighted read of the (2*GR+1)^3 cells around the pixel, GR = dmax (ReadSpec of
// bin/make_spectra.py:39-68, 104-129): for the cell holding p (index floor(p/dcell)), weights
// exp(-|r_cell - p|^2 / (2 dcell^2)) = prod_d exp(-(c_d + 0.5 - f_d)^2 / 2), one 1D factor per
// axis; value = sum(w rho) / sum(w), with periodic wrap.
// GR > 0: the Gaussian (2 GR + 1)^3 read (more registers, two blocks per SM); GR = 0: trilinear
// or per-pixel inputs (four blocks per SM).  smem holds the small-scale FFT of the longest line
// the launch needs (a.ss_nmax points: line, twiddles, slots).
template <int GR>
__global__ void __launch_bounds__(SK_T, GR ? 2 : 4) skewer_kernel(const SkArgs a) {
    constexpr bool GAUSS = GR > 0;
    extern __shared__ float2 smem[];
    float2* s = smem;                                          // ss_nmax
    float2* tw = smem + a.ss_nmax;                             // ss_nmax
    int* sof = reinterpret_cast<int*>(smem + 2 * a.ss_nmax);   // slot of each frequency
    __shared__ long long item_sh;
    __shared__ SkewerGeo geo[2];
    __shared__ int sk_id[2], sk_np[2];
    __shared__ int64_t sk_off[2];
    __shared__ int sk_f0[2], sk_f1[2], sk_set[2];
    __shared__ float sk_sig_eff[2];
    __shared__ double zsum_sh[2][SK_T / 32];
    int cur_nz = 0;
    const int dims[3] = {a.nx, a.ny, a.nz};
    for (;;) {
        if (threadIdx.x == 0) item_sh = (long long)atomicAdd(a.counter, 1ULL);
        __syncthreads();
        const long long item = item_sh;
        if (item >= a.n_items) break;
        if (threadIdx.x < 2) {
            const int t = threadIdx.x;
            const int sid = a.order[2 * item + t];
            sk_id[t] = sid;
            sk_np[t] = sid >= 0 ? a.npix[sid] : 0;
            sk_off[t] = sid >= 0 ? a.offset[sid] : 0;
            if (sid >= 0 && a.interp != SMK_INTERP_PIXELS) {
                for (int d = 0; d < 3; ++d) {
                    const double st0 = a.start64 ? a.start64[3 * sid + d] : (double)a.start[3 * sid + d];
                    const double dr = a.dir64 ? a.dir64[3 * sid + d] : (double)a.dir[3 * sid + d];
                    const double u0 = st0 / a.dcell - 0.5;
                    const double fl = floor(u0);
                    geo[t].i0[d] = wrap((int64_t)fl, dims[d]);
                    geo[t].i0u[d] = (long long)fl;
                    geo[t].f0[d] = __double2ll_rn((u0 - fl) * 4294967296.0);
                    geo[t].step[d] = __double2ll_rn(a.dpix * dr / a.dcell * 4294967296.0);
                }
                int near = 1;
                for (int d = 0; d < 3; ++d) {
                    const long long qa = geo[t].f0[d], qb = qa + (long long)max(sk_np[t] - 1, 0) * geo[t].step[d];
                    const long long lo = min(qa, qb) >> 32, hi = (max(qa, qb) >> 32) + 1;
                    near &= dims[d] >= 16 && lo >= -(long long)(dims[d] - 8) && hi <= (long long)(dims[d] - 8);
                }
                geo[t].near = near;
            }
            // forest pixels (bin/merge_spectra.py:305-306): no range given means all pixels
            int f0 = 0, f1 = sk_np[t];
            if (sid >= 0 && a.forest) {
                f0 = max(0, a.forest[2 * sid]);
                f1 = min(sk_np[t], a.forest[2 * sid + 1]);
            }
            sk_f0[t] = f0;
            sk_f1[t] = max(f0, f1);
            sk_set[t] = 0;
            sk_sig_eff[t] = 1.f;
        }
        __syncthreads();
        const int np0 = sk_np[0], np1 = sk_np[1];
        // redshift tables: zeff = mean z over the forest pixels (bin/merge_spectra.py:315), the
        // table set of the nearest redshift (util.InterpP1Dmissing, util.py:467-474) and
        // sigma_s(zeff) for the sigma_s(z)/sigma_s(zeff) rescale (:324-325)
        if (a.ss_mode != SMK_SS_NONE && a.ss_nztab > 0) {
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                double zs = 0.0;
                for (int i = sk_f0[t] + threadIdx.x; i < sk_f1[t]; i += SK_T)
                    zs += a.interp == SMK_INTERP_PIXELS ? (double)__ldg(a.pix_z + sk_off[t] + i)
                                                        : (double)pixel_z_box(a, geo[t], i);
#pragma unroll
                for (int m = 16; m; m >>= 1) zs += __shfl_xor_sync(0xffffffffu, zs, m);
                if ((threadIdx.x & 31) == 0) zsum_sh[t][threadIdx.x >> 5] = zs;
            }
            __syncthreads();
            if (threadIdx.x < 2) {
                const int t = threadIdx.x;
                const int cnt = sk_f1[t] - sk_f0[t];
                if (cnt > 0) {
                    double zs = 0.0;
                    for (int w = 0; w < SK_T / 32; ++w) zs += zsum_sh[t][w];
                    const float zeff = (float)(zs / cnt);
                    int best = 0;
                    float bd = fabsf(a.ss_ztab[0] - zeff);
                    for (int j = 1; j < a.ss_nztab; ++j) {
                        const float d = fabsf(a.ss_ztab[j] - zeff);
                        if (d < bd) { bd = d; best = j; }
                    }
                    sk_set[t] = best;
                    if (a.ss_zsigma) sk_sig_eff[t] = zsigma_at(a, zeff);
                }
            }
            __syncthreads();
        }
        // skewers without forest pixels get no small-scale field (bin/merge_spectra.py:327-330)
        const bool live0 = sk_id[0] >= 0 && sk_f1[0] > sk_f0[0];
        const bool live1 = sk_id[1] >= 0 && sk_f1[1] > sk_f0[1];
        float inv_nz = 0.f;
        // a pair whose small-scale field does not fit the launch's FFT length (a table built
        // without smk_skewer_schedule's checks) gets NaN flux instead of a read past the line
        bool too_long = false;
        if (a.ss_mode != SMK_SS_NONE) {
            const int npmax = max(np0, np1);
            int nzz = a.ss_nz;
            if (nzz <= 0) {
                nzz = 256;
                while (nzz < npmax + 50 && nzz < a.ss_nmax) nzz *= 2;
                too_long = nzz < npmax + 50;
            } else {
                too_long = npmax > nzz;
            }
        }
        if (a.ss_mode != SMK_SS_NONE && !too_long) {
            int nzz = a.ss_nz;
            if (nzz <= 0) {
                nzz = 256;
                while (nzz < max(np0, np1) + 50) nzz *= 2;
            }
            const int cls = ss_class(nzz);
            const FftPlan& pl = a.plans[cls];
            if (nzz != cur_nz) {
                fill_stage_twiddles(tw, pl);
                for (int k = threadIdx.x; k < nzz; k += SK_T) sof[k] = slot_of_freq(pl, k);
                cur_nz = nzz;
                __syncthreads();
            }
            const float* S = a.ss_scale + (int64_t)sk_set[0] * SK_SS_SET + ss_table_offset(cls);
            const float* S1 = a.ss_scale + (int64_t)sk_set[1] * SK_SS_SET + ss_table_offset(cls);
            const bool one_set = S1 == S;
            const int half = nzz / 2;
            if (a.ss_mode == SMK_SS_HOST) {
                const float* n0 = live0 ? a.ss_noise + a.ss_noise_offset[sk_id[0]] : nullptr;
                const float* n1 = live1 ? a.ss_noise + a.ss_noise_offset[sk_id[1]] : nullptr;
                for (int e = threadIdx.x; e < nzz; e += SK_T)
                    s[e] = make_float2(n0 ? __ldg(n0 + e) : 0.f, n1 ? __ldg(n1 + e) : 0.f);
                __syncthreads();
                fft_tile<false, 1, 1, SK_T, 16>(s, tw, pl);
                if (one_set) {
                    for (int e = threadIdx.x; e < nzz; e += SK_T) {
                        const int f = freq_of_slot(pl, e);
                        s[e] = cscale(s[e], __ldg(S + (f <= half ? f : nzz - f)));
                    }
                } else {
                    // Y_k = A_k + i B_k holds both spectra; with Z_k = S0_k A_k + i S1_k B_k:
                    // Z_k = P Y_k + M conj(Y_{nz-k}), P = (S0 + S1)/2, M = (S0 - S1)/2
                    for (int k = threadIdx.x; k <= half; k += SK_T) {
                        const int e = sof[k], em = sof[k == 0 ? 0 : nzz - k];
                        const float s0 = __ldg(S + k), s1 = __ldg(S1 + k);
                        const float P = 0.5f * (s0 + s1), M = 0.5f * (s0 - s1);
                        const float2 y = s[e], ym = s[em];
                        const float2 z = make_float2(P * y.x + M * ym.x, P * y.y - M * ym.y);
                        const float2 zm = make_float2(P * ym.x + M * y.x, P * ym.y - M * y.y);
                        s[e] = z;   // slots e and em belong to this thread alone
                        if (em != e) s[em] = zm;
                    }
                }
                __syncthreads();
            } else {
                // Fourier modes of two white-noise fields: X_k = sqrt(nz/2)(g_re + i g_im), X_0 and
                // X_{nz/2} real with variance nz; Z_k = S_k (X0_k + i X1_k), Z_{nz-k} = S_k (X0_k* + i X1_k*)
                const float rh = sqrtf(0.5f * (float)nzz), r1 = sqrtf((float)nzz);
                for (int j = threadIdx.x; 2 * j <= half; j += SK_T) {
                    float g[2][4];
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        if (t == 0 ? live0 : live1)
                            philox_gauss4(a.seed, (uint64_t)sk_id[t], (uint32_t)j, STREAM_SKEWER, g[t]);
                        else
                            g[t][0] = g[t][1] = g[t][2] = g[t][3] = 0.f;
                    }
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int k = 2 * j + h;
                        if (k > half) break;
                        const float sk = __ldg(S + k);
                        if (one_set) {
                            if (k == 0 || k == half) {
                                s[sof[k]] = make_float2(sk * r1 * g[0][2 * h], sk * r1 * g[1][2 * h]);
                            } else {
                                const float ar = rh * g[0][2 * h], ai = rh * g[0][2 * h + 1];
                                const float br = rh * g[1][2 * h], bi = rh * g[1][2 * h + 1];
                                s[sof[k]] = make_float2(sk * (ar - bi), sk * (ai + br));
                                s[sof[nzz - k]] = make_float2(sk * (ar + bi), sk * (br - ai));
                            }
                        } else {
                            // each skewer's modes scaled by its own table set
                            const float sk1 = __ldg(S1 + k);
                            if (k == 0 || k == half) {
                                s[sof[k]] = make_float2(sk * r1 * g[0][2 * h], sk1 * r1 * g[1][2 * h]);
                            } else {
                                const float ar = sk * rh * g[0][2 * h], ai = sk * rh * g[0][2 * h + 1];
                                const float br = sk1 * rh * g[1][2 * h], bi = sk1 * rh * g[1][2 * h + 1];
                                s[sof[k]] = make_float2(ar - bi, ai + br);
                                s[sof[nzz - k]] = make_float2(ar + bi, br - ai);
                            }
                        }
                    }
                }
                __syncthreads();
            }
            if (nzz == 2048)   // the plan of the most common length as compile-time constants
                fft_tile<true, 1, 1, SK_T, 16, 2048>(s, tw, pl);
            else
                fft_tile<true, 1, 1, SK_T, 16>(s, tw, pl);
            inv_nz = 1.0f / (float)nzz;
        }
        // pixels of both skewers
        const int64_t ntot = (int64_t)np0 + np1;
        const float nxf = (float)a.nx;
        for (int64_t idx = threadIdx.x; idx < ntot; idx += SK_T) {
            const int t = idx < np0 ? 0 : 1;
            const int i = (int)(idx - (t ? np0 : 0));
            const int64_t o = sk_off[t] + i;
            float dl, et, z;
            if (a.interp == SMK_INTERP_PIXELS) {
                dl = __ldg(a.pix_delta + o);
                et = a.pix_eta ? __ldg(a.pix_eta + o) : 0.f;
                z = __ldg(a.pix_z + o);
            } else if (GAUSS) {
                const SkewerGeo& g = geo[t];
                int ci[3];
                float ew[3][2 * GR + 1 + !GAUSS];
                double rpos[3];
                float fux = 0.f;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    // p/dcell = i0 + q 2^-32 + 0.5: shift by half a cell to get floor(p/dcell)
                    const long long q = g.f0[d] + (long long)i * g.step[d] + (1LL << 31);
                    const float fu = (float)(unsigned)(q & 0xffffffffLL) * 2.3283064365386963e-10f;
                    ci[d] = g.near ? wrap_near(g.i0[d] + (int)(q >> 32), dims[d]) : wrap32(g.i0[d] + (int)(q >> 32), dims[d]);
                    rpos[d] = ((double)(g.i0u[d] + (q >> 32)) + (double)fu) * a.dcell - a.obs[d];
                    if (d == 0) fux = fu;
#pragma unroll
                    for (int c = -GR; c <= GR; ++c) {
                        const float x = (float)c + 0.5f - fu;
                        ew[d][c + GR] = expf(-0.5f * x * x);
                    }
                }
                float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
                for (int c = 0; c < 2 * GR + 1; ++c) {
                    sx += ew[0][c];
                    sy += ew[1][c];
                    sz += ew[2][c];
                }
                int ixs[2 * GR + 1 + !GAUSS], iys[2 * GR + 1 + !GAUSS], izs[2 * GR + 1 + !GAUSS];
#pragma unroll
                for (int c = 0; c < 2 * GR + 1; ++c) {
                    ixs[c] = g.near ? wrap_near(ci[0] + c - GR, dims[0]) : wrap32(ci[0] + c - GR, dims[0]);
                    iys[c] = g.near ? wrap_near(ci[1] + c - GR, dims[1]) : wrap32(ci[1] + c - GR, dims[1]);
                    izs[c] = g.near ? wrap_near(ci[2] + c - GR, dims[2]) : wrap32(ci[2] + c - GR, dims[2]);
                }
                const bool rsd = a.eta6[0] != nullptr;
                float acc[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                for (int cx = -GR; cx <= GR; ++cx) {
                    const int ixw = ixs[cx + GR];
                    for (int cy = -GR; cy <= GR; ++cy) {
                        const int iyw = iys[cy + GR];
                        const float wxy = ew[0][cx + GR] * ew[1][cy + GR];
                        const int64_t row = ((int64_t)ixw * a.ny + iyw) * a.pitch;
#pragma unroll
                        for (int cz = -GR; cz <= GR; ++cz) {
                            const int izw = izs[cz + GR];
                            const float w = wxy * ew[2][cz + GR];
                            acc[0] = fmaf(w, __ldg(a.delta + row + izw), acc[0]);
                            if (rsd) {
#pragma unroll
                                for (int f = 0; f < 6; ++f) acc[1 + f] = fmaf(w, __ldg(a.eta6[f] + row + izw), acc[1 + f]);
                            }
                        }
                    }
                }
                const float inv = 1.0f / (sx * sy * sz);
                dl = acc[0] * inv;
                et = 0.f;
                if (rsd) {
                    const double X = rpos[0], Y = rpos[1], Z = rpos[2];
                    const double RR = X * X + Y * Y + Z * Z;
                    const double e = (X * acc[1] * X + Y * acc[2] * Y + Z * acc[3] * Z + 2 * X * acc[4] * Y +
                                      2 * X * acc[5] * Z + 2 * Y * acc[6] * Z) / RR;
                    et = (float)e * inv;
                }
                // redshift from the wrapped x coordinate x / dcell = ci_x + fu_x (as the trilinear read)
                const float xc = (float)ci[0] + fux;
                z = a.z_lo + (a.z_hi - a.z_lo) * (xc / nxf);
            } else {
                const SkewerGeo& g = geo[t];
                int c0[3], c1[3];
                float fr[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const long long q = g.f0[d] + (long long)i * g.step[d];
                    fr[d] = (float)(unsigned)(q & 0xffffffffLL) * 2.3283064365386963e-10f;  // 2^-32
                    c0[d] = g.near ? wrap_near(g.i0[d] + (int)(q >> 32), dims[d]) : wrap32(g.i0[d] + (int)(q >> 32), dims[d]);
                    c1[d] = c0[d] + 1 == dims[d] ? 0 : c0[d] + 1;
                }
                const int64_t r00 = ((int64_t)c0[0] * a.ny + c0[1]) * a.pitch;
                const int64_t r01 = ((int64_t)c0[0] * a.ny + c1[1]) * a.pitch;
                const int64_t r10 = ((int64_t)c1[0] * a.ny + c0[1]) * a.pitch;
                const int64_t r11 = ((int64_t)c1[0] * a.ny + c1[1]) * a.pitch;
                const float wx1 = fr[0], wx0 = 1.f - fr[0], wy1 = fr[1], wy0 = 1.f - fr[1];
                const float wz1 = fr[2], wz0 = 1.f - fr[2];
                const int z0 = c0[2], z1 = c1[2];
                auto tri = [&](const float* __restrict__ box) {
                    const float v00 = wz0 * __ldg(box + r00 + z0) + wz1 * __ldg(box + r00 + z1);
                    const float v01 = wz0 * __ldg(box + r01 + z0) + wz1 * __ldg(box + r01 + z1);
                    const float v10 = wz0 * __ldg(box + r10 + z0) + wz1 * __ldg(box + r10 + z1);
                    const float v11 = wz0 * __ldg(box + r11 + z0) + wz1 * __ldg(box + r11 + z1);
                    return wx0 * (wy0 * v00 + wy1 * v01) + wx1 * (wy0 * v10 + wy1 * v11);
                };
                dl = tri(a.delta);
                et = a.eta ? tri(a.eta) : 0.f;
                // redshift from the wrapped x coordinate: x / dcell = c0x + frx + 0.5
                float xc = (float)c0[0] + fr[0] + 0.5f;
                if (xc >= nxf) xc -= nxf;
                z = a.z_lo + (a.z_hi - a.z_lo) * (xc / nxf);
            }
            float ds = 0.f;
            if (a.ss_mode != SMK_SS_NONE && (t ? live1 : live0)) {
                ds = too_long ? __int_as_float(0x7fc00000) : (t ? s[i].y : s[i].x) * inv_nz;
                if (a.ss_zsigma && a.ss_nztab > 0) ds *= zsigma_at(a, z) / sk_sig_eff[t];
            }
            float pa = a.a, pb = a.b, pc = a.c;
            if (a.abc_mode == SMK_ABC_POWERLAW) {
                // a ((1 + z)/zref1)^power as exp2(power log2(.)): relative error ~3e-7 on the
                // 1.8-3.6 range (powf's extra-precise product is not needed for the flux tolerance)
                pa = a.a * exp2f(a.a_power * log2f((1.0f + z) / a.a_zref1));
            } else if (a.abc_mode == SMK_ABC_TABLE) {
                const float tt = (z - a.z_tab0) / a.dz_tab;
                int it = (int)floorf(tt);
                it = max(0, min(a.n_tab - 2, it));
                const float ft = fminf(fmaxf(tt - (float)it, 0.f), 1.f);
                const float* r0 = a.abc_tab + 3 * it;
                pa = fmaf(ft, __ldg(r0 + 3) - __ldg(r0), __ldg(r0));
                pb = fmaf(ft, __ldg(r0 + 4) - __ldg(r0 + 1), __ldg(r0 + 1));
                pc = fmaf(ft, __ldg(r0 + 5) - __ldg(r0 + 2), __ldg(r0 + 2));
            }
            const float G = a.growth_mode == SMK_G_MERGE ? a.growth24 * 3.4f / (1.0f + z) : 1.0f;
            const float dtot = dl + ds;
            const float F = expf(-pa * expf(pb * G * (dtot + pc * et)));
            a.flux[o] = F;
            if (a.delta_out) a.delta_out[o] = dtot;
            if (a.eta_out) a.eta_out[o] = et;
            if (a.z_out) a.z_out[o] = z;
        }
        __syncthreads();
    }
}

}  // namespace smk

using namespace smk;

extern "C" {

size_t smk_skewers_workspace_size(const SmkSkewers* sk, const SmkSpectraParams* p) {
    (void)sk;
    (void)p;
    return 256;  // work counter
}

int smk_skewers_flux(const SmkSkewers* sk, const SmkSpectraParams* p, const float* delta_box,
                     const float* eta_box, float* flux, float* delta_out, float* eta_out, float* z_out,
                     void* workspace, size_t workspace_bytes, void* stream) {
    if (!sk || !p) return fail(SMK_EINVAL, "smk_skewers_flux: null argument");
    if (sk->n_slots == 0 && sk->n >= 0) return SMK_OK;   // empty table: nothing to read or write
    if (!flux) return fail(SMK_EINVAL, "smk_skewers_flux: null flux");
    if (p->interp != SMK_INTERP_PIXELS && !delta_box)
        return fail(SMK_EINVAL, "smk_skewers_flux: a box read needs the delta box");
    if (p->interp == SMK_INTERP_GAUSS343) {
        const int nset = !!p->eta6[0] + !!p->eta6[1] + !!p->eta6[2] + !!p->eta6[3] + !!p->eta6[4] + !!p->eta6[5];
        if (nset != 0 && nset != 6) return fail(SMK_EINVAL, "smk_skewers_flux: give all six eta_ij boxes or none");
        if (p->gauss_dmax < 0 || p->gauss_dmax > 4)
            return fail(SMK_EINVAL, "smk_skewers_flux: gauss_dmax must be 0 (= 3) or 1..4");
    }
    if (p->interp == SMK_INTERP_PIXELS && (!sk->pix_delta || !sk->pix_z))
        return fail(SMK_EINVAL, "smk_skewers_flux: SMK_INTERP_PIXELS needs pix_delta and pix_z");
    if (sk->n < 0 || sk->n_slots < 0 || (sk->n_slots & 1)) return fail(SMK_EINVAL, "smk_skewers_flux: bad counts");
    if (sk->n_slots == 0) return SMK_OK;
    if (!sk->npix || !sk->offset || !sk->order) return fail(SMK_EINVAL, "smk_skewers_flux: null skewer table array");
    if (p->interp == SMK_INTERP_TRILINEAR || p->interp == SMK_INTERP_GAUSS343) {
        if ((!sk->start && !sk->start64) || (!sk->dir && !sk->dir64))
            return fail(SMK_EINVAL, "smk_skewers_flux: null start/dir");
        if (p->nx < 1 || p->ny < 1 || p->nz < 1 || p->pitch < p->nz || !(p->dcell > 0) || !(sk->dpix > 0))
            return fail(SMK_EINVAL, "smk_skewers_flux: bad box geometry");
        // a skewer then advances fewer than 2^30 cells (npix <= 2^24), the kernel's 32-bit index range
        if (sk->dpix > 64.0 * p->dcell)
            return fail(SMK_EINVAL, "smk_skewers_flux: pixel spacing above 64 cells");
    } else if (p->interp != SMK_INTERP_PIXELS) {
        return fail(SMK_EINVAL, "smk_skewers_flux: unknown interp");
    }
    if (p->ss_mode != SMK_SS_NONE && p->ss_mode != SMK_SS_HOST && p->ss_mode != SMK_SS_PHILOX)
        return fail(SMK_EINVAL, "smk_skewers_flux: unknown ss_mode");
    if (p->ss_mode != SMK_SS_NONE) {
        if (!p->ss_scale) return fail(SMK_EINVAL, "smk_skewers_flux: null ss_scale");
        if (p->ss_nz != 0 && (p->ss_nz < 256 || p->ss_nz > FFT_MAX_N || (p->ss_nz & (p->ss_nz - 1))))
            return fail(SMK_EINVAL, "smk_skewers_flux: ss_nz must be 0 or a power of two in 256..4096");
        if (p->ss_mode == SMK_SS_HOST && (!p->ss_noise || !p->ss_noise_offset))
            return fail(SMK_EINVAL, "smk_skewers_flux: SMK_SS_HOST needs ss_noise and offsets");
        if (p->ss_nztab < 0 || (p->ss_nztab > 0 && !p->ss_ztab))
            return fail(SMK_EINVAL, "smk_skewers_flux: ss_nztab > 0 needs the ss_ztab redshifts");
    }
    if (p->abc_mode == SMK_ABC_TABLE && (!p->abc_tab || p->n_tab < 2 || !(p->dz_tab > 0)))
        return fail(SMK_EINVAL, "smk_skewers_flux: bad a,b,c table");
    if (p->abc_mode == SMK_ABC_POWERLAW && !(p->a_zref1 > 0))
        return fail(SMK_EINVAL, "smk_skewers_flux: a_zref1 must be > 0");
    if (p->abc_mode < SMK_ABC_CONST || p->abc_mode > SMK_ABC_TABLE)
        return fail(SMK_EINVAL, "smk_skewers_flux: unknown abc_mode");
    if (!workspace || workspace_bytes < smk_skewers_workspace_size(sk, p))
        return fail(SMK_EWORKSPACE, "smk_skewers_flux: needs %zu workspace bytes",
                    smk_skewers_workspace_size(sk, p));
    SkArgs a;
    a.start = sk->start;
    a.dir = sk->dir;
    a.start64 = sk->start64;
    a.dir64 = sk->dir64;
    a.npix = sk->npix;
    a.offset = sk->offset;
    a.dpix = sk->dpix;
    a.order = sk->order;
    a.n_items = sk->n_slots / 2;
    a.interp = p->interp;
    for (int f = 0; f < 6; ++f) a.eta6[f] = p->eta6[f];
    for (int d = 0; d < 3; ++d) a.obs[d] = p->obs[d];
    a.pix_delta = sk->pix_delta;
    a.pix_eta = sk->pix_eta;
    a.pix_z = sk->pix_z;
    a.delta = delta_box;
    a.eta = eta_box;
    a.nx = p->nx;
    a.ny = p->ny;
    a.nz = p->nz;
    a.pitch = p->pitch;
    a.dcell = p->dcell;
    a.ss_mode = p->ss_mode;
    a.ss_nz = p->ss_nz;
    a.ss_scale = p->ss_scale;
    a.ss_noise = p->ss_noise;
    a.ss_noise_offset = p->ss_noise_offset;
    a.seed = p->seed;
    a.forest = sk->forest;
    a.ss_nztab = p->ss_mode != SMK_SS_NONE ? p->ss_nztab : 0;
    a.ss_ztab = p->ss_ztab;
    a.ss_zsigma = p->ss_zsigma;
    for (int j = 0; j < SK_NCLASS; ++j) make_plan(256 << j, &a.plans[j], 16);
    a.abc_mode = p->abc_mode;
    a.a = p->a;
    a.b = p->b;
    a.c = p->c;
    a.a_zref1 = p->a_zref1;
    a.a_power = p->a_power;
    a.abc_tab = p->abc_tab;
    a.n_tab = p->n_tab;
    a.z_tab0 = p->z_tab0;
    a.dz_tab = p->dz_tab;
    a.z_lo = p->z_lo;
    a.z_hi = p->z_hi;
    a.growth_mode = p->growth_mode;
    a.growth24 = p->growth24;
    a.flux = flux;
    a.delta_out = delta_out;
    a.eta_out = eta_out;
    a.z_out = z_out;
    a.counter = reinterpret_cast<unsigned long long*>(workspace);
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), st) != cudaSuccess)
        return check_launch("cudaMemsetAsync(counter)");
    // small-scale lines: fixed ss_nz, or (ss_nz = 0) per skewer up to FFT_MAX_N
    a.ss_nmax = p->ss_mode == SMK_SS_NONE ? 0 : (p->ss_nz > 0 ? p->ss_nz : FFT_MAX_N);
    const size_t smem = 2 * (size_t)a.ss_nmax * sizeof(float2) + (size_t)a.ss_nmax * sizeof(int) + 16;
    const bool gauss = p->interp == SMK_INTERP_GAUSS343;
    const int dmax = p->gauss_dmax > 0 ? p->gauss_dmax : 3;
    auto kern = !gauss ? skewer_kernel<0> : dmax == 1 ? skewer_kernel<1> : dmax == 2 ? skewer_kernel<2>
              : dmax == 3 ? skewer_kernel<3> : skewer_kernel<4>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute(skewer_kernel)");
    int per_sm = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SK_T, smem) != cudaSuccess)
        return check_launch("occupancy(skewer_kernel)");
    int per = std::max(per_sm, 1);
    const int cap = g_skewer_blocks.load();
    if (cap > 0) per = std::min(per, cap);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(a.n_items, (int64_t)per * nsm));
    kern<<<grid, SK_T, smem, st>>>(a);
    return check_launch("skewer_kernel");
}

}  // extern "C"

// ------------------------------------------------------------------ allocation-free variant
// Scratch of smk_skewers_flux_static, resident in every process that loads the library:
// words [0, 64) hold the persistent launch's work counter (the 256-byte workspace of
// smk_skewers_flux), words [64, 64 + SMK_STATIC_MAX_SLOTS) the work schedule.  Host code may
// not use this name as a device address; it takes the address from cudaGetSymbolAddress.
static __device__ __align__(256) int32_t g_skewer_scratch[64 + SMK_STATIC_MAX_SLOTS];

namespace {
std::mutex g_scratch_mutex;
int32_t* g_scratch_ptr[SMK_STATIC_MAX_DEVICES] = {};

// Device address of the scratch on the current device, looked up once per device.
int scratch_address(int32_t** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("cudaGetDevice");
    if (dev < 0 || dev >= SMK_STATIC_MAX_DEVICES)
        return fail(SMK_ENOTSUPP, "smk_skewers_flux_static: device %d beyond the %d supported", dev,
                    SMK_STATIC_MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_skewer_scratch);
        if (e != cudaSuccess)
            return fail(SMK_ECUDA, "smk_skewers_flux_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<int32_t*>(ptr);
    }
    *out = g_scratch_ptr[dev];
    return SMK_OK;
}
}  // namespace

extern "C" int smk_skewers_flux_static(const SmkSkewers* sk, const int32_t* npix_host,
                                       const SmkSpectraParams* p, const float* delta_box,
                                       const float* eta_box, float* flux, float* delta_out,
                                       float* eta_out, float* z_out, void* stream) {
    if (!sk || !p || !npix_host) return fail(SMK_EINVAL, "smk_skewers_flux_static: null argument");
    if (sk->n < 0 || sk->n > SMK_STATIC_MAX_SLOTS - 16)
        return fail(SMK_EINVAL, "smk_skewers_flux_static: %lld skewers; the static scratch holds the "
                    "schedule of at most %d", (long long)sk->n, SMK_STATIC_MAX_SLOTS - 16);
    int32_t* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    // host-side schedule (same as smk_skewer_schedule), then into the static scratch
    std::vector<int32_t> order((size_t)(2 * sk->n + 16));
    int64_t n_slots = 0;
    const int32_t ss_nz = p->ss_mode != SMK_SS_NONE ? p->ss_nz : -1;
    if ((rc = smk_skewer_schedule(sk->n, npix_host, ss_nz, order.data(), &n_slots))) return rc;
    if (n_slots > SMK_STATIC_MAX_SLOTS)
        return fail(SMK_EINVAL, "smk_skewers_flux_static: schedule of %lld slots exceeds %d",
                    (long long)n_slots, SMK_STATIC_MAX_SLOTS);
    cudaStream_t st = (cudaStream_t)stream;
    // pageable source: the copy has read it when cudaMemcpyAsync returns
    if (n_slots > 0 && cudaMemcpyAsync(scratch + 64, order.data(), (size_t)n_slots * sizeof(int32_t),
                                       cudaMemcpyHostToDevice, st) != cudaSuccess)
        return check_launch("smk_skewers_flux_static: schedule copy");
    SmkSkewers s2 = *sk;
    s2.order = scratch + 64;
    s2.n_slots = n_slots;
    // the work counter is zeroed by smk_skewers_flux itself (cudaMemsetAsync on the stream)
    return smk_skewers_flux(&s2, p, delta_box, eta_box, flux, delta_out, eta_out, z_out, scratch,
                            64 * sizeof(int32_t), stream);
}
