// GRF boxes (make_boxes) on GB300: host orchestration of the HBM passes (kernels in
// smk_grf_kernels.cuh, instantiated per tile variant in smk_grf_{zpass,line,x}.cu), the FP64
// P(k) normalisation, the box check, and the tile-variant tuning table.
#include "smk_grf_kernels.cuh"

namespace smk {

// ------------------------------------------------------------------ P(k) normalisation
__global__ void pk_norm_kernel(int nx, int ny, int nz, double kfac, float inv_k0, double* acc) {
    // k_z of every column once per block (the per-mode arithmetic stays in float32: FP64 is a
    // small fraction of the FP32 rate on this GPU)
    extern __shared__ float kzt[];
    const int nzh = nz / 2 + 1;
    for (int z = threadIdx.x; z < nzh; z += blockDim.x) kzt[z] = kaxis(z, nz, kfac, false);
    __syncthreads();
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
            const float kz = kzt[z];
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


int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

// ------------------------------------------------------------------ tile-variant tables
#define X(W, T, N, R, B) {W, T, N, R, B},
static const TileVariant kZVar[] = {SMK_Z_VARIANTS(X)};
static const TileVariant kZInvVar[] = {SMK_ZINV_VARIANTS(X)};
static const TileVariant kLineVar[] = {SMK_LINE_VARIANTS(X)};
static const TileVariant kXVar[] = {SMK_X_VARIANTS(X)};
static const TileVariant kXGenVar[] = {SMK_XGEN_VARIANTS(X)};
#undef X

static std::atomic<int> g_choice[NPASS][4];  // tuned variant per pass and length class, -1: default
static struct ChoiceInit {
    ChoiceInit() {
        for (auto& row : g_choice)
            for (auto& c : row) c.store(-1);
    }
} g_choice_init;

static std::atomic<int> g_xgen_split{-1};  // -1: by footprint, 0: never, 1: always
static std::atomic<int> g_prefetch{1};     // L2 prefetch of the next tile in the y and z passes
static std::atomic<int> g_tma{1};          // TMA tensor loads of the y pass's tiles
static std::atomic<int> g_tma_wait_test{0};  // y-pass TMA waits made to run out (failure test)

static int length_class(int n) { return n <= 512 ? 0 : n <= 1024 ? 1 : n <= 2560 ? 2 : 3; }

const TileVariant* variant_table(int pass) {
    switch (pass) {
        case PASS_ZFWD: return kZVar;
        case PASS_ZINV: return kZInvVar;
        case PASS_LINE: return kLineVar;
        case PASS_XPASS: return kXVar;
        case PASS_XGEN: return kXGenVar;
        default: return nullptr;
    }
}

int variant_count(int pass) {
    switch (pass) {
        case PASS_ZFWD: return (int)(sizeof(kZVar) / sizeof(kZVar[0]));
        case PASS_ZINV: return (int)(sizeof(kZInvVar) / sizeof(kZInvVar[0]));
        case PASS_LINE: return (int)(sizeof(kLineVar) / sizeof(kLineVar[0]));
        case PASS_XPASS: return (int)(sizeof(kXVar) / sizeof(kXVar[0]));
        case PASS_XGEN: return (int)(sizeof(kXGenVar) / sizeof(kXGenVar[0]));
        default: return 0;
    }
}

int variant_for(int pass, int n) {
    const TileVariant* t = variant_table(pass);
    const int cnt = variant_count(pass);
    const int c = g_choice[pass][length_class(n)].load();
    if (c >= 0 && c < cnt && variant_fits(t[c], n)) return c;
    // built-in choice: a variant compiled for exactly this length, else the z passes prefer
    // the one-warp-per-row-pair engine (W = 0), every pass otherwise the first variant whose
    // line length covers n
    for (int i = 0; i < cnt; ++i)
        if (t[i].nmax == -n) return i;
    if (pass == PASS_ZINV || pass == PASS_ZFWD)
        for (int i = 0; i < cnt; ++i)
            if (t[i].w == 0 && variant_fits(t[i], n)) return i;
    for (int i = 0; i < cnt; ++i)
        if (variant_fits(t[i], n)) return i;
    return cnt - 1;
}

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

// k_z columns per chunk of the x pass's blocked intermediate (0: in place).
static int64_t xi_chunk_cols(const SmkGrfParams* p) {
    if (!p || p->xi_chunk_kz <= 0 || p->nz < 2) return 0;
    const int64_t nzh16 = (p->nz / 2 + 1 + 15) / 16 * 16;
    return std::min<int64_t>(((int64_t)p->xi_chunk_kz + 15) / 16 * 16, nzh16);
}

size_t smk_grf_workspace_size(const SmkGrfParams* p) {
    // [0] FP64 mode sum, [1] amplitude A; then the intermediate of one chunk
    const int64_t cols = xi_chunk_cols(p);
    if (!cols) return 256;
    const int64_t nf = p->want_eta ? 2 : 1;
    return 256 + (size_t)(nf * p->batch * (int64_t)p->nx * p->ny * cols) * sizeof(float2);
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
    pk_norm_kernel<<<grid, 256, (size_t)(nz / 2 + 1) * sizeof(float), st>>>(nx, ny, nz, kfac, (float)(1.0 / k0),
                                                                          amp_dev);
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

// y inverse reading the blocked intermediate I of a chunk of xcols columns (blocks of kb
// columns, nf fields): the in-place arguments with the source, and 5-D TMA maps over I.
static LineArgs staged_y(const LineArgs& ya, float2* const* I, int nf, int kb, int wy, int64_t xcols,
                         int64_t nouter, int ny) {
    LineArgs yi = ya;
    yi.nbuf = nf;
    yi.src[0] = I[0];
    yi.src[1] = nf > 1 ? I[1] : nullptr;
    yi.src_kb = kb;
    if (yi.tma == 2) yi.tma = 1;   // stores go to the boxes; the maps cover the intermediate
    const int per = wy / kb;         // intermediate blocks per y tile
    const uint64_t dims[5] = {(uint64_t)kb, (uint64_t)per, (uint64_t)ny, (uint64_t)nouter, (uint64_t)(xcols / wy)};
    const uint64_t strides[5] = {1, (uint64_t)(nouter * ny * kb), (uint64_t)kb, (uint64_t)ny * kb,
                                 (uint64_t)(per * nouter * ny * kb)};
    const uint32_t box[5] = {(uint32_t)kb, (uint32_t)per, (uint32_t)std::max(ya.box_rows, 1), 1, 1};
    for (int f = 0; f < nf && yi.tma; ++f)
        if (!encode_map_5d_8b(&yi.tmap[f], I[f], dims, strides, box)) yi.tma = 0;
    return yi;
}

int smk_grf_boxes(const SmkGrfParams* p, float* delta, float* eta, double* stats, void* workspace,
                  size_t workspace_bytes, void* stream) {
    if (!p || !delta) return fail(SMK_EINVAL, "smk_grf_boxes: null params or delta");
    if (p->batch < 1 || p->nx < 2 || p->ny < 2 || p->nz < 2 || (p->nz & 1))
        return fail(SMK_EINVAL, "smk_grf_boxes: need nx, ny >= 2, nz >= 2 even, batch >= 1");
    if (!(p->dcell > 0)) return fail(SMK_EINVAL, "smk_grf_boxes: dcell must be > 0");
    if (p->want_eta && !eta) return fail(SMK_EINVAL, "smk_grf_boxes: want_eta needs an eta box");
    if (((uintptr_t)delta & 15) || (p->want_eta && ((uintptr_t)eta & 15)) || ((uintptr_t)workspace & 15))
        return fail(SMK_EINVAL, "smk_grf_boxes: delta, eta and workspace must be 16-byte aligned");
    if (p->eta_comp < SMK_ETA_ZZ || p->eta_comp > SMK_ETA_VZ)
        return fail(SMK_EINVAL, "smk_grf_boxes: unknown eta_comp");
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
    // tile variant of every pass, and each pass's radix plan within its register budget
    const bool gpu_noise = p->noise_mode == SMK_NOISE_PHILOX;
    const int pass_x = gpu_noise ? PASS_XGEN : PASS_XPASS;
    const int vx = variant_for(pass_x, p->nx), vy = variant_for(PASS_LINE, p->ny);
    const int vzf = variant_for(PASS_ZFWD, p->nz), vzi = variant_for(PASS_ZINV, p->nz);
    auto rmax = [](int pass, int v) { return variant_table(pass)[v].rmax; };
    FftPlan plx, ply, plzf, plzi;
    if (!make_plan(p->nx, &plx, rmax(pass_x, vx)) || !make_plan(p->ny, &ply, rmax(PASS_LINE, vy)) ||
        !make_plan(p->nz, &plzf, rmax(PASS_ZFWD, vzf)) || !make_plan(p->nz, &plzi, rmax(PASS_ZINV, vzi)))
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
    LineArgs ya = {};
    ya.pl = ply;
    ya.base[0] = d2;
    ya.base[1] = e2;
    ya.nbuf = 1;
    ya.n_outer = (int64_t)p->batch * p->nx;
    ya.ostride = (int64_t)p->ny * cp;
    ya.estride = cp;
    ya.ncol = nzh;
    ya.prefetch = g_prefetch.load();
    ya.tma = 0;
    const bool wait_test = g_tma_wait_test.load() != 0;
    ya.tma_extra_tx = wait_test ? 16 : 0;
    ya.tma_wait_limit = wait_test ? 20000000LL : 2000000000LL;   // ~10 ms / ~1 s at 2 GHz
    if (g_tma.load()) {
        // tile boxes: the variant's W columns x the largest divisor of ny up to 256 rows (128-row
        // boxes, which let a 2560 tile load in four parts instead of two, measured slower)
        const int wl = variant_table(PASS_LINE)[vy].w;
        int rows = 1;
        for (int d = std::min(p->ny, 256); d >= 1; --d)
            if (p->ny % d == 0) {
                rows = d;
                break;
            }
        ya.box_rows = rows;
        // every box lands on a 128-byte boundary of the tile
        ya.tma = ((size_t)rows * wl * sizeof(float2)) % 128 == 0 &&
                 encode_map_3d_8b(&ya.tmap[0], delta, (uint64_t)nzh, (uint64_t)p->ny, (uint64_t)ya.n_outer,
                                  (uint64_t)cp, (uint64_t)ya.ostride, (uint32_t)wl, (uint32_t)rows) &&
                         (!p->want_eta || encode_map_3d_8b(&ya.tmap[1], eta, (uint64_t)nzh, (uint64_t)p->ny,
                                                           (uint64_t)ya.n_outer, (uint64_t)cp, (uint64_t)ya.ostride,
                                                           (uint32_t)wl, (uint32_t)rows))
                     ? g_tma.load() : 0;
    }
    const int64_t rows_per_box = (int64_t)p->nx * p->ny;
    const float inv_vcell = 1.0f / (float)(p->dcell * p->dcell * p->dcell);
    if (gpu_noise) {
        // Fourier modes drawn in the x pass: no forward z / y passes
        if ((rc = mark(1)) || (rc = mark(2))) return rc;
        XGenArgs ga = {};
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
        philox_round_keys(p->seed, ga.rk0, ga.rk1);
        ga.eta_comp = p->eta_comp;
        ga.vfac = (float)p->vel_factor;
        const int nf = p->want_eta ? 2 : 1;
        const int wx = variant_table(PASS_XGEN)[vx].w, wy = variant_table(PASS_LINE)[vy].w;
        const int kb = wx / nf;   // k_z columns per block of the intermediate
        const int64_t xcols = xi_chunk_cols(p);
        if (xcols > 0 && (!workspace || workspace_bytes < smk_grf_workspace_size(p)))
            return fail(SMK_EWORKSPACE, "smk_grf_boxes: xi_chunk_kz needs %zu workspace bytes",
                        smk_grf_workspace_size(p));
        const bool staged = xcols > 0 && kb >= 2 && kb % 2 == 0 && wy % kb == 0 && xcols % wy == 0;
        if (staged) {
            // Chunks of xcols k_z columns: the x pass of both fields into the intermediate (each
            // mode drawn once; the rows of a tile ny * kb * 8 bytes apart instead of ny * pitch *
            // 4), then the y pass reading its tiles from the intermediate as contiguous runs.
            float2* I0 = reinterpret_cast<float2*>(reinterpret_cast<char*>(workspace) + 256);
            const int64_t nouter = (int64_t)p->batch * p->nx;
            ga.I[0] = I0;
            ga.I[1] = p->want_eta ? I0 + nouter * p->ny * xcols : nullptr;
            ga.fields = p->want_eta ? XGEN_BOTH : XGEN_DELTA;
            LineArgs yi = staged_y(ya, ga.I, nf, kb, wy, xcols, nouter, p->ny);
            const bool one_chunk = xcols >= nzh;
            for (int64_t c0 = 0; c0 < nzh; c0 += xcols) {
                ga.cb0 = (int)(c0 / kb);
                ga.ncb = (int)ceil_div(std::min<int64_t>(xcols, nzh - c0), kb);
                if ((rc = run_xgi(vx, ga, st))) return rc;
                if (one_chunk && (rc = mark(3))) return rc;
                yi.col0 = (int)c0;
                yi.ncol = (int)std::min<int64_t>(xcols, nzh - c0);
                if ((rc = run_line(vy, yi, true, st))) return rc;
            }
            if ((!one_chunk && (rc = mark(3))) || (rc = mark(4))) return rc;
        } else {
            // A tile writes all nx rows of its columns, so one wave of tiles touches rows spread
            // over the whole of each output box.  Past ~64 GiB for the two boxes together (2 x 40
            // GB at 2560x2560x1536) that spread outruns the GPU's address-translation reach and
            // the pass slows by 1.7x; writing delta and eta in two launches keeps each wave
            // within one box.
            const double pair_bytes = 2.0 * 4.0 * (double)p->batch * p->nx * p->ny * (double)pitch;
            const int sm = g_xgen_split.load();
            const bool split = p->want_eta && (sm < 0 ? pair_bytes > 64.0 * (1ull << 30) : sm == 1);
            ga.fields = !p->want_eta ? XGEN_DELTA : (split ? XGEN_DELTA : XGEN_BOTH);
            if ((rc = run_xgen(vx, ga, st))) return rc;
            if (split) {
                ga.fields = XGEN_ETA;
                if ((rc = run_xgen(vx, ga, st))) return rc;
            }
            if ((rc = mark(3))) return rc;
            // 4. c2c along y, inverse, on delta (and eta)
            ya.nbuf = nf;
            if ((rc = run_line(vy, ya, true, st))) return rc;
            if ((rc = mark(4))) return rc;
        }
    } else {
        // 1. r2c along z of the caller's noise
        ZFwdArgs za = {};
        za.pl = plzf;
        za.batch = p->batch;
        za.pitch = pitch;
        za.noise = p->noise;
        za.out = delta;
        za.prefetch = g_prefetch.load();
        if ((rc = run_zfwd(vzf, za, rows_per_box, st))) return rc;
        if ((rc = mark(1))) return rc;
        // 2. c2c along y, forward (the y spectrum stays in digit-reversed order); 3. x: forward,
        // P(k) scaling + eta split, inverse
        XArgs xa = {};
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
        xa.eta_comp = p->eta_comp;
        xa.vfac = (float)p->vel_factor;
        const int nf = p->want_eta ? 2 : 1;
        const int wxp = variant_table(PASS_XPASS)[vx].w, wy = variant_table(PASS_LINE)[vy].w;
        const int kb = p->want_eta ? wxp / 2 : wxp;
        const int64_t xcols = xi_chunk_cols(p);
        if (xcols > 0 && (!workspace || workspace_bytes < smk_grf_workspace_size(p)))
            return fail(SMK_EWORKSPACE, "smk_grf_boxes: xi_chunk_kz needs %zu workspace bytes",
                        smk_grf_workspace_size(p));
        if (xcols > 0 && kb >= 2 && kb % 2 == 0 && wy % kb == 0 && wy / kb <= 8 && xcols % wy == 0) {
            // chunks of xcols k_z columns: the y forward of the chunk's columns writes the blocked
            // layout of the intermediate's first field, the x pass reads it there as rows
            // ny * kb * 8 bytes apart (not ny * pitch * 4) and writes both fields back into the
            // intermediate, and the y inverse reads them as contiguous runs
            float2* I0 = reinterpret_cast<float2*>(reinterpret_cast<char*>(workspace) + 256);
            const int64_t nouter = (int64_t)p->batch * p->nx;
            xa.I[0] = I0;
            xa.I[1] = p->want_eta ? I0 + nouter * p->ny * xcols : nullptr;
            xa.prefetch = g_prefetch.load();
            xa.src_blocked = 1;
            LineArgs yf = ya;
            yf.nbuf = 1;
            yf.dst = I0;
            yf.dst_kb = kb;
            if (yf.tma == 2) yf.tma = 1;
            LineArgs yi = staged_y(ya, xa.I, nf, kb, wy, xcols, nouter, p->ny);
            const bool one_chunk = xcols >= nzh;
            for (int64_t c0 = 0; c0 < nzh; c0 += xcols) {
                const int ncol = (int)std::min<int64_t>(xcols, nzh - c0);
                yf.col0 = (int)c0;
                yf.ncol = ncol;
                if ((rc = run_line(vy, yf, false, st))) return rc;
                if (one_chunk && (rc = mark(2))) return rc;
                xa.cb0 = (int)(c0 / kb);
                xa.ncb = (int)ceil_div(ncol, kb);
                if ((rc = run_xpi(vx, xa, st))) return rc;
                if (one_chunk && (rc = mark(3))) return rc;
                yi.col0 = (int)c0;
                yi.ncol = ncol;
                if ((rc = run_line(vy, yi, true, st))) return rc;
            }
            if ((!one_chunk && ((rc = mark(2)) || (rc = mark(3)))) || (rc = mark(4))) return rc;
        } else {
            if ((rc = run_line(vy, ya, false, st))) return rc;
            if ((rc = mark(2))) return rc;
            if ((rc = run_xpass(vx, xa, st))) return rc;
            if ((rc = mark(3))) return rc;
            // 4. c2c along y, inverse, on delta (and eta)
            ya.nbuf = nf;
            if ((rc = run_line(vy, ya, true, st))) return rc;
            if ((rc = mark(4))) return rc;
        }
    }

    // 5. c2r along z, / N, statistics
    ZInvArgs ia;
    ia.pl = plzi;
    ia.batch = p->batch;
    ia.buf[0] = delta;
    ia.buf[1] = eta;
    ia.nbuf = p->want_eta ? 2 : 1;
    ia.pitch = pitch;
    ia.scale = (float)(1.0 / ((double)p->nx * p->ny * p->nz));
    ia.stats = stats;
    ia.prefetch = g_prefetch.load();
    if ((rc = run_zinv(vzi, ia, rows_per_box, st))) return rc;
    return mark(5);
}

int smk_tune_flag(int32_t flag, int32_t value, int32_t* previous) {
    int old;
    if (flag == SMK_TUNE_XGEN_SPLIT) {
        if (value < -1 || value > 1) return fail(SMK_EINVAL, "smk_tune_flag: XGEN_SPLIT must be -1, 0 or 1");
        old = g_xgen_split.exchange(value);
    } else if (flag == SMK_TUNE_TMA_WAIT_TEST) {
        if (value < 0 || value > 1) return fail(SMK_EINVAL, "smk_tune_flag: TMA_WAIT_TEST must be 0 or 1");
        old = g_tma_wait_test.exchange(value);
    } else if (flag == SMK_TUNE_TMA) {
        if (value < 0 || value > 2) return fail(SMK_EINVAL, "smk_tune_flag: TMA must be 0, 1 or 2");
        old = g_tma.exchange(value);
    } else if (flag == SMK_TUNE_SKEWER_BLOCKS) {
        if (value < 0 || value > 32) return fail(SMK_EINVAL, "smk_tune_flag: SKEWER_BLOCKS must be 0..32");
        old = g_skewer_blocks.exchange(value);
    } else if (flag == SMK_TUNE_PREFETCH) {
        if (value < 0 || value > 1) return fail(SMK_EINVAL, "smk_tune_flag: PREFETCH must be 0 or 1");
        old = g_prefetch.exchange(value);
    } else {
        return fail(SMK_EINVAL, "smk_tune_flag: unknown flag %d", flag);
    }
    if (previous) *previous = old;
    return SMK_OK;
}

int smk_tune_count(int32_t pass) { return variant_count(pass); }

int smk_tune_info(int32_t pass, int32_t v, int32_t* w, int32_t* t, int32_t* nmax) {
    const TileVariant* tab = variant_table(pass);
    if (!tab || v < 0 || v >= variant_count(pass)) return fail(SMK_EINVAL, "smk_tune_info: bad pass or variant");
    if (w) *w = tab[v].w;
    if (t) *t = tab[v].t;
    if (nmax) *nmax = tab[v].nmax;
    return SMK_OK;
}

int smk_tune_set(int32_t pass, int32_t n, int32_t v) {
    const TileVariant* tab = variant_table(pass);
    if (!tab || n < 2 || n > FFT_MAX_N) return fail(SMK_EINVAL, "smk_tune_set: bad pass or length");
    if (v >= variant_count(pass) || (v >= 0 && !variant_fits(tab[v], n)))
        return fail(SMK_EINVAL, "smk_tune_set: variant %d cannot run length %d", v, n);
    g_choice[pass][length_class(n)].store(v < 0 ? -1 : v);
    return SMK_OK;
}

int smk_tune_get(int32_t pass, int32_t n) {
    if (!variant_table(pass) || n < 2 || n > FFT_MAX_N) return fail(SMK_EINVAL, "smk_tune_get: bad pass or length");
    return variant_for(pass, n);
}

}  // extern "C"
