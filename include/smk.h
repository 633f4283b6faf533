/*
 * smk.h -- C ABI of the GB300 (sm_103a) SaclayMocks hot-path library (libsmk.so).
 *
 * The reference (igmhub/SaclayMocks) is pure Python; its "operator API" for this path is
 * a set of functions, scripts and file formats, not an FFI.  Each entry point below states
 * which reference interface it replaces (file:line inside igmhub/SaclayMocks).
 *
 * Conventions
 *  - Every buffer argument is a DEVICE pointer owned by the caller (e.g. a torch tensor's
 *    data_ptr()); the library never allocates device memory.  Scratch memory is the
 *    caller's ``workspace`` sized by the matching *_workspace_size() query.
 *  - Work is enqueued on ``stream`` (a cudaStream_t, NULL = legacy default stream) and is
 *    stream-ordered: results are ready when the stream is synchronised.  One host thread
 *    per stream; calls on different streams may run concurrently unless they share
 *    buffers or a workspace.
 *  - Every function returns SMK_OK (0) or a negative SMK_E* code; it never calls exit,
 *    abort or __trap.  smk_strerror() names a code, smk_last_error() gives the message of
 *    the last failure on the calling host thread.
 *  - Boxes are C-ordered [batch][nx][ny][pitch] float32 arrays, with the z row padded to
 *    ``pitch = smk_grf_pitch(nz)`` floats (>= 2*(nz/2+1), a multiple of 8): the layout of
 *    an in-place real<->half-complex transform.  Cell (x,y,z) of box b is element
 *    ((b*nx + x)*ny + y)*pitch + z, z < nz.
 */
#ifndef SMK_H
#define SMK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define SMK_OK 0
#define SMK_EINVAL (-1)     /* invalid argument (null pointer, size, mode)          */
#define SMK_ENOTSUPP (-2)   /* size not handled by the kernels (see smk_fft_supported) */
#define SMK_ECUDA (-3)      /* a CUDA runtime call or kernel launch failed            */
#define SMK_EWORKSPACE (-4) /* workspace missing or smaller than the size query       */
#define SMK_ENULLBOX (-5)   /* produced box is all zero or holds non-finite values    */

/* Name of a status code (static string). */
const char* smk_strerror(int status);
/* Message of the last failure on this host thread ("" if none). */
const char* smk_last_error(void);
/* Library version as 10000*major + 100*minor + patch. */
int smk_version(void);
/* 1 if a line FFT of length n runs on the kernels (2 <= n <= 4096, n = 2^a 3^b 5^c). */
int smk_fft_supported(int32_t n);

/* ---------------------------------------------------------------- GRF boxes (make_boxes) */
#define SMK_NOISE_HOST 0   /* white noise given by the caller (dense [batch][nx][ny][nz])  */
#define SMK_NOISE_PHILOX 1 /* Fourier modes of white noise drawn on the GPU (Philox4x32-10 */
                           /* + Box-Muller, Hermitian planes kz = 0, nz/2): same statistics */
                           /* as the r2c of N(0,1) noise, two HBM passes fewer              */

#define SMK_PK_ANALYTIC 0  /* P(k) = amp * k / (1 + (k/k0)^2)^2, evaluated in the kernel   */
#define SMK_PK_GRID 1      /* sqrt(P/Vcell) read from a float32 [nx][ny][nz/2+1] grid       */

#define SMK_ETA_ZZ 0 /* eta components k_i k_j / k^2 delta_k (bin/make_boxes.py:315-391) */
#define SMK_ETA_XX 1
#define SMK_ETA_YY 2
#define SMK_ETA_XY 3
#define SMK_ETA_XZ 4
#define SMK_ETA_YZ 5
#define SMK_ETA_VX 6 /* velocity components -i k_i / k^2 * vel_factor * delta_k           */
#define SMK_ETA_VY 7 /* (bin/make_boxes.py:393-431; vel_factor = H0 * dD/dz at z = 0)     */
#define SMK_ETA_VZ 8

typedef struct {
    int32_t nx, ny, nz;   /* cells; nz even; every axis passes smk_fft_supported            */
    int32_t batch;        /* independent boxes in one launch (>= 1)                          */
    double dcell;         /* cell size, Mpc/h                                                */
    int32_t pk_mode;      /* SMK_PK_ANALYTIC or SMK_PK_GRID                                  */
    double k0;            /* break scale of the analytic spectrum, h/Mpc                     */
    double amp;           /* amplitude A of the analytic spectrum; <= 0: A such that         */
                          /* E[var delta] = 1, computed on the device in FP64                */
    const float* pk_grid; /* SMK_PK_GRID: device sqrt(P/Vcell) grid (shared by the batch)    */
    int32_t noise_mode;   /* SMK_NOISE_HOST or SMK_NOISE_PHILOX                              */
    const float* noise;   /* SMK_NOISE_HOST: device dense noise [batch][nx][ny][nz]          */
    uint64_t seed;        /* SMK_NOISE_PHILOX: box b uses key seed + b                       */
    int32_t want_eta;     /* 1: also produce eta_zz = irfftn(kz^2/k^2 delta_k)               */
    void* const* pass_events; /* optional cudaEvent_t[6]: recorded on the stream before the    */
    int32_t n_pass_events;    /* first HBM pass and after each of the five (0: none)          */
    int32_t eta_comp;     /* SMK_ETA_*: which eta_ij or velocity the eta box holds (0 = zz)  */
    double vel_factor;    /* SMK_ETA_VX/VY/VZ: H0 * dD/dz(z = 0) (km/s/(Mpc/h) per unit z)    */
    int32_t xi_chunk_kz;  /* > 0 runs the x pass into a blocked intermediate in the workspace */
                          /* (both fields from one launch, each GPU-noise mode drawn once, the */
                          /* rows of a tile ny x 16..64 bytes apart instead of ny x pitch x 4) */
                          /* that the y pass reads as contiguous runs, xi_chunk_kz k_z columns */
                          /* at a time (rounded up to 16); 0: the x pass writes the boxes in   */
                          /* place.  The boxes are the same, bit for bit.                      */
} SmkGrfParams;

/* Row pitch (floats) of the padded box layout for a z extent nz. */
int64_t smk_grf_pitch(int32_t nz);
/* Floats of one padded output box array (all batch members). */
int64_t smk_grf_box_floats(const SmkGrfParams* p);
/* Workspace bytes smk_grf_boxes needs: 256 (the FP64 normalisation accumulator), plus, with
 * xi_chunk_kz > 0, the intermediate of one chunk: fields (2 with eta, else 1) x batch x nx x
 * ny x min(roundup(xi_chunk_kz, 16), roundup(nz/2+1, 16)) complex floats. */
size_t smk_grf_workspace_size(const SmkGrfParams* p);

/*
 * Replaces bin/make_boxes.py DrawGRF_boxk (:40-72), the P0 multiply (:288-292),
 * FFTandStore's c2r + normalisation + sigma + null check (:77-105) and the eta_zz box
 * (:299-306, :341-352).  delta (and eta when want_eta) are padded output boxes; the
 * forward r2c runs in place in delta.  stats (device, may be NULL; 8*batch doubles,
 * zeroed by the call) receives for box b and field f (0 = delta, 1 = eta_zz):
 * stats[8b+4f+0] = sum, [8b+4f+1] = sum of squares, [8b+4f+2] = count of non-finite
 * cells, [8b+4f+3] = 0 (FP64); the caller derives sigma and the null check
 * (smk_grf_check does it on the host from one 4-double record).  delta, eta and the workspace
 * must be 16-byte aligned (the passes move 16-byte vectors); SMK_EINVAL otherwise.
 */
int smk_grf_boxes(const SmkGrfParams* p, float* delta, float* eta, double* stats,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Host-side check of a stats record (copied to host): SMK_ENULLBOX if the box is all
 * zero or holds non-finite cells (bin/make_boxes.py:100-105), else SMK_OK; sigma_out
 * (may be NULL) gets the standard deviation of the box (bin/make_boxes.py:92). */
int smk_grf_check(const double* stats_host, int64_t ncells, double* sigma_out);

/* Normalisation A with E[var delta] = 1 for the analytic spectrum (FP64 sum over the
 * half spectrum); enqueues on stream and writes *amp_dev (a device double). */
int smk_pk_normalisation(int32_t nx, int32_t ny, int32_t nz, double dcell, double k0,
                         double* amp_dev, void* stream);

/* Tile variants of the HBM passes (autotuner hooks; no counterpart in the reference).  Each
 * pass has a table of variants (tile width W and threads per block T, valid up to a line
 * length); smk_tune_set picks the variant used for the lengths of n's class (<=512, <=1024,
 * <=2560, <=4096; v = -1 restores the built-in choice).  Process-wide setting.  The built-in
 * choice is a variant compiled for exactly n if there is one, else the first variant whose
 * length covers n; for SMK_PASS_ZFWD and SMK_PASS_ZINV the first such variant with W = 0 (one
 * warp per row pair, as many warps per block as fit, up to T/32). */
#define SMK_PASS_ZFWD 0  /* r2c along z (host noise)                              */
#define SMK_PASS_LINE 1  /* c2c along y                                            */
#define SMK_PASS_XPASS 2 /* x pass of host noise                                   */
#define SMK_PASS_XGEN 3  /* x pass drawing the GPU noise                           */
#define SMK_PASS_ZINV 4  /* c2r along z + statistics                               */
int smk_tune_count(int32_t pass);
/* n_max < 0: the variant runs the length -n_max only (its FFT plan fixed at compile time). */
int smk_tune_info(int32_t pass, int32_t variant, int32_t* w, int32_t* threads, int32_t* n_max);
int smk_tune_set(int32_t pass, int32_t n, int32_t variant);
int smk_tune_get(int32_t pass, int32_t n);
/* Process-wide switches of smk_grf_boxes (no reference counterpart; tuning knobs of this
 * library).  The previous value goes to *previous (if not null).
 *   SMK_TUNE_XGEN_SPLIT: GPU-noise x pass writing delta and eta in one launch (0), in two
 *     launches of one field each (1), or by footprint (-1, default: two launches when the
 *     delta + eta boxes span more than 64 GiB, where one launch's spread of rows outruns
 *     address translation);
 *   SMK_TUNE_PREFETCH: the x (host noise, into the intermediate), y and z passes pull their
 *     next tile into L2 while transforming the current one (1, default) or not (0). */
#define SMK_TUNE_XGEN_SPLIT 0
#define SMK_TUNE_PREFETCH 1
#define SMK_TUNE_TMA 3  /* y pass tiles loaded by TMA tensor copies (1, default), loaded and */
                        /* stored by TMA tensor copies (2), or loaded by cp.async (0)         */
/* Failure test of the y pass's bounded TMA waits (0 by default): 1 makes every tile's barrier
 * expect 16 bytes more than its copies deliver, with a ~10 ms limit, so each wait runs out; the
 * pass then writes NaN and smk_grf_check reports SMK_ENULLBOX.  Nothing faults or hangs. */
#define SMK_TUNE_TMA_WAIT_TEST 4
/* Resident blocks per SM of smk_skewers_flux's persistent launch: 0 (default) as many as fit,
 * k in 1..32 at most k (the skewer autotuner's knob). */
#define SMK_TUNE_SKEWER_BLOCKS 5
int smk_tune_flag(int32_t flag, int32_t value, int32_t* previous);

/* ---------------------------------------------------------------- skewers (make_spectra +
 *                                                                   merge_spectra) */
#define SMK_INTERP_TRILINEAR 0 /* 8-corner read, periodic, cell centres at (i+0.5)dcell */
#define SMK_INTERP_PIXELS 1    /* no box read: delta_l, eta_par, z given per pixel      */
                               /* (the merge_spectra input, bin/merge_spectra.py:282-300) */
#define SMK_INTERP_GAUSS343 2  /* the reference's read: Gaussian weights over the 7^3   */
                               /* cells around the pixel ((2 dmax + 1)^3 with gauss_dmax), */
                               /* eta_par = r_i r_j eta_ij / r^2                          */
                               /* from six eta boxes (bin/make_spectra.py:39-139)         */

#define SMK_SS_NONE 0     /* no small-scale field                                      */
#define SMK_SS_HOST 1     /* white noise given per skewer (length nz_s)                 */
#define SMK_SS_PHILOX 2   /* Gaussian modes drawn on the GPU in Fourier space            */

#define SMK_ABC_CONST 0    /* a, b, c constants                                        */
#define SMK_ABC_POWERLAW 1 /* a(z) = a * ((1+z)/a_zref1)^a_power, b, c constants        */
#define SMK_ABC_TABLE 2    /* a, b, c linear in z on a uniform table [z_tab0, +dz_tab)  */

#define SMK_G_ONE 0        /* growth G = 1                                             */
#define SMK_G_MERGE 1      /* G(z) = growth24 * (1+2.4) / (1+z)                        */

typedef struct {
    int64_t n;             /* number of skewers                                         */
    const float* start;    /* [n][3] first pixel, box-corner frame, Mpc/h (or start64)   */
    const float* dir;      /* [n][3] unit direction (or dir64)                           */
    const int32_t* npix;   /* [n] pixels                                                 */
    const int64_t* offset; /* [n] index of the skewer's first pixel in the packed outputs */
    double dpix;           /* pixel spacing along the skewer, Mpc/h (at most 64 cells)   */
    const int32_t* order;  /* [n_slots] schedule from smk_skewer_schedule (device)       */
    int64_t n_slots;       /* 2 * work items                                             */
    const float* pix_delta;/* SMK_INTERP_PIXELS: packed delta_l per pixel                */
    const float* pix_eta;  /* SMK_INTERP_PIXELS: packed eta_par per pixel (NULL: no RSD)  */
    const float* pix_z;    /* SMK_INTERP_PIXELS: packed redshift per pixel               */
    const int32_t* forest; /* [n][2] Lya-forest pixel range [f0, f1) of each skewer, or     */
                           /* NULL (every pixel).  A skewer with an empty range gets no     */
                           /* small-scale field (bin/merge_spectra.py:305-306, 327-330)      */
    const double* start64; /* optional [n][3] FP64 start points; when given, start is unused */
    const double* dir64;   /* optional [n][3] FP64 unit directions; when given, dir is unused */
} SmkSkewers;

typedef struct {
    /* boxes */
    int32_t nx, ny, nz;
    int64_t pitch;         /* floats between consecutive (x,y) rows of the boxes          */
    double dcell;
    int32_t interp;        /* SMK_INTERP_TRILINEAR / PIXELS / GAUSS343                    */
    const float* eta6[6];  /* GAUSS343: eta_xx, yy, zz, xy, xz, yz boxes (all or none)     */
    double obs[3];         /* GAUSS343: observer position, box-corner frame, Mpc/h         */
    /* small scales (bin/merge_spectra.py:303-331) */
    int32_t ss_mode;       /* SMK_SS_NONE / SMK_SS_HOST / SMK_SS_PHILOX                   */
    int32_t ss_nz;         /* FFT length (power of two 256..4096) or 0: 256*2^n >= npix+50 */
    const float* ss_scale; /* sqrt(P1Dmiss(k)/pixsize) for nz = 256<<j, j = 0..4, table j  */
                           /* (nz/2+1 floats) at offset sum_{i<j} ((256<<i)/2+1)           */
    const float* ss_noise; /* SMK_SS_HOST: noise of skewer s at ss_noise_offset[s]          */
    const int64_t* ss_noise_offset;
    uint64_t seed;         /* SMK_SS_PHILOX                                               */
    /* FGPA (util.fgpa, py/SaclayMocks/util.py:421-433) */
    int32_t abc_mode;
    float a, b, c;
    float a_zref1, a_power;
    const float* abc_tab;  /* SMK_ABC_TABLE: [n_tab][3] (a,b,c)                            */
    int32_t n_tab;
    float z_tab0, dz_tab;
    float z_lo, z_hi;      /* redshift mapped linearly along x: z = z_lo + (z_hi-z_lo) x/Lx */
    int32_t growth_mode;   /* SMK_G_ONE / SMK_G_MERGE                                     */
    float growth24;        /* fgrowth(2.4) for SMK_G_MERGE                                */
    /* redshift-dependent P1Dmiss (util.InterpP1Dmissing, py/SaclayMocks/util.py:448-474, as
     * bin/merge_spectra.py:116-118, 305-325 use it without --fit-p1d): with ss_nztab > 0,
     * ss_scale holds ss_nztab table sets of SMK_SS_SET_FLOATS floats (set j: the five nz
     * classes above for redshift ss_ztab[j]); each skewer takes the set whose redshift is
     * nearest to zeff = mean redshift of its forest pixels, and, with ss_zsigma, its delta_s
     * is multiplied pixel by pixel by sigma_s(z)/sigma_s(zeff) (linear in z on ss_ztab,
     * clamped at the ends).  ss_nztab = 0: one set (the layout above).                       */
    int32_t ss_nztab;
    const float* ss_ztab;   /* [ss_nztab] ascending redshifts (device)                     */
    const float* ss_zsigma; /* [ss_nztab] sigma_s at ss_ztab (device), or NULL            */
    int32_t gauss_dmax;     /* GAUSS343: half-width of the Gaussian read in cells, 1..4 (the */
                            /* reference's -dmax); 0 means 3 (the 7^3 read)                 */
} SmkSpectraParams;
#define SMK_SS_SET_FLOATS 3973 /* sum over nz = 256<<j, j = 0..4, of nz/2+1 */

/* Host: build the work schedule of smk_skewers_flux from the host copy of npix (each 0..2^24).  Skewers
 * are grouped by small-scale FFT length, longest first, in pairs of equal length (one
 * complex FFT carries two skewers); order_out must hold 2*n + 16 ints, n_slots_out gets
 * the used length (even; empty slots are -1).  ss_nz is SmkSpectraParams.ss_nz: 0 applies
 * the rule nz = 256*2^k >= npix + 50 (SMK_ENOTSUPP beyond 4096), a fixed nz must be
 * >= every npix (SMK_EINVAL otherwise); a negative ss_nz (small-scale field off) pairs
 * skewers by length only. */
int smk_skewer_schedule(int64_t n, const int32_t* npix_host, int32_t ss_nz, int32_t* order_out,
                        int64_t* n_slots_out);

/* Workspace bytes smk_skewers_flux needs (the persistent launch's work counter). */
size_t smk_skewers_workspace_size(const SmkSkewers* sk, const SmkSpectraParams* p);

/*
 * Replaces bin/make_spectra.py ReadSpec (:90-139, trilinear read instead of the Gaussian
 * 7^3 read) + the small-scale loop and FGPA of bin/merge_spectra.py (:303-339).  For every
 * pixel: delta_l, eta_par by trilinear read of the boxes (eta may be NULL: no RSD) or, with
 * SMK_INTERP_PIXELS, from the per-pixel arrays of the skewer table (boxes unused, may be
 * NULL; the redshift is then pix_z instead of the z_lo..z_hi map along x);
 * delta = delta_l + delta_s, F = exp(-a exp(b G (delta + c eta_par))).  flux receives F
 * in the packed layout; delta_out / eta_out / z_out (may be NULL) receive delta_l+delta_s,
 * eta_par and the redshift of each pixel.
 */
int smk_skewers_flux(const SmkSkewers* sk, const SmkSpectraParams* p, const float* delta_box,
                     const float* eta_box, float* flux, float* delta_out, float* eta_out,
                     float* z_out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Allocation-free form of smk_skewers_flux, for callers that cannot allocate device memory
 * (code that runs where cudaMalloc is not allowed, e.g. inside a host framework that owns all
 * device memory, or a program that must not allocate after start-up).  No counterpart in the
 * reference, which runs on the CPU.  Same inputs and outputs as smk_skewers_flux except that
 * the work schedule is built here from the host copy of npix (sk->order and sk->n_slots are
 * ignored) and all scratch (schedule + work counter) lives in a static device array of
 * 4 MiB + 256 B that every process loading the library holds on each GPU it uses until exit:
 * at most SMK_STATIC_MAX_SLOTS - 16 skewers (1,048,560; the schedule has at most n + 6 slots);
 * larger tables are rejected with SMK_EINVAL.  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  Calls share the
 * array: calls that overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  No device memory is allocated or freed.
 */
#define SMK_STATIC_MAX_SLOTS (1 << 20)
#define SMK_STATIC_MAX_DEVICES 64
int smk_skewers_flux_static(const SmkSkewers* sk, const int32_t* npix_host, const SmkSpectraParams* p,
                            const float* delta_box, const float* eta_box, float* flux,
                            float* delta_out, float* eta_out, float* z_out, void* stream);

/* ---------------------------------------------------------------- the (a,b,c) fit */
/*
 * Replaces the objective of fit_az.Fitter (py/SaclayMocks/fit_az.py:194-279: FGPA on stored
 * delta_l + delta_s, eta_par, growth -> <F> -> dF = F/<F> - 1 -> binned P1D -> chi2) with the
 * per-redshift-bin loss L = sum_j (<F>_j - Fbar*_j)^2 + sum_b ((P_b - P*_b)/P*_b)^2 and its
 * exact gradient, so Migrad's finite differences become one adjoint pass.  The reductions run
 * on the GPU (FP64 accumulators); the loss itself is assembled on the host from them.
 * Pixels are recomputed from the fields in every pass, never stored (only, optionally, the
 * forward pass's spectra, for the backward).
 */
typedef struct {
    const float* delta;     /* [n_total] delta_l + delta_s                                */
    const float* eta;       /* [n_total] eta_par, or NULL                                 */
    const float* G;         /* [n_total] growth, or NULL (G = 1)                          */
    const int16_t* zbin;    /* [n_total] redshift bin of each pixel, 0..nzb-1             */
    const int64_t* offset;  /* [n] first pixel of each skewer                             */
    const int32_t* npix;    /* [n] pixels (1..2048)                                       */
    const int32_t* order;   /* [n_slots] pairs of equal length, smk_fit_schedule (device) */
    int64_t n_slots;
    int64_t n_total;
    int32_t nzb, nkb;       /* redshift bins, log-k bins (1..64 each)                     */
    const double* kedges;   /* [nkb+1] k bin edges, h/Mpc (device)                        */
    double dx;              /* pixel size, Mpc/h                                          */
    const float* chirp;     /* optional (with chirp_off): smk_fit_chirps' table of the chirp */
                            /* spectra and chirps of the problem's lengths (one transform of */
                            /* the three of each Bluestein DFT saved), or NULL              */
    const int64_t* chirp_off; /* [2049]: offset (complex elements) of length N's spectrum in */
                              /* chirp, or -1 (then computed in the kernel)                    */
    int32_t n_max;          /* largest npix of the problem (sizes the kernels' shared memory */
                            /* to its Bluestein length); 0: up to 2048                      */
    float* spectrum;        /* optional [2 n_total] (8-byte aligned): smk_fit_forward stores  */
                            /* the packed DFT of every pair of skewers there (N complex at  */
                            /* the pair's first offset) and smk_fit_backward reads it back   */
                            /* instead of transforming the pair again, so the backward must */
                            /* follow a forward with the same theta; NULL: recomputed        */
} SmkFitProblem;

/* Cyclic convolution length of the Bluestein DFT of a length-n skewer: the smallest
 * 2^a 3^b 5^c >= 2n - 1 (0 outside 1..2048).  No counterpart in the reference. */
int smk_fit_bluestein_m(int32_t n);
/* Chirp tables of the Bluestein DFTs (they depend on the skewer lengths only, not on theta):
 * for i < n_lengths, out[2*offsets[i] .. 2*(offsets[i] + M_i + N_i)) receives the complex FFT_M
 * of the length-N_i chirp (N_i = lengths[i], M_i = smk_fit_bluestein_m(N_i)) followed by the
 * chirp w_n = exp(-i pi n^2 / N_i) itself for n < N_i (device arrays, offsets in complex
 * elements).  SmkFitProblem.chirp_off[N] = offsets[i] for N = lengths[i], -1 for lengths
 * without an entry.  No counterpart in the reference. */
int smk_fit_chirps(int32_t n_lengths, const int32_t* lengths, const int64_t* offsets, float* out,
                   void* stream);
/* Host: pairs of equal-length skewers for the fit kernels (order_out: 2n + 16 ints). */
int smk_fit_schedule(int64_t n, const int32_t* npix_host, int32_t* order_out, int64_t* n_slots_out);
/* Length (doubles) of the accumulator array: [nzb] sum F per z bin, [1] sum F,
 * [nkb] sum P per k bin (P = |X|^2 dx/N of one skewer mode), [nzb][3] A, [nzb][3] B, [1] S,
 * [nkb] sum P^2 per k bin (for the rms / sqrt(n) errors of util.MakeProfileHisto). */
int smk_fit_acc_len(int32_t nzb, int32_t nkb);
/* Forward: zeroes acc, fills sum F per z bin, sum F, P1D power sums and squared-power sums
 * per k bin.
 * theta: device [nzb][3] (a, b, c).  Workspace: 256 bytes. */
int smk_fit_forward(const SmkFitProblem* fp, const float* theta, double* acc, void* workspace,
                    size_t workspace_bytes, void* stream);
/* Backward (after smk_fit_forward on the same acc): with gM_j = dL/d<F>_j / n_j and
 * gP_b = dL/dP_b / count_b (device), fills A_j = sum (gM_j + gdF/<F>) dF/dtheta_j,
 * B_j = sum dF/dtheta_j, S = sum gdF F; the gradient is A_j - S B_j / (n_total <F>^2). */
int smk_fit_backward(const SmkFitProblem* fp, const float* theta, double* acc, const double* gM,
                     const double* gP, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------- FGPA (util.fgpa) */
/*
 * Replaces util.fgpa (py/SaclayMocks/util.py:421-433) as called from
 * bin/merge_spectra.py:337 and fit_az.py:251: flux[i] = exp(-a exp(b G (delta + c eta))).
 * eta may be NULL (no RSD: bin/merge_spectra.py:339).  Each of G, a, b, c is a per-element
 * device array, or NULL to use the scalar that follows it.
 */
int smk_fgpa(int64_t n, const float* delta, const float* eta, const float* G, float G0,
             const float* a, float a0, const float* b, float b0, const float* c, float c0,
             float* flux, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SMK_H */
