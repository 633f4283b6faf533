/* C restatement of the skewer stage for the CPU baseline and cross-checks -- TEST
 * INFRASTRUCTURE ONLY (the oracle; never linked into the product).
 *
 * Per pixel of every skewer: trilinear read of the padded delta / eta_par boxes (cell centres
 * at (i+0.5)*dcell, periodic; the read the configs ask for in place of the Gaussian 7^3 read
 * of bin/make_spectra.py:39-139), optional small-scale delta_s added (bin/merge_spectra.py:325),
 * FGPA F = exp(-a exp(b G (delta + c eta))) (py/SaclayMocks/util.py:421-433) with a(z) constant
 * or a0*((1+z)/zref1)^power and z mapped linearly along x.  float64 arithmetic, OpenMP over
 * skewers.
 */
#include <math.h>
#include <stdint.h>

static inline int64_t wrapi(int64_t c, int64_t n) {
    int64_t r = c % n;
    return r < 0 ? r + n : r;
}

static inline double tri(const float* box, int64_t ny, int64_t pitch, const int64_t c0[3],
                         const int64_t c1[3], const double f[3]) {
    double v = 0.0;
    for (int cx = 0; cx < 2; ++cx)
        for (int cy = 0; cy < 2; ++cy)
            for (int cz = 0; cz < 2; ++cz) {
                const double w = (cx ? f[0] : 1 - f[0]) * (cy ? f[1] : 1 - f[1]) * (cz ? f[2] : 1 - f[2]);
                const int64_t ix = cx ? c1[0] : c0[0], iy = cy ? c1[1] : c0[1], iz = cz ? c1[2] : c0[2];
                v += w * (double)box[(ix * ny + iy) * pitch + iz];
            }
    return v;
}

void oracle_skewer_flux(int64_t nsk, const float* start, const float* dir, const int32_t* npix,
                        const int64_t* offset, double dpix, const float* delta, const float* eta,
                        int32_t nx, int32_t ny, int32_t nz, int64_t pitch, double dcell,
                        const double* ds_packed, int32_t abc_mode, double a, double b, double c,
                        double zref1, double power, double z_lo, double z_hi, int32_t growth_mode,
                        double growth24, float* flux, int32_t nthreads) {
    const int64_t dims[3] = {nx, ny, nz};
    const double lx = nx * dcell;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int64_t s = 0; s < nsk; ++s) {
        for (int32_t i = 0; i < npix[s]; ++i) {
            int64_t c0[3], c1[3];
            double f[3], p[3];
            for (int d = 0; d < 3; ++d) {
                p[d] = (double)start[3 * s + d] + i * dpix * (double)dir[3 * s + d];
                const double u = p[d] / dcell - 0.5;
                const double fl = floor(u);
                f[d] = u - fl;
                c0[d] = wrapi((int64_t)fl, dims[d]);
                c1[d] = c0[d] + 1 == dims[d] ? 0 : c0[d] + 1;
            }
            const double dl = tri(delta, ny, pitch, c0, c1, f);
            const double et = eta ? tri(eta, ny, pitch, c0, c1, f) : 0.0;
            const int64_t o = offset[s] + i;
            const double ds = ds_packed ? ds_packed[o] : 0.0;
            double xw = fmod(p[0], lx);
            if (xw < 0) xw += lx;
            const double z = z_lo + (z_hi - z_lo) * xw / lx;
            const double pa = abc_mode == 1 ? a * pow((1 + z) / zref1, power) : a;
            const double G = growth_mode == 1 ? growth24 * 3.4 / (1 + z) : 1.0;
            flux[o] = (float)exp(-pa * exp(b * G * (dl + ds + c * et)));
        }
    }
}
