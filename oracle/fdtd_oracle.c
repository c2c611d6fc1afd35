/*
 * fdtd_oracle.c -- CPU restatement of wavey-solver's FDTD run loop.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  This file is the checker for the
 * CUDA path: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  The product path (wavey_gb300, libwavey_cuda.so) never
 * links or calls it.
 *
 * Two entry points:
 *
 *   wo_run_f64  -- restates `fdtd::run_cpu_with` (core/wavey-solver/src/
 *                  fdtd.rs:644-725) in FP64: record p^n at the receivers
 *                  (running DFT, fdtd.rs:673-683, optional time series,
 *                  fdtd.rs:628-641), bulk leapfrog update of plain air cells
 *                  in place into `prev` (fdtd.rs:684-708), the joint boundary
 *                  solve `boundary_update` (fdtd.rs:580-598) for nodes with
 *                  admittance slots, then injection of the source taps in
 *                  the given order (fdtd.rs:718-720) and the buffer swap.
 *
 *   wo_run_f32  -- the same scheme in FP32 with the operation order of the
 *                  reference's GPU shader (core/wavey-solver/src/fdtd.wgsl:
 *                  44-119) and host packing (core/wavey-solver/src/
 *                  gpu_fdtd.rs:67-88): taps merged per cell in FP64 then
 *                  rounded, slot constants rounded to f32, l2 and lambda
 *                  rounded from FP64.  It must be compiled without
 *                  floating-point contraction (-ffp-contract=off) so that
 *                  every product and sum rounds separately; the CUDA kernels
 *                  use explicitly rounded intrinsics in the same order, which
 *                  makes receiver time series bit-identical.
 *
 * Grid arrays follow `FdtdGrid` (fdtd.rs:196-209): flags (bit 6 air, bits
 * 0-5 air neighbour -x,+x,-y,+y,-z,+z), bidx per cell (0xFFFFFFFF = none),
 * and the slot table in CSR form (bstart per boundary node, slots as
 * (inv_d, cv, k, w) quadruples, fdtd.rs:178-187).  Linear cell index
 * (z*ny + y)*nx + x (fdtd.rs:227-229).
 *
 * DFT: acc[r*nf + f] += p^n * exp(-j 2 pi frac(f*dt*n)) for n = 0..steps-1
 * (fdtd.rs:679-682).  The reference accumulates serially; here the (r, f)
 * pairs are split over threads, each pair still summed in step order, so
 * the result is the same.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define WO_NO_BOUNDARY 0xFFFFFFFFu
#define WO_AIR 64u
/* fdtd.rs:138 */
#define WO_COURANT 0.5773502691896257
#define WO_TWO_PI 6.283185307179586

static void set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

int wo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static double now_seconds(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
#endif
}

/* Seconds spent in the time-step loop of the last wo_run_f64 call, after the
 * fields were allocated and first touched (for timing the CPU baseline
 * without its set-up). */
static double g_last_loop_seconds = 0.0;
double wo_last_loop_seconds(void) { return g_last_loop_seconds; }

/* -------------------------------------------------------------------------
 * FP64: fdtd.rs:644-725
 * ------------------------------------------------------------------------- */

/* fdtd.rs:685-696: laplacian over air neighbours, l2*(sum - k*p). */
static inline double lap64(const double *p, uint8_t f, size_t i, ptrdiff_t nx, ptrdiff_t nxy, double l2) {
    const ptrdiff_t offs[6] = {-1, 1, -nx, nx, -nxy, nxy};
    double sum = 0.0, kair = 0.0;
    for (int d = 0; d < 6; d++) {
        if (f & (1u << d)) {
            sum += p[(ptrdiff_t)i + offs[d]];
            kair += 1.0;
        }
    }
    return l2 * (sum - kair * p[i]);
}

/* One receiver sample into the running DFT (fdtd.rs:679-682). */
static void record64(const double *p, const int64_t *recv, size_t n_recv, const double *freqs, size_t nf,
                     double dt, size_t n, double *acc, double *ir, size_t steps) {
    const size_t pairs = n_recv * nf;
#pragma omp parallel for schedule(static) if (pairs > 4096)
    for (size_t q = 0; q < pairs; q++) {
        size_t ri = q / nf, fi = q % nf;
        double v = p[recv[ri]];
        double x = freqs[fi] * dt * (double)n;
        double ph = -WO_TWO_PI * (x - trunc(x));
        acc[2 * q] += v * cos(ph);
        acc[2 * q + 1] += v * sin(ph);
    }
    if (ir)
        for (size_t ri = 0; ri < n_recv; ri++) ir[ri * steps + n] = p[recv[ri]];
}

int wo_run_f64(int64_t nx, int64_t ny, int64_t nz, double dt,
               const uint8_t *flags, const uint32_t *bidx,
               int64_t n_boundary, const uint32_t *bcell, const uint32_t *bstart, const double *slots,
               const int64_t *tap_cell, const double *tap_w, int64_t n_taps,
               const double *signal, int64_t steps,
               const int64_t *recv, int64_t n_recv,
               const double *freqs, int64_t nf,
               double *out, double *ir, int threads) {
    set_threads(threads);
    const size_t cells = (size_t)(nx * ny * nz);
    const ptrdiff_t sx = (ptrdiff_t)nx, sxy = (ptrdiff_t)(nx * ny);
    const double l2 = WO_COURANT * WO_COURANT, lam = WO_COURANT;
    double *p = calloc(cells, sizeof(double));
    double *prev = calloc(cells, sizeof(double));
    size_t nslots = n_boundary > 0 ? bstart[n_boundary] : 0;
    double *st_u = calloc(nslots + 1, sizeof(double));
    double *st_g = calloc(nslots + 1, sizeof(double));
    double *bnext = calloc((size_t)n_boundary + 1, sizeof(double));
    if (!p || !prev || !st_u || !st_g || !bnext) {
        free(p); free(prev); free(st_u); free(st_g); free(bnext);
        return -1;
    }
    memset(out, 0, sizeof(double) * 2 * (size_t)(n_recv * nf));
    /* First touch of both fields by the threads that update them (the loop's
     * static z-slab schedule), before the timed loop. */
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++) {
        memset(p + (size_t)(z * sxy), 0, sizeof(double) * (size_t)sxy);
        memset(prev + (size_t)(z * sxy), 0, sizeof(double) * (size_t)sxy);
    }
    const double t_loop = now_seconds();
    for (int64_t n = 0; n < steps; n++) {
        record64(p, recv, (size_t)n_recv, freqs, (size_t)nf, dt, (size_t)n, out, ir, (size_t)steps);
        /* fdtd.rs:699-708: z-slabs in parallel, plain air only. */
#pragma omp parallel for schedule(static)
        for (int64_t z = 0; z < nz; z++) {
            size_t base = (size_t)(z * sxy);
            for (ptrdiff_t k = 0; k < sxy; k++) {
                size_t i = base + (size_t)k;
                uint8_t f = flags[i];
                if (!(f & WO_AIR) || bidx[i] != WO_NO_BOUNDARY) continue;
                prev[i] = 2.0 * p[i] - prev[i] + lap64(p, f, i, sx, sxy, l2);
            }
        }
        /* fdtd.rs:710-716 and boundary_update (fdtd.rs:580-598). */
#pragma omp parallel for schedule(static)
        for (int64_t b = 0; b < n_boundary; b++) {
            size_t i = bcell[b];
            double pc = p[i], pp = prev[i];
            double lap = lap64(p, flags[i], i, sx, sxy, l2);
            double s1 = 0.0, s2 = 0.0;
            for (uint32_t j = bstart[b]; j < bstart[b + 1]; j++) {
                const double *sl = slots + 4 * (size_t)j;
                double e = (sl[1] * st_u[j] - sl[2] * st_g[j] + 0.5 * pc + sl[3] * pp) * sl[0];
                s1 += (0.5 - sl[3]) * sl[0];
                s2 += e - st_u[j];
            }
            double next = (2.0 * pc - pp + lap - lam * s2) / (1.0 + lam * s1);
            for (uint32_t j = bstart[b]; j < bstart[b + 1]; j++) {
                const double *sl = slots + 4 * (size_t)j;
                double e = (sl[1] * st_u[j] - sl[2] * st_g[j] + 0.5 * pc + sl[3] * pp) * sl[0];
                double u = (0.5 - sl[3]) * sl[0] * next + e;
                st_g[j] += 0.5 * dt * (u + st_u[j]);
                st_u[j] = u;
            }
            bnext[b] = next;
        }
        for (int64_t b = 0; b < n_boundary; b++) prev[bcell[b]] = bnext[b];
        /* fdtd.rs:718-720: taps in the given order, not merged. */
        for (int64_t t = 0; t < n_taps; t++) prev[tap_cell[t]] += tap_w[t] * signal[n];
        double *tmp = p; p = prev; prev = tmp;
    }
    g_last_loop_seconds = now_seconds() - t_loop;
    free(p); free(prev); free(st_u); free(st_g); free(bnext);
    return 0;
}

/* -------------------------------------------------------------------------
 * FP32 in the shader's order: fdtd.wgsl:44-119, gpu_fdtd.rs:67-88
 * ------------------------------------------------------------------------- */

int wo_run_f32(int64_t nx, int64_t ny, int64_t nz, double dt,
               const uint8_t *flags, const uint32_t *bidx,
               int64_t n_boundary, const uint32_t *bcell, const uint32_t *bstart, const double *slots,
               const int64_t *tap_cell, const double *tap_w, int64_t n_taps,
               const double *signal, int64_t steps,
               const int64_t *recv, int64_t n_recv,
               const double *freqs, int64_t nf,
               double *out, double *ir, int threads) {
    set_threads(threads);
    const size_t cells = (size_t)(nx * ny * nz);
    const ptrdiff_t sx = (ptrdiff_t)nx, sxy = (ptrdiff_t)(nx * ny);
    const float l2 = (float)(WO_COURANT * WO_COURANT), lam = (float)WO_COURANT, dtf = (float)dt;
    float *p = calloc(cells, sizeof(float));
    float *prev = calloc(cells, sizeof(float));
    size_t nslots = n_boundary > 0 ? bstart[n_boundary] : 0;
    float *sl32 = malloc(sizeof(float) * 4 * (nslots + 1));
    float *st_u = calloc(nslots + 1, sizeof(float));
    float *st_g = calloc(nslots + 1, sizeof(float));
    /* gpu_fdtd.rs:67-75: one tap per cell, weights of a repeated cell summed in FP64. */
    int64_t *mcell = malloc(sizeof(int64_t) * (size_t)(n_taps + 1));
    double *mw = malloc(sizeof(double) * (size_t)(n_taps + 1));
    if (!p || !prev || !sl32 || !st_u || !st_g || !mcell || !mw) {
        free(p); free(prev); free(sl32); free(st_u); free(st_g); free(mcell); free(mw);
        return -1;
    }
    for (size_t j = 0; j < 4 * nslots; j++) sl32[j] = (float)slots[j];
    int64_t nm = 0;
    for (int64_t t = 0; t < n_taps; t++) {
        int64_t k = 0;
        while (k < nm && mcell[k] != tap_cell[t]) k++;
        if (k < nm) mw[k] += tap_w[t];
        else { mcell[nm] = tap_cell[t]; mw[nm] = tap_w[t]; nm++; }
    }
    memset(out, 0, sizeof(double) * 2 * (size_t)(n_recv * nf));
    for (int64_t n = 0; n < steps; n++) {
        /* The receiver samples go into the FP64 DFT exactly as in wo_run_f64. */
        const size_t pairs = (size_t)(n_recv * nf);
#pragma omp parallel for schedule(static) if (pairs > 4096)
        for (size_t q = 0; q < pairs; q++) {
            size_t ri = q / (size_t)nf, fi = q % (size_t)nf;
            double v = (double)p[recv[ri]];
            double x = freqs[fi] * dt * (double)n;
            double ph = -WO_TWO_PI * (x - trunc(x));
            out[2 * q] += v * cos(ph);
            out[2 * q + 1] += v * sin(ph);
        }
        if (ir)
            for (int64_t ri = 0; ri < n_recv; ri++) ir[ri * steps + n] = (double)p[recv[ri]];
        /* fdtd.wgsl:44-106, one cell at a time; every cell reads only p and
         * its own prev, so the loop order does not matter. */
#pragma omp parallel for schedule(static)
        for (int64_t z = 0; z < nz; z++) {
            size_t base = (size_t)(z * sxy);
            for (ptrdiff_t k = 0; k < sxy; k++) {
                size_t i = base + (size_t)k;
                uint8_t m = flags[i];
                if (!(m & WO_AIR)) continue;
                float sum = 0.0f, kk = 0.0f;
                if (m & 1u) { sum = sum + p[i - 1]; kk = kk + 1.0f; }
                if (m & 2u) { sum = sum + p[i + 1]; kk = kk + 1.0f; }
                if (m & 4u) { sum = sum + p[i - sx]; kk = kk + 1.0f; }
                if (m & 8u) { sum = sum + p[i + sx]; kk = kk + 1.0f; }
                if (m & 16u) { sum = sum + p[i - sxy]; kk = kk + 1.0f; }
                if (m & 32u) { sum = sum + p[i + sxy]; kk = kk + 1.0f; }
                float pc = p[i];
                float lap = l2 * (sum - kk * pc);
                uint32_t b = bidx[i];
                float next;
                if (b == WO_NO_BOUNDARY) {
                    next = 2.0f * pc - prev[i] + lap;
                } else {
                    float pp = prev[i];
                    float s1 = 0.0f, s2 = 0.0f;
                    for (uint32_t j = bstart[b]; j < bstart[b + 1]; j++) {
                        const float *sl = sl32 + 4 * (size_t)j;
                        float e = (sl[1] * st_u[j] - sl[2] * st_g[j] + 0.5f * pc + sl[3] * pp) * sl[0];
                        s1 = s1 + (0.5f - sl[3]) * sl[0];
                        s2 = s2 + e - st_u[j];
                    }
                    next = (2.0f * pc - pp + lap - lam * s2) / (1.0f + lam * s1);
                    for (uint32_t j = bstart[b]; j < bstart[b + 1]; j++) {
                        const float *sl = sl32 + 4 * (size_t)j;
                        float e = (sl[1] * st_u[j] - sl[2] * st_g[j] + 0.5f * pc + sl[3] * pp) * sl[0];
                        float u = (0.5f - sl[3]) * sl[0] * next + e;
                        st_g[j] = st_g[j] + 0.5f * dtf * (u + st_u[j]);
                        st_u[j] = u;
                    }
                }
                prev[i] = next;
            }
        }
        /* fdtd.wgsl:110-119 */
        float s = (float)signal[n];
        for (int64_t t = 0; t < nm; t++) prev[mcell[t]] = prev[mcell[t]] + s * (float)mw[t];
        float *tmp = p; p = prev; prev = tmp;
    }
    (void)n_boundary; (void)bcell;
    free(p); free(prev); free(sl32); free(st_u); free(st_g); free(mcell); free(mw);
    return 0;
}
