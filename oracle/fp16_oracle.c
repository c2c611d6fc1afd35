/*
 * fp16_oracle.c -- CPU restatement of the FP16-storage form of the time step.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only the tests load it; the product
 * path never links or calls it.
 *
 * The scheme is the FP32 path of fdtd_oracle.c (the reference shader's order,
 * core/wavey-solver/src/fdtd.wgsl:44-119, with the host packing of
 * core/wavey-solver/src/gpu_fdtd.rs:67-88) with the fields stored as FP16
 * times a power of two per (z slab, time level), shared by the V right-hand
 * sides of one source chunk:
 *
 *   - a value of slab z at time level k is stored as half(p * 2^-E) and read
 *     back as float(h) * 2^E, E = E^k[z] (both scalings are exact);
 *   - before the step that writes level n+1, E^(n+1)[z] = max(e - shift, -60)
 *     where M < 2^e, M = 8 * max of the slab maxima of levels n and n-1 over
 *     slabs z-1..z+1, plus the largest |signal[n] * sum |tap weights|| over
 *     the chunk's lanes (M = 0 gives -60);
 *   - the slab maximum of level n+1 is the largest |p^(n+1)| (FP32, after
 *     injection) stored in the slab over all lanes;
 *   - a stored value beyond 65504 after scaling is an error, not a
 *     saturation; rounding to FP16 is to nearest, ties to even, with FP16
 *     subnormals;
 *   - branch states stay FP32; receivers sample float(h) * 2^E of level n
 *     before the update; injection is added to the updated value before it
 *     is rounded and stored (the tap weights of a cell merged per source in
 *     FP64, every lane of a tap cell adding signal * its weight, 0 where its
 *     source has no tap there).
 *
 * Levels 0 and -1 are zero fields whose scales are never needed.  Compile
 * with -ffp-contract=off (oracle/build.py).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define F16_NO_BOUNDARY 0xFFFFFFFFu
#define F16_AIR 64u
#define F16_COURANT 0.5773502691896257
#define F16_E_FLOOR (-60)
#define F16_MAX 65504.0f

/* RNE rounding of f to the nearest FP16 value (normal or subnormal), as a
 * float.  |f| <= 65504 (larger values are range errors before this). */
static float half_round(float f) {
    if (f == 0.0f) return f;
    int e;
    frexpf(fabsf(f), &e);       /* |f| in [2^(e-1), 2^e) */
    int q = e - 11;             /* spacing of FP16 values in that binade: 2^(e-1-10) */
    if (q < -24) q = -24;       /* FP16 subnormal spacing */
    const float r = nearbyintf(ldexpf(f, -q));  /* exact scaling; rounds to nearest even */
    return ldexpf(r, q);
}

/* The slab exponent of level k (k >= 1) from the maxima of levels k-1, k-2. */
static int slab_exponent(const float *amax, int64_t nz, int64_t k, int64_t z, float inj, int shift) {
    float m = 0.0f;
    const int64_t z0 = z > 0 ? z - 1 : 0, z1 = z + 1 < nz ? z + 1 : nz - 1;
    for (int64_t zz = z0; zz <= z1; zz++) {
        const float a = k - 1 >= 0 ? amax[((k - 1) % 3) * nz + zz] : 0.0f;
        const float b = k - 2 >= 0 ? amax[((k - 2) % 3) * nz + zz] : 0.0f;
        m = fmaxf(m, fmaxf(a, b));
    }
    m = 8.0f * m + inj;
    if (m == 0.0f) return F16_E_FLOOR;
    int e;
    frexpf(m, &e);
    return e - shift > F16_E_FLOOR ? e - shift : F16_E_FLOOR;
}

/*
 * One chunk of `lanes` right-hand sides (lanes = the chunk width V: 1, 2 or
 * 4; a lane without taps is a padding lane).  Taps of lane l are
 * tap_cell/tap_w[tap_start[l] .. tap_start[l+1]); signals [lanes][steps].
 * ir: [lanes][n_recv][steps] receiver time series.  Returns 0, 2 when a value
 * left the FP16 range of its slab scale, -1 when memory ran out.
 */
int wo_run_f16(int64_t nx, int64_t ny, int64_t nz, double dt,
               const uint8_t *flags, const uint32_t *bidx,
               int64_t n_boundary, const uint32_t *bstart, const double *slots,
               int64_t lanes, const int64_t *tap_start, const int64_t *tap_cell, const double *tap_w,
               const double *signals, int64_t steps,
               const int64_t *recv, int64_t n_recv, double *ir, int shift) {
    const size_t cells = (size_t)(nx * ny * nz);
    const ptrdiff_t sx = (ptrdiff_t)nx, sxy = (ptrdiff_t)(nx * ny);
    const size_t L = (size_t)lanes;
    const float l2 = (float)(F16_COURANT * F16_COURANT), lam = (float)F16_COURANT, dtf = (float)dt;
    const size_t nslots = n_boundary > 0 ? bstart[n_boundary] : 0;
    float *p = calloc(cells * L, sizeof(float));      /* stored FP16 values of level n, unscaled */
    float *prev = calloc(cells * L, sizeof(float));   /* level n-1, then n+1 */
    float *sl32 = malloc(sizeof(float) * 4 * (nslots + 1));
    float *st_u = calloc((nslots + 1) * L, sizeof(float));
    float *st_g = calloc((nslots + 1) * L, sizeof(float));
    float *scale = calloc(3 * (size_t)nz, sizeof(float));  /* 2^E of levels mod 3 */
    float *inv = calloc(3 * (size_t)nz, sizeof(float));    /* 2^-E */
    float *amax = calloc(3 * (size_t)nz, sizeof(float));   /* slab maxima of levels mod 3 */
    float *sig = malloc(sizeof(float) * (L * (size_t)steps + 1));
    float *wsum = calloc(L, sizeof(float));
    const int64_t n_taps = tap_start[lanes];
    int64_t *rcell = malloc(sizeof(int64_t) * (size_t)(n_taps + 1));     /* tap rows: distinct cells */
    double *rw = calloc((size_t)(n_taps + 1) * L, sizeof(double));        /* [row][lane] merged weight */
    float *rwf = malloc(sizeof(float) * (size_t)(n_taps + 1) * L);
    int32_t *row_of = malloc(sizeof(int32_t) * cells);
    if (!p || !prev || !sl32 || !st_u || !st_g || !scale || !inv || !amax || !sig || !wsum || !rcell || !rw || !rwf ||
        !row_of) {
        free(p); free(prev); free(sl32); free(st_u); free(st_g); free(scale); free(inv); free(amax); free(sig);
        free(wsum); free(rcell); free(rw); free(rwf); free(row_of);
        return -1;
    }
    for (size_t j = 0; j < 4 * nslots; j++) sl32[j] = (float)slots[j];
    for (size_t j = 0; j < L * (size_t)steps; j++) sig[j] = (float)signals[j];
    for (size_t i = 0; i < cells; i++) row_of[i] = -1;
    int64_t nrows = 0;
    for (size_t l = 0; l < L; l++) {
        double acc = 0.0;
        for (int64_t t = tap_start[l]; t < tap_start[l + 1]; t++) {
            const int64_t c = tap_cell[t];
            if (row_of[c] < 0) { row_of[c] = (int32_t)nrows; rcell[nrows] = c; nrows++; }
            rw[(size_t)row_of[c] * L + l] += tap_w[t];
            acc += fabs(tap_w[t]);
        }
        wsum[l] = (float)(acc * (1.0 + 1e-6));
    }
    for (size_t j = 0; j < (size_t)nrows * L; j++) rwf[j] = (float)rw[j];

    int err = 0;
    for (int64_t n = 0; n < steps; n++) {
        const int64_t cur = n % 3, old = (n + 2) % 3, nxt = (n + 1) % 3;
        /* Scales of level n+1 and a cleared maxima slot for it. */
        float inj = 0.0f;
        for (size_t l = 0; l < L; l++) inj = fmaxf(inj, fabsf(sig[l * (size_t)steps + (size_t)n]) * wsum[l]);
        for (int64_t z = 0; z < nz; z++) {
            const int e = slab_exponent(amax, nz, n + 1, z, inj, shift);
            scale[nxt * nz + z] = ldexpf(1.0f, e);
            inv[nxt * nz + z] = ldexpf(1.0f, -e);
        }
        for (int64_t z = 0; z < nz; z++) amax[nxt * nz + z] = 0.0f;
        /* Receivers: level n before the update. */
        for (size_t l = 0; l < L; l++)
            for (int64_t r = 0; r < n_recv; r++) {
                const int64_t c = recv[r];
                ir[(l * (size_t)n_recv + (size_t)r) * (size_t)steps + (size_t)n] =
                    (double)(p[(size_t)c * L + l] * scale[cur * nz + c / sxy]);
            }
        for (int64_t z = 0; z < nz; z++) {
            const float sm = z > 0 ? scale[cur * nz + z - 1] : 0.0f, sc = scale[cur * nz + z],
                        sp = z + 1 < nz ? scale[cur * nz + z + 1] : 0.0f, so = scale[old * nz + z],
                        si = inv[nxt * nz + z];
            float mx = 0.0f;
            for (ptrdiff_t k = 0; k < sxy; k++) {
                const size_t i = (size_t)(z * sxy + k);
                const uint8_t m = flags[i];
                if (!(m & F16_AIR)) continue;
                const uint32_t b = bidx[i];
                const int32_t row = row_of[i];
                for (size_t l = 0; l < L; l++) {
                    float sum = 0.0f, kk = 0.0f;
                    if (m & 1u) { sum = sum + p[(i - 1) * L + l] * sc; kk = kk + 1.0f; }
                    if (m & 2u) { sum = sum + p[(i + 1) * L + l] * sc; kk = kk + 1.0f; }
                    if (m & 4u) { sum = sum + p[(i - sx) * L + l] * sc; kk = kk + 1.0f; }
                    if (m & 8u) { sum = sum + p[(i + sx) * L + l] * sc; kk = kk + 1.0f; }
                    if (m & 16u) { sum = sum + p[(i - sxy) * L + l] * sm; kk = kk + 1.0f; }
                    if (m & 32u) { sum = sum + p[(i + sxy) * L + l] * sp; kk = kk + 1.0f; }
                    const float pc = p[i * L + l] * sc, pp = prev[i * L + l] * so;
                    const float lap = l2 * (sum - kk * pc);
                    float next;
                    if (b == F16_NO_BOUNDARY) {
                        next = 2.0f * pc - pp + lap;
                    } else {
                        float s1 = 0.0f, s2 = 0.0f;
                        for (uint32_t j = bstart[b]; j < bstart[b + 1]; j++) {
                            const float *q = sl32 + 4 * (size_t)j;
                            const float u = st_u[j * L + l], g = st_g[j * L + l];
                            const float e = (q[1] * u - q[2] * g + 0.5f * pc + q[3] * pp) * q[0];
                            s1 = s1 + (0.5f - q[3]) * q[0];
                            s2 = s2 + e - u;
                        }
                        next = (2.0f * pc - pp + lap - lam * s2) / (1.0f + lam * s1);
                        for (uint32_t j = bstart[b]; j < bstart[b + 1]; j++) {
                            const float *q = sl32 + 4 * (size_t)j;
                            const float u = st_u[j * L + l], g = st_g[j * L + l];
                            const float e = (q[1] * u - q[2] * g + 0.5f * pc + q[3] * pp) * q[0];
                            const float un = (0.5f - q[3]) * q[0] * next + e;
                            st_g[j * L + l] = g + 0.5f * dtf * (un + u);
                            st_u[j * L + l] = un;
                        }
                    }
                    if (row >= 0) next = next + sig[l * (size_t)steps + (size_t)n] * rwf[(size_t)row * L + l];
                    const float s = next * si;
                    if (!(fabsf(s) <= F16_MAX)) err = 1;
                    prev[i * L + l] = err ? 0.0f : half_round(s);
                    mx = fmaxf(mx, fabsf(next));
                }
            }
            amax[nxt * nz + z] = mx;
        }
        float *tmp = p; p = prev; prev = tmp;
        if (err) break;
    }
    free(p); free(prev); free(sl32); free(st_u); free(st_g); free(scale); free(inv); free(amax); free(sig);
    free(wsum); free(rcell); free(rw); free(rwf); free(row_of);
    return err ? 2 : 0;
}
