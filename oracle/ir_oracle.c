/* ir_oracle.c -- CPU restatement of the reference's impulse-response
 * analysis (core/wavey-solver/src/analysis.rs) for the band parameters of
 * simulated receiver time series.  Test infrastructure only: the checker of
 * the device kernels, never the product path.
 *
 *   octave sections      analysis.rs:143-168  (6th-order Butterworth Qs, HP at fc/sqrt2, LP at min(fc sqrt2, 0.45 fs))
 *   biquad (DF I)        analysis.rs:124-141
 *   octave_filter        analysis.rs:170-183  (forward, then backward: zero phase)
 *   onset                analysis.rs:185-189  (first sample within 20 dB of the peak)
 *   lundeby              analysis.rs:191-251
 *   linreg               analysis.rs:253-264
 *   decay_time           analysis.rs:266-279
 *   params_from          analysis.rs:300-325  (Schroeder integration, EDT, T20, T30, C80, D50, Ts)
 *   running sum of p     core/wavey-cli/examples/bras_wave.rs:46-52 (response to the pulse's integral)
 *
 * Sums run left to right in FP64 as Rust's Iterator::sum does; Rust's
 * saturating float-to-integer casts are spelled out (to_index).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PI_ 3.14159265358979323846

typedef struct {
    double b[3], a[3];
} biquad;

/* Rust `x as usize`: NaN and negatives to 0, saturating above. */
static int64_t to_index(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 9.2e18) return INT64_MAX;
    return (int64_t)x;
}

static void sections(double fc, double fs, biquad s[6]) {
    const double lo = fc / sqrt(2.0);
    double hi = fc * sqrt(2.0);
    if (0.45 * fs < hi) hi = 0.45 * fs;
    const double qs[3] = {0.517638, 0.707107, 1.931852};
    for (int k = 0; k < 3; k++) {
        double w = 2.0 * PI_ * lo / fs, c = cos(w), sn = sin(w), alpha = sn / (2.0 * qs[k]), a0 = 1.0 + alpha;
        biquad *h = &s[2 * k];
        h->b[0] = (1.0 + c) / 2.0 / a0;
        h->b[1] = -(1.0 + c) / a0;
        h->b[2] = (1.0 + c) / 2.0 / a0;
        h->a[0] = 1.0;
        h->a[1] = -2.0 * c / a0;
        h->a[2] = (1.0 - alpha) / a0;
        w = 2.0 * PI_ * hi / fs;
        c = cos(w);
        sn = sin(w);
        alpha = sn / (2.0 * qs[k]);
        a0 = 1.0 + alpha;
        biquad *l = &s[2 * k + 1];
        l->b[0] = (1.0 - c) / 2.0 / a0;
        l->b[1] = (1.0 - c) / a0;
        l->b[2] = (1.0 - c) / 2.0 / a0;
        l->a[0] = 1.0;
        l->a[1] = -2.0 * c / a0;
        l->a[2] = (1.0 - alpha) / a0;
    }
}

static void run_section(const biquad *s, double *x, int64_t n, int backward) {
    double x1 = 0.0, x2 = 0.0, y1 = 0.0, y2 = 0.0;
    for (int64_t k = 0; k < n; k++) {
        double *v = backward ? &x[n - 1 - k] : &x[k];
        const double y = s->b[0] * *v + s->b[1] * x1 + s->b[2] * x2 - s->a[1] * y1 - s->a[2] * y2;
        x2 = x1;
        x1 = *v;
        y2 = y1;
        y1 = y;
        *v = y;
    }
}

void wo_octave_filter(double *x, int64_t n, double fc, double fs) {
    biquad s[6];
    sections(fc, fs, s);
    for (int k = 0; k < 6; k++) run_section(&s[k], x, n, 0);
    for (int k = 0; k < 6; k++) run_section(&s[k], x, n, 1);
}

int64_t wo_onset(const double *x, int64_t n) {
    double peak = 0.0;
    for (int64_t i = 0; i < n; i++) peak = fmax(peak, x[i] * x[i]);
    for (int64_t i = 0; i < n; i++)
        if (x[i] * x[i] >= peak * 0.01) return i;
    return 0;
}

static void linreg(const double *px, const double *py, int64_t n, double *slope, double *icpt) {
    double sx = 0.0, sy = 0.0;
    for (int64_t i = 0; i < n; i++) {
        sx += px[i];
        sy += py[i];
    }
    const double mx = sx / (double)n, my = sy / (double)n;
    double sxy = 0.0, sxx = 0.0;
    for (int64_t i = 0; i < n; i++) {
        sxy += (px[i] - mx) * (py[i] - my);
        sxx += (px[i] - mx) * (px[i] - mx);
    }
    *slope = sxx > 0.0 ? sxy / sxx : 0.0;
    *icpt = my - *slope * mx;
}

static double db10(double v) { return 10.0 * log10(v > 1e-300 ? v : 1e-300); }

static double noise_from(const double *e, int64_t n, int64_t start) {
    const int64_t s = start < n - 1 ? start : n - 1;
    double sum = 0.0;
    for (int64_t i = s; i < n; i++) sum += e[i];
    const int64_t len = n - s > 1 ? n - s : 1;
    const double m = sum / (double)len;
    return m > 1e-300 ? m : 1e-300;
}

void wo_lundeby(const double *e, int64_t n, double fs, int64_t *end, double *comp) {
    if (n < 100) {
        *end = n;
        *comp = 0.0;
        return;
    }
    int64_t win = to_index(0.01 * fs);
    if (win < 1) win = 1;
    const int64_t nb = (n + win - 1) / win;
    double *blocks = malloc(sizeof(double) * nb), *px = malloc(sizeof(double) * nb), *py = malloc(sizeof(double) * nb);
    for (int64_t b = 0; b < nb; b++) {
        const int64_t a0 = b * win, a1 = a0 + win < n ? a0 + win : n;
        double s = 0.0;
        for (int64_t i = a0; i < a1; i++) s += e[i];
        blocks[b] = s / (double)(a1 - a0);
    }
#define T_OF(b) ((double)((b) * win + win / 2) / fs)
    double noise = noise_from(e, n, n * 9 / 10);
    int64_t cross = n;
    for (int it = 0; it < 5; it++) {
        int64_t peak_b = 0;
        for (int64_t b = 0; b < nb; b++)
            if (blocks[b] >= blocks[peak_b]) peak_b = b;  // max_by: the last of equal maxima
        const double lim = db10(noise) + 5.0;
        int64_t end_b = nb - 1;
        for (int64_t b = peak_b; b < nb; b++)
            if (db10(blocks[b]) < lim) {
                end_b = b;
                break;
            }
        if (end_b <= peak_b + 2) break;
        const int64_t np = end_b - peak_b;
        for (int64_t k = 0; k < np; k++) {
            px[k] = T_OF(peak_b + k);
            py[k] = db10(blocks[peak_b + k]);
        }
        double slope, icpt;
        linreg(px, py, np, &slope, &icpt);
        if (slope >= 0.0) break;
        const double tc = (db10(noise) - icpt) / slope;
        int64_t new_cross = to_index(tc * fs);
        if (new_cross < 1) new_cross = 1;
        if (new_cross > n) new_cross = n;
        const double t_noise = tc + 10.0 / -slope;
        int64_t start = to_index(t_noise * fs);
        if (start > n * 9 / 10) start = n * 9 / 10;
        noise = noise_from(e, n, start);
        const int64_t d = new_cross - cross;
        if ((d < 0 ? -d : d) < (int64_t)(0.001 * fs)) {
            cross = new_cross;
            break;
        }
        cross = new_cross;
    }
    const int64_t back = to_index(0.1 * fs);
    const int64_t tail_from = cross > back ? cross - back : 0;
    const int64_t b0 = tail_from / win, b1 = cross / win;
    double c = 0.0;
    if (b1 - b0 > 2) {
        for (int64_t b = b0; b < b1; b++) {
            px[b - b0] = T_OF(b);
            py[b - b0] = db10(blocks[b < nb - 1 ? b : nb - 1]);
        }
        double slope, icpt;
        linreg(px, py, b1 - b0, &slope, &icpt);
        if (slope < 0.0) {
            const double k = -slope * log(10.0) / 10.0;  // energy decay rate (1/s)
            const double e_cross = pow(10.0, (icpt + slope * (double)cross / fs) / 10.0);
            c = e_cross / k * fs;
        }
    }
#undef T_OF
    free(blocks);
    free(px);
    free(py);
    *end = cross > 1 ? cross : 1;
    *comp = c;
}

static double decay_time(const double *edc_db, int64_t n, double fs, double from, double to) {
    int64_t a = -1, b = -1;
    for (int64_t i = 0; i < n && a < 0; i++)
        if (edc_db[i] <= from) a = i;
    for (int64_t i = 0; i < n && b < 0; i++)
        if (edc_db[i] <= to) b = i;
    if (a < 0 || b < 0 || b <= a + 2) return NAN;
    int64_t step = (b - a) / 400;
    if (step < 1) step = 1;
    const int64_t np = (b - a + step - 1) / step;
    double *px = malloc(sizeof(double) * np), *py = malloc(sizeof(double) * np);
    for (int64_t k = 0; k < np; k++) {
        const int64_t i = a + k * step;
        px[k] = (double)i / fs;
        py[k] = edc_db[i];
    }
    double slope, icpt;
    linreg(px, py, np, &slope, &icpt);
    free(px);
    free(py);
    return slope < 0.0 ? -60.0 / slope : NAN;
}

/* out: edt, t20, t30, c80, d50, ts */
void wo_params_from(const double *e, int64_t n, double comp, double fs, double out[6]) {
    double *edc = malloc(sizeof(double) * (n > 0 ? n : 1));
    double acc = comp;
    for (int64_t i = n - 1; i >= 0; i--) {
        acc += e[i];
        edc[i] = acc;
    }
    double total = n > 0 ? edc[0] : 0.0;
    if (!(total > 1e-300)) total = 1e-300;  // f64::max(x, 1e-300)
    for (int64_t i = 0; i < n; i++) {
        const double r = edc[i] / total;
        edc[i] = 10.0 * log10(r > 1e-300 ? r : 1e-300);
    }
    double all = 0.0;
    for (int64_t i = 0; i < n; i++) all += e[i];
    all += comp;
    int64_t i50 = to_index(0.05 * fs), i80 = to_index(0.08 * fs);
    if (i50 > n) i50 = n;
    if (i80 > n) i80 = n;
    double e50 = 0.0, e80 = 0.0, ts = 0.0;
    for (int64_t i = 0; i < i50; i++) e50 += e[i];
    for (int64_t i = 0; i < i80; i++) e80 += e[i];
    for (int64_t i = 0; i < n; i++) ts += (double)i / fs * e[i];
    const double all_c = all > 1e-300 ? all : 1e-300;
    const double late = all - e80 > 1e-300 ? all - e80 : 1e-300;
    out[0] = decay_time(edc, n, fs, -0.0 - 1e-9, -10.0);
    out[1] = decay_time(edc, n, fs, -5.0, -25.0);
    out[2] = decay_time(edc, n, fs, -5.0, -35.0);
    out[3] = 10.0 * log10(e80 / late);
    out[4] = e50 / all_c;
    out[5] = ts / all_c;
    free(edc);
}

/* One receiver's time series p[0..n) sampled at fs: optionally its running
 * sum (integrate), the broadband onset, then per band the octave-filtered
 * series squared from the onset and its parameters, with Lundeby's
 * truncation and compensation (lundeby) or over the whole series.
 * out: [n_bands][6]. */
void wo_ir_params(const double *p, int64_t n, double fs, const double *bands, int n_bands, int integrate, int lundeby,
                  double *out) {
    double *h = malloc(sizeof(double) * (n > 0 ? n : 1)), *y = malloc(sizeof(double) * (n > 0 ? n : 1));
    double acc = 0.0;
    for (int64_t i = 0; i < n; i++) {
        acc += p[i];
        h[i] = integrate ? acc : p[i];
    }
    const int64_t t0 = wo_onset(h, n);
    for (int b = 0; b < n_bands; b++) {
        memcpy(y, h, sizeof(double) * n);
        wo_octave_filter(y, n, bands[b], fs);
        const int64_t ne = n - t0;
        for (int64_t i = 0; i < ne; i++) y[i] = y[t0 + i] * y[t0 + i];
        int64_t end = ne;
        double comp = 0.0;
        if (lundeby) wo_lundeby(y, ne, fs, &end, &comp);
        wo_params_from(y, end < ne ? end : ne, comp, fs, out + 6 * b);
    }
    free(h);
    free(y);
}
