// ir_analysis.cuh -- ISO 3382-1 band parameters of receiver time series on
// the device (core/wavey-solver/src/analysis.rs), for IR-mode runs: the time
// series stay in HBM and only six numbers per receiver and band come back.
//
// One thread per (time series, band), FP64 throughout, every step in the
// reference's order:
//   running sum of p (optional: the response to the source pulse's integral,
//   core/wavey-cli/examples/bras_wave.rs:46-52), broadband onset
//   (analysis.rs:185-189), octave band-pass of six biquads run forward and
//   backward (analysis.rs:143-183), squared from the onset, Lundeby
//   truncation and noise compensation (analysis.rs:191-251, optional), then
//   Schroeder integration, EDT / T20 / T30 by regression (analysis.rs:266-279),
//   C80, D50 and centre time (analysis.rs:300-325).
// The band-passed series lives in a scratch buffer laid out [sample][thread]
// so that a warp's accesses to one sample are contiguous.
#pragma once
#include <cstdint>

#include "fdtd_kernels.cuh"

namespace wk {

constexpr int IR_INTEGRATE = 1;
constexpr int IR_LUNDEBY = 2;
constexpr double IR_PI = 3.14159265358979323846;

struct IrBiquad {
    double b0, b1, b2, a1, a2;
};

// Rust `x as usize` for the indices the analysis derives from times.
__device__ __forceinline__ long long ir_index(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 9.2e18) return 0x7fffffffffffffffLL;
    return (long long)x;
}

__device__ __forceinline__ double ir_db(double v) { return 10.0 * log10(v > 1e-300 ? v : 1e-300); }

__device__ void ir_sections(double fc, double fs, IrBiquad s[6]) {
    const double lo = fc / sqrt(2.0);
    const double hi = fmin(fc * sqrt(2.0), 0.45 * fs);
    const double qs[3] = {0.517638, 0.707107, 1.931852};
    for (int k = 0; k < 3; k++) {
        double w = 2.0 * IR_PI * lo / fs, c = cos(w), alpha = sin(w) / (2.0 * qs[k]), a0 = 1.0 + alpha;
        s[2 * k] = {(1.0 + c) / 2.0 / a0, -(1.0 + c) / a0, (1.0 + c) / 2.0 / a0, -2.0 * c / a0, (1.0 - alpha) / a0};
        w = 2.0 * IR_PI * hi / fs;
        c = cos(w);
        alpha = sin(w) / (2.0 * qs[k]);
        a0 = 1.0 + alpha;
        s[2 * k + 1] = {(1.0 - c) / 2.0 / a0, (1.0 - c) / a0, (1.0 - c) / 2.0 / a0, -2.0 * c / a0, (1.0 - alpha) / a0};
    }
}

// Direct form I with states (x1, x2, y1, y2), the reference's operation order.
__device__ __forceinline__ double ir_biquad(const IrBiquad &q, double v, double st[4]) {
    double y = __dadd_rn(__dmul_rn(q.b0, v), __dmul_rn(q.b1, st[0]));
    y = __dadd_rn(y, __dmul_rn(q.b2, st[1]));
    y = __dsub_rn(y, __dmul_rn(q.a1, st[2]));
    y = __dsub_rn(y, __dmul_rn(q.a2, st[3]));
    st[1] = st[0];
    st[0] = v;
    st[3] = st[2];
    st[2] = y;
    return y;
}

// Least-squares line through n points given by a functor (x_k, y_k).
template <class P>
__device__ void ir_linreg(long long n, P pt, double &slope, double &icpt) {
    double sx = 0.0, sy = 0.0;
    for (long long k = 0; k < n; k++) {
        double x, y;
        pt(k, x, y);
        sx = __dadd_rn(sx, x);
        sy = __dadd_rn(sy, y);
    }
    const double mx = __ddiv_rn(sx, (double)n), my = __ddiv_rn(sy, (double)n);
    double sxy = 0.0, sxx = 0.0;
    for (long long k = 0; k < n; k++) {
        double x, y;
        pt(k, x, y);
        sxy = __dadd_rn(sxy, __dmul_rn(__dsub_rn(x, mx), __dsub_rn(y, my)));
        sxx = __dadd_rn(sxx, __dmul_rn(__dsub_rn(x, mx), __dsub_rn(x, mx)));
    }
    slope = sxx > 0.0 ? __ddiv_rn(sxy, sxx) : 0.0;
    icpt = __dsub_rn(my, __dmul_rn(slope, mx));
}

// The series of this thread: element i at y[i * stride].
struct IrSeries {
    double *y;
    long long stride;
    __device__ __forceinline__ double &operator[](long long i) const { return y[i * stride]; }
};

__device__ double ir_block_mean(const IrSeries &e, long long n, long long win, long long b) {
    const long long a0 = b * win, a1 = min(a0 + win, n);
    double s = 0.0;
    for (long long i = a0; i < a1; i++) s = __dadd_rn(s, e[i]);
    return __ddiv_rn(s, (double)(a1 - a0));
}

__device__ double ir_noise_from(const IrSeries &e, long long n, long long start) {
    const long long s0 = min(start, n - 1);
    double s = 0.0;
    for (long long i = s0; i < n; i++) s = __dadd_rn(s, e[i]);
    const double m = __ddiv_rn(s, (double)max(n - s0, 1LL));
    return m > 1e-300 ? m : 1e-300;
}

// analysis.rs:191-251: (end, compensation energy) of a squared band series.
__device__ void ir_lundeby(const IrSeries &e, long long n, double fs, long long &end, double &comp) {
    if (n < 100) {
        end = n;
        comp = 0.0;
        return;
    }
    const long long win = max(ir_index(0.01 * fs), 1LL);
    const long long nb = (n + win - 1) / win;
    auto t_of = [&](long long b) { return (double)(b * win + win / 2) / fs; };
    double noise = ir_noise_from(e, n, n * 9 / 10);
    long long cross = n;
    for (int it = 0; it < 5; it++) {
        long long peak_b = 0;
        double peak = ir_block_mean(e, n, win, 0);
        for (long long b = 1; b < nb; b++) {
            const double v = ir_block_mean(e, n, win, b);
            if (v >= peak) {
                peak = v;
                peak_b = b;
            }
        }
        const double lim = ir_db(noise) + 5.0;
        long long end_b = nb - 1;
        for (long long b = peak_b; b < nb; b++)
            if (ir_db(ir_block_mean(e, n, win, b)) < lim) {
                end_b = b;
                break;
            }
        if (end_b <= peak_b + 2) break;
        double slope, icpt;
        ir_linreg(end_b - peak_b, [&](long long k, double &x, double &y) {
            x = t_of(peak_b + k);
            y = ir_db(ir_block_mean(e, n, win, peak_b + k));
        }, slope, icpt);
        if (slope >= 0.0) break;
        const double tc = (ir_db(noise) - icpt) / slope;
        const long long new_cross = min(max(ir_index(tc * fs), 1LL), n);
        const double t_noise = tc + 10.0 / -slope;
        const long long start = min(ir_index(t_noise * fs), n * 9 / 10);
        noise = ir_noise_from(e, n, start);
        const long long d = new_cross - cross;
        if ((d < 0 ? -d : d) < (long long)(0.001 * fs)) {
            cross = new_cross;
            break;
        }
        cross = new_cross;
    }
    const long long back = ir_index(0.1 * fs);
    const long long tail_from = cross > back ? cross - back : 0;
    const long long b0 = tail_from / win, b1 = cross / win;
    comp = 0.0;
    if (b1 - b0 > 2) {
        double slope, icpt;
        ir_linreg(b1 - b0, [&](long long k, double &x, double &y) {
            x = t_of(b0 + k);
            y = ir_db(ir_block_mean(e, n, win, min(b0 + k, nb - 1)));
        }, slope, icpt);
        if (slope < 0.0) {
            const double k = -slope * log(10.0) / 10.0;
            const double e_cross = pow(10.0, (icpt + slope * (double)cross / fs) / 10.0);
            comp = e_cross / k * fs;
        }
    }
    end = max(cross, 1LL);
}

// analysis.rs:266-279 over the Schroeder curve held as energies edc[i]
// (dB taken on the fly against total).
__device__ double ir_decay_time(const IrSeries &edc, long long n, double total, double fs, double from, double to) {
    auto db = [&](long long i) {
        const double r = edc[i] / total;
        return 10.0 * log10(r > 1e-300 ? r : 1e-300);
    };
    long long a = -1, b = -1;
    for (long long i = 0; i < n && a < 0; i++)
        if (db(i) <= from) a = i;
    for (long long i = 0; i < n && b < 0; i++)
        if (db(i) <= to) b = i;
    if (a < 0 || b < 0 || b <= a + 2) return nan("");
    const long long step = max((b - a) / 400, 1LL);
    const long long np = (b - a + step - 1) / step;
    double slope, icpt;
    ir_linreg(np, [&](long long k, double &x, double &y) {
        const long long i = a + k * step;
        x = (double)i / fs;
        y = db(i);
    }, slope, icpt);
    return slope < 0.0 ? -60.0 / slope : nan("");
}

// One (series, band) per thread.  series[s * steps + t] (T = float or
// double), onset[s] from ir_onsets, scratch [steps][threads of this launch],
// out[(s * n_bands + band) * 6 + k] = edt, t20, t30, c80, d50, ts.
template <class T>
__global__ void __launch_bounds__(128) ir_band_params(const T *series, long long steps, const long long *onset,
                                                      long long first_series, long long n_series, const double *bands,
                                                      int n_bands, double fs, int flags, double *scratch,
                                                      double *out) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long threads = n_series * n_bands;
    if (tid >= threads) return;
    const long long s = first_series + tid / n_bands;
    const int band = (int)(tid % n_bands);
    const T *p = series + s * steps;
    IrSeries y{scratch + tid, threads};
    IrBiquad sec[6];
    ir_sections(bands[band], fs, sec);
    // Band-pass forward, then backward (zero phase).
    {
        double st[6][4] = {};
        double acc = 0.0;
        for (long long t = 0; t < steps; t++) {
            acc = __dadd_rn(acc, (double)p[t]);
            double v = (flags & IR_INTEGRATE) ? acc : (double)p[t];
#pragma unroll
            for (int k = 0; k < 6; k++) v = ir_biquad(sec[k], v, st[k]);
            y[t] = v;
        }
    }
    {
        double st[6][4] = {};
        for (long long t = steps - 1; t >= 0; t--) {
            double v = y[t];
#pragma unroll
            for (int k = 0; k < 6; k++) v = ir_biquad(sec[k], v, st[k]);
            y[t] = v;
        }
    }
    // Squared from the onset, in place.
    const long long t0 = onset[s];
    const long long ne = steps - t0;
    for (long long i = 0; i < ne; i++) {
        const double v = y[t0 + i];
        y[i] = __dmul_rn(v, v);
    }
    long long n = ne;
    double comp = 0.0;
    if (flags & IR_LUNDEBY) {
        long long end;
        ir_lundeby(y, ne, fs, end, comp);
        n = min(end, ne);
    }
    // Energy sums, then the Schroeder curve in place.
    double all = 0.0, e50 = 0.0, e80 = 0.0, ts = 0.0;
    const long long i50 = min(ir_index(0.05 * fs), n), i80 = min(ir_index(0.08 * fs), n);
    for (long long i = 0; i < n; i++) {
        const double v = y[i];
        all = __dadd_rn(all, v);
        if (i < i50) e50 = __dadd_rn(e50, v);
        if (i < i80) e80 = __dadd_rn(e80, v);
        ts = __dadd_rn(ts, __dmul_rn(__ddiv_rn((double)i, fs), v));
    }
    all = __dadd_rn(all, comp);
    double acc = comp;
    for (long long i = n - 1; i >= 0; i--) {
        acc = __dadd_rn(acc, y[i]);
        y[i] = acc;
    }
    double total = n > 0 ? y[0] : 0.0;
    if (!(total > 1e-300)) total = 1e-300;
    const double all_c = all > 1e-300 ? all : 1e-300;
    const double late = all - e80 > 1e-300 ? all - e80 : 1e-300;
    double *o = out + (s * n_bands + band) * 6;
    o[0] = ir_decay_time(y, n, total, fs, -0.0 - 1e-9, -10.0);
    o[1] = ir_decay_time(y, n, total, fs, -5.0, -25.0);
    o[2] = ir_decay_time(y, n, total, fs, -5.0, -35.0);
    o[3] = 10.0 * log10(e80 / late);
    o[4] = e50 / all_c;
    o[5] = ts / all_c;
}

// The broadband onset of every series (analysis.rs:185-189), of its running
// sum when IR_INTEGRATE is set.  One thread per series.
template <class T>
__global__ void __launch_bounds__(128) ir_onsets(const T *series, long long steps, long long n_series, int flags,
                                                 long long *onset) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_series) return;
    const T *p = series + s * steps;
    double peak = 0.0, acc = 0.0;
    for (long long t = 0; t < steps; t++) {
        acc = __dadd_rn(acc, (double)p[t]);
        const double v = (flags & IR_INTEGRATE) ? acc : (double)p[t];
        peak = fmax(peak, __dmul_rn(v, v));
    }
    long long at = 0;
    acc = 0.0;
    for (long long t = 0; t < steps; t++) {
        acc = __dadd_rn(acc, (double)p[t]);
        const double v = (flags & IR_INTEGRATE) ? acc : (double)p[t];
        if (__dmul_rn(v, v) >= __dmul_rn(peak, 0.01)) {
            at = t;
            break;
        }
    }
    onset[s] = at;
}

}  // namespace wk
