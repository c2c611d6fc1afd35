// signal.cpp -- source signal, frequency grid and the FP64 post-processing
// of receiver spectra.
//
// Restates:
//   source_signal         wavey-solver/src/fdtd.rs:601-610
//   frequency_grid        wavey-solver/src/freq.rs:15-22 (fractional octave)
//   FdtdSettings::weight  wavey-solver/src/fdtd.rs:166-175
//   phase_error_deg_per_m wavey-solver/src/fdtd.rs:157-162
//   auto_duration         wavey-solver/src/fdtd.rs:866-869
//   to_transfer           wavey-solver/src/fdtd.rs:819-840
//   blend                 wavey-solver/src/fdtd.rs:847-863
//   fit_first_order       wavey-solver/src/fdtd.rs:749-807
//   component_weights     wavey-solver/src/fdtd.rs:812-815
//   SpeakerInstance::rotation  wavey-speaker/src/instance.rs:44-48
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../../include/wavey_host.h"
#include "cplx.hpp"

using wh::cx;

namespace {
constexpr double PI = 3.141592653589793;

// Column-major 3x3 (glam DMat3) times a vector: col0*x + col1*y + col2*z.
inline void mat_vec(const double m[9], const double v[3], double out[3]) {
    for (int r = 0; r < 3; r++) out[r] = m[r] * v[0] + m[3 + r] * v[1] + m[6 + r] * v[2];
}
inline void mat_mul(const double a[9], const double b[9], double out[9]) {
    double t[9];
    for (int c = 0; c < 3; c++) mat_vec(a, b + 3 * c, t + 3 * c);
    for (int i = 0; i < 9; i++) out[i] = t[i];
}
}  // namespace

extern "C" void wh_source_signal(double f_max, double dt, int64_t steps, double *out) {
    const double sigma = 0.342 / f_max;
    const double t0 = 6.0 * sigma;
    for (int64_t n = 0; n < steps; n++) {
        double t = (double)n * dt - t0;
        out[n] = -t / (sigma * sigma) * std::exp(-(t * t) / (2.0 * sigma * sigma)) * dt;
    }
}

extern "C" int32_t wh_frequency_grid(double f_min, double f_max, int32_t n, double *out, int32_t cap) {
    const double nn = (double)std::max(n, 1);
    const int64_t k0 = (int64_t)std::ceil(nn * std::log2(f_min / 1.03 / 1000.0));
    const int64_t k1 = (int64_t)std::floor(nn * std::log2(f_max * 1.03 / 1000.0));
    int32_t count = 0;
    for (int64_t k = k0; k <= k1; k++, count++)
        if (count < cap && out) out[count] = 1000.0 * std::pow(2.0, (double)k / nn);
    return count;
}

extern "C" double wh_crossover_weight(double crossover_hz, double f) {
    double x = std::log2(f / crossover_hz);
    if (x <= -0.5) return 1.0;
    if (x >= 0.5) return 0.0;
    return 0.5 * (1.0 + std::cos(PI * (x + 0.5)));
}

extern "C" double wh_phase_error_deg_per_m(double f, double c, double dx) {
    double dt = WAVEY_COURANT * dx / c;
    double w = 2.0 * PI * f;
    double k_num = 2.0 / dx * std::asin(std::sin(w * dt / 2.0) / WAVEY_COURANT);
    return std::fabs(k_num - w / c) * (180.0 / PI);
}

extern "C" double wh_auto_duration(const double *rt, int32_t n) {
    double t = 0.0;
    for (int32_t i = 0; i < n && i < 3; i++)
        if (std::isfinite(rt[i])) t = std::max(t, rt[i]);
    return std::clamp(1.2 * t, 0.3, 4.0);
}

extern "C" void wh_to_transfer(const double *spectra, int64_t n_recv, const double *signal, int64_t steps, double dt,
                               double dx, const double *freqs, int64_t nf, double c, double r_ref, const double *h0,
                               double *out) {
    std::vector<cx> s(nf);
    for (int64_t fi = 0; fi < nf; fi++) {
        cx acc{0.0, 0.0};
        for (int64_t n = 0; n < steps; n++) {
            double x = freqs[fi] * dt * (double)n;
            acc = acc + wh::from_polar(signal[n], -2.0 * PI * (x - std::trunc(x)));
        }
        s[fi] = acc;
    }
    const double scale = dt * dt / (dx * (dx * dx)) * 4.0 * PI * c * c * r_ref;
    for (int64_t i = 0; i < n_recv * nf; i++) {
        int64_t fi = i % nf;
        cx v{spectra[2 * i], spectra[2 * i + 1]};
        cx h{h0[2 * fi], h0[2 * fi + 1]};
        cx r = v / s[fi] * scale * h;
        out[2 * i] = r.re;
        out[2 * i + 1] = r.im;
    }
}

extern "C" void wh_blend(const double ism_[2], const double wave_[2], double w, double out[2]) {
    cx ism{ism_[0], ism_[1]}, wave{wave_[0], wave_[1]};
    cx r;
    if (w <= 0.0) {
        r = ism;
    } else if (w >= 1.0) {
        r = wave;
    } else {
        double target = (1.0 - w) * wh::norm_sqr(ism) + w * wh::norm_sqr(wave);
        cx p = ism * (1.0 - w) + wave * w;
        double m2 = wh::norm_sqr(p);
        if (m2 < 1e-6 * target) {
            cx dir = wh::norm_sqr(wave) * w >= wh::norm_sqr(ism) * (1.0 - w) ? wave : ism;
            r = dir / std::max(wh::norm(dir), 1e-300) * std::sqrt(target);
        } else {
            r = p * std::sqrt(target / m2);
        }
    }
    out[0] = r.re;
    out[1] = r.im;
}

extern "C" void wh_fit_directions(double out[WH_FIT_DIRECTIONS][3]) {
    const int N = WH_FIT_DIRECTIONS;
    const double golden = PI * (3.0 - std::sqrt(5.0));
    for (int i = 0; i < N; i++) {
        double z = 1.0 - 2.0 * ((double)i + 0.5) / (double)N;
        double r = std::sqrt(1.0 - z * z);
        out[i][0] = r * std::cos(golden * (double)i);
        out[i][1] = r * std::sin(golden * (double)i);
        out[i][2] = z;
    }
}

extern "C" void wh_fit_first_order(const double *d_samples, const double d_axis[2], const double to_room[9],
                                   double out_a[8], double *residual) {
    const int N = WH_FIT_DIRECTIONS;
    static thread_local double dirs[WH_FIT_DIRECTIONS][3];
    wh_fit_directions(dirs);
    double m[4][4] = {};
    cx rhs[4] = {};
    std::vector<std::pair<std::vector<double>, cx>> samples;
    for (int i = 0; i < N; i++) {
        cx d{d_samples[2 * i], d_samples[2 * i + 1]};
        double room[3];
        mat_vec(to_room, dirs[i], room);
        double b[4] = {1.0, room[0], room[1], room[2]};
        for (int a = 0; a < 4; a++) {
            for (int c = 0; c < 4; c++) m[a][c] += b[a] * b[c];
            rhs[a] = rhs[a] + d * b[a];
        }
        samples.push_back({{b[0], b[1], b[2], b[3]}, d});
    }
    // Gaussian elimination with partial pivoting (max_by keeps the last maximum).
    auto solve = [&](const cx in[4], cx out[4]) {
        double mm[4][4];
        cx x[4];
        for (int i = 0; i < 4; i++) {
            x[i] = in[i];
            for (int j = 0; j < 4; j++) mm[i][j] = m[i][j];
        }
        for (int col = 0; col < 4; col++) {
            int piv = col;
            for (int r = col + 1; r < 4; r++)
                if (!(std::fabs(mm[r][col]) < std::fabs(mm[piv][col]))) piv = r;
            for (int j = 0; j < 4; j++) std::swap(mm[col][j], mm[piv][j]);
            std::swap(x[col], x[piv]);
            for (int row = 0; row < 4; row++) {
                if (row == col) continue;
                double k = mm[row][col] / mm[col][col];
                for (int c = 0; c < 4; c++) mm[row][c] -= k * mm[col][c];
                x[row] = x[row] - x[col] * k;
            }
        }
        for (int i = 0; i < 4; i++) out[i] = x[i] / mm[i][i];
    };
    cx ls[4];
    solve(rhs, ls);
    const double xaxis[3] = {1.0, 0.0, 0.0};
    double axis[3];
    mat_vec(to_room, xaxis, axis);
    const double e[4] = {1.0, axis[0], axis[1], axis[2]};
    cx want{d_axis[0], d_axis[1]};
    cx got{0.0, 0.0};
    for (int i = 0; i < 4; i++) got = got + ls[i] * e[i];
    cx ec[4] = {{e[0], 0.0}, {e[1], 0.0}, {e[2], 0.0}, {e[3], 0.0}};
    cx me[4];
    solve(ec, me);
    double ete = -0.0;
    for (int i = 0; i < 4; i++) ete += me[i].re * e[i];
    cx a[4];
    for (int i = 0; i < 4; i++) a[i] = ls[i] + me[i] * ((want - got) / ete);
    double err = 0.0, tot = 0.0;
    for (auto &s : samples) {
        const std::vector<double> &b = s.first;
        cx fit = a[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
        err += wh::norm_sqr(fit - s.second);
        tot += wh::norm_sqr(s.second);
    }
    for (int i = 0; i < 4; i++) {
        out_a[2 * i] = a[i].re;
        out_a[2 * i + 1] = a[i].im;
    }
    *residual = std::sqrt(err / std::max(tot, 1e-30));
}

extern "C" void wh_component_weights(const double a0[2], const double a[6], double k, double dx, double out[8]) {
    cx dip{0.0, 2.0 * std::sin(k * dx)};
    cx w[4] = {{a0[0], a0[1]}, cx{a[0], a[1]} / dip, cx{a[2], a[3]} / dip, cx{a[4], a[5]} / dip};
    for (int i = 0; i < 4; i++) {
        out[2 * i] = w[i].re;
        out[2 * i + 1] = w[i].im;
    }
}

extern "C" void wh_speaker_rotation(double yaw_deg, double pitch_deg, double roll_deg, double out[9]) {
    auto rz = [](double a, double m[9]) {
        double s = std::sin(a), c = std::cos(a);
        double t[9] = {c, s, 0, -s, c, 0, 0, 0, 1};
        std::copy(t, t + 9, m);
    };
    auto ry = [](double a, double m[9]) {
        double s = std::sin(a), c = std::cos(a);
        double t[9] = {c, 0, -s, 0, 1, 0, s, 0, c};
        std::copy(t, t + 9, m);
    };
    auto rx = [](double a, double m[9]) {
        double s = std::sin(a), c = std::cos(a);
        double t[9] = {1, 0, 0, 0, c, s, 0, -s, c};
        std::copy(t, t + 9, m);
    };
    const double d2r = PI / 180.0;
    double a[9], b[9], c[9], ab[9];
    rz(yaw_deg * d2r, a);
    ry(-pitch_deg * d2r, b);
    rx(roll_deg * d2r, c);
    mat_mul(a, b, ab);
    mat_mul(ab, c, out);
}
