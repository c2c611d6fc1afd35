// materials.cpp -- absorption spectra and the boundary admittance fit.
//
// Restates, in FP64 with the reference's operation order:
//   Spectrum::eval             wavey-materials/src/spectrum.rs:24-44
//   statistical_absorption     wavey-materials/src/material.rs:81-91
//   fit_real_impedance         wavey-materials/src/material.rs:96-111
//   AdmittanceFit::admittance  wavey-materials/src/impedance_fit.rs:48-55
//   paris                      wavey-materials/src/impedance_fit.rs:73-84
//   nelder_mead                wavey-materials/src/impedance_fit.rs:87-131
//   decode / encode_branch     wavey-materials/src/impedance_fit.rs:140-155
//   fit_admittance             wavey-materials/src/impedance_fit.rs:158-235
#include <algorithm>
#include <cmath>
#include <functional>
#include <numeric>
#include <vector>

#include "../../../include/wavey_host.h"
#include "../../../include/wavey_status.h"
#include "cplx.hpp"

using wh::cx;

namespace {

constexpr double PI = 3.141592653589793;
constexpr double MAX_Q = 2.0;  // impedance_fit.rs:136

struct Branch {
    double r, m, k;
};

cx admittance(double beta0, const std::vector<Branch> &br, double f) {
    cx jw{0.0, 2.0 * PI * std::max(f, 1e-6)};
    cx y{beta0, 0.0};
    for (const Branch &b : br) y = y + 1.0 / (b.r + jw * b.m + b.k / jw);
    return y;
}

// R = (cos th - beta)/(cos th + beta), alpha = sum (1 - |R|^2) sin 2th h.
double paris(cx beta, int n) {
    double h = PI / 2.0 / n;
    double a = 0.0;
    for (int i = 0; i < n; i++) {
        double th = (i + 0.5) * h;
        double c = std::cos(th);
        cx r = (c - beta) / (c + beta);
        a += (1.0 - wh::norm_sqr(r)) * std::sin(2.0 * th) * h;
    }
    return a;
}

double statistical_absorption_real(double z) {
    const int N = 256;
    double h = (PI / 2.0) / N;
    double s = -0.0;
    for (int i = 0; i < N; i++) {
        double th = (i + 0.5) * h;
        double c = std::cos(th);
        double r = (z * c - 1.0) / (z * c + 1.0);
        s += (1.0 - (r * r + 0.0 * 0.0)) * std::sin(2.0 * th) * h;
    }
    return s;
}

using Cost = std::function<double(const std::vector<double> &)>;

std::pair<std::vector<double>, double> nelder_mead(const Cost &f, const std::vector<double> &x0, double step, int iters) {
    const size_t n = x0.size();
    std::vector<std::vector<double>> pts{x0};
    for (size_t i = 0; i < n; i++) {
        std::vector<double> p = x0;
        p[i] += step;
        pts.push_back(p);
    }
    std::vector<double> vals;
    for (auto &p : pts) vals.push_back(f(p));
    for (int it = 0; it < iters; it++) {
        std::vector<size_t> idx(n + 1);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return vals[a] < vals[b]; });
        std::vector<std::vector<double>> p2;
        std::vector<double> v2;
        for (size_t i : idx) {
            p2.push_back(pts[i]);
            v2.push_back(vals[i]);
        }
        pts.swap(p2);
        vals.swap(v2);
        if (std::fabs(vals[n] - vals[0]) < 1e-14) break;
        std::vector<double> centroid(n);
        for (size_t d = 0; d < n; d++) {
            double s = -0.0;
            for (size_t i = 0; i < n; i++) s += pts[i][d];
            centroid[d] = s / (double)n;
        }
        auto along = [&](double t) {
            std::vector<double> r(n);
            for (size_t d = 0; d < n; d++) r[d] = centroid[d] + t * (pts[n][d] - centroid[d]);
            return r;
        };
        std::vector<double> xr = along(-1.0);
        double fr = f(xr);
        if (fr < vals[0]) {
            std::vector<double> xe = along(-2.0);
            double fe = f(xe);
            if (fe < fr) {
                pts[n] = xe;
                vals[n] = fe;
            } else {
                pts[n] = xr;
                vals[n] = fr;
            }
        } else if (fr < vals[n - 1]) {
            pts[n] = xr;
            vals[n] = fr;
        } else {
            std::vector<double> xc = along(fr < vals[n] ? -0.5 : 0.5);
            double fc = f(xc);
            if (fc < std::min(vals[n], fr)) {
                pts[n] = xc;
                vals[n] = fc;
            } else {
                for (size_t i = 1; i <= n; i++) {
                    for (size_t d = 0; d < n; d++) pts[i][d] = pts[0][d] + 0.5 * (pts[i][d] - pts[0][d]);
                    vals[i] = f(pts[i]);
                }
            }
        }
    }
    // min_by keeps the first minimum.
    size_t best = 0;
    for (size_t i = 1; i <= n; i++)
        if (vals[i] < vals[best]) best = i;
    return {pts[best], vals[best]};
}

void decode(const std::vector<double> &x, int nb, double &beta0, std::vector<Branch> &br) {
    beta0 = std::exp(x[0]);
    br.clear();
    for (int b = 0; b < nb; b++) {
        double m = std::exp(x[1 + 3 * b]), k = std::exp(x[2 + 3 * b]);
        double q = MAX_Q / (1.0 + std::exp(-x[3 + 3 * b]));
        br.push_back({std::sqrt(m * k) / std::max(q, 1e-9), m, k});
    }
}

void encode_branch(double r, double m, double k, double out[3]) {
    double q = std::clamp(std::sqrt(m * k) / r / MAX_Q, 1e-6, 1.0 - 1e-6);
    out[0] = std::log(m);
    out[1] = std::log(k);
    out[2] = std::log(q / (1.0 - q));
}

}  // namespace

extern "C" double wh_spectrum_eval(const wh_spectrum *s, double f) {
    if (s->n <= 0) return s->value;
    int n = s->n;
    const double *fz = s->freqs_hz, *v = s->values;
    if (f <= fz[0]) return v[0];
    if (f >= fz[n - 1]) return v[n - 1];
    int i = (int)(std::upper_bound(fz, fz + n, f) - fz) - 1;  // partition_point(x <= f) - 1
    double f0 = std::log(fz[i]), f1 = std::log(fz[i + 1]);
    double t = (std::log(f) - f0) / (f1 - f0);
    return v[i] + t * (v[i + 1] - v[i]);
}

extern "C" double wh_fit_real_impedance(double alpha) {
    double lo = 1.567, hi = 1e7;
    if (alpha >= statistical_absorption_real(lo)) return lo;
    if (alpha <= 0.0) return hi;
    for (int i = 0; i < 80; i++) {
        double mid = std::sqrt(lo * hi);
        if (statistical_absorption_real(mid) > alpha)
            lo = mid;
        else
            hi = mid;
    }
    return std::sqrt(lo * hi);
}

static std::vector<Branch> branches_of(const wh_fit *fit) {
    std::vector<Branch> br;
    for (int b = 0; b < fit->n_branches; b++) br.push_back({fit->r[b], fit->m[b], fit->k[b]});
    return br;
}

extern "C" void wh_fit_admittance_at(const wh_fit *fit, double f, double out[2]) {
    cx y = admittance(fit->beta0, branches_of(fit), f);
    out[0] = y.re;
    out[1] = y.im;
}

extern "C" double wh_fit_absorption(const wh_fit *fit, double f) {
    return paris(admittance(fit->beta0, branches_of(fit), f), 256);
}

extern "C" int wh_fit_admittance(const wh_spectrum *absorption, double band_lo, double band_hi, int32_t max_branches,
                                 wh_fit *out) {
    if (!absorption || !out || max_branches < 0 || max_branches > WH_MAX_BRANCHES) return WAVEY_E_INVALID;
    const double lo = std::max(band_lo, 1.0), hi = std::max(band_hi, band_lo + 1.0);
    const int nf = 32;
    std::vector<double> freqs(nf), target(nf);
    for (int i = 0; i < nf; i++) freqs[i] = lo * std::pow(hi / lo, (double)i / (double)(nf - 1));
    for (int i = 0; i < nf; i++) target[i] = std::clamp(std::clamp(wh_spectrum_eval(absorption, freqs[i]), 0.0, 1.0), 0.0, 0.95);
    *out = wh_fit{};
    out->band_lo = lo;
    out->band_hi = hi;
    bool all_small = true;
    double tmax = 0.0;
    for (double t : target) {
        all_small = all_small && t < 1e-6;
        tmax = std::max(tmax, t);
    }
    if (all_small) {
        out->rms_error = tmax;
        out->max_error = tmax;
        return WAVEY_OK;
    }
    auto errors = [&](double beta0, const std::vector<Branch> &br, double &rms, double &mx) {
        double ss = -0.0;
        mx = 0.0;
        for (int i = 0; i < nf; i++) {
            double e = paris(admittance(beta0, br, freqs[i]), 96) - target[i];
            ss += e * e;
            mx = std::max(mx, std::fabs(e));
        }
        rms = std::sqrt(ss / nf);
    };
    double mean = -0.0;
    for (double t : target) mean += t;
    mean /= nf;
    const double beta_mean = 1.0 / wh_fit_real_impedance(std::max(mean, 1e-4));
    bool have = false;
    double best_rms = 0.0, best_b0 = 0.0;
    std::vector<Branch> best_br;
    for (int nb = 0; nb <= max_branches; nb++) {
        Cost cost = [&](const std::vector<double> &x) {
            double b0;
            std::vector<Branch> br;
            decode(x, nb, b0, br);
            double s = 0.0;
            for (int i = 0; i < nf; i++) {
                double e = paris(admittance(b0, br, freqs[i]), 48) - target[i];
                s += e * e;
            }
            return s;
        };
        std::vector<std::vector<double>> starts;
        if (nb == 0) {
            starts.push_back({std::log(beta_mean)});
        } else {
            for (double corner : {0.3, 1.0, 3.0})
                for (double level : {0.3, 1.0, 3.0}) {
                    std::vector<double> x{std::log(std::max(beta_mean * 0.3, 1e-6))};
                    for (int b = 0; b < nb; b++) {
                        double fc = std::sqrt(lo * hi) * corner * std::pow(3.0, b);
                        double wc = 2.0 * PI * fc;
                        double r = 1.0 / std::max(beta_mean * level, 1e-6);
                        double e[3];
                        encode_branch(r, r / (wc * 3.0), r * wc, e);
                        x.insert(x.end(), e, e + 3);
                    }
                    starts.push_back(x);
                }
        }
        for (auto &x0 : starts) {
            auto r1 = nelder_mead(cost, x0, 1.0, 1500 * (1 + nb));
            auto r2 = nelder_mead(cost, r1.first, 0.2, 1000 * (1 + nb));
            double b0, rms, mx;
            std::vector<Branch> br;
            decode(r2.first, nb, b0, br);
            errors(b0, br, rms, mx);
            if (!have || rms < best_rms - 1e-6) {
                have = true;
                best_rms = rms;
                best_b0 = b0;
                best_br = br;
            }
        }
        if (have && best_rms < 0.005) break;
    }
    // Drop negligible branches (impedance_fit.rs:227-231).
    std::vector<Branch> kept;
    for (const Branch &b : best_br) {
        bool any = false;
        for (double f : freqs) {
            cx jw{0.0, 2.0 * PI * f};
            cx z = b.r + jw * b.m + b.k / jw;
            if (wh::norm(1.0 / z) > 1e-5) {
                any = true;
                break;
            }
        }
        if (any) kept.push_back(b);
    }
    double beta0 = best_b0 < 1e-7 ? 0.0 : best_b0;
    double rms, mx;
    errors(beta0, kept, rms, mx);
    out->beta0 = beta0;
    out->n_branches = (int32_t)kept.size();
    for (size_t b = 0; b < kept.size(); b++) {
        out->r[b] = kept[b].r;
        out->m[b] = kept[b].m;
        out->k[b] = kept[b].k;
    }
    out->rms_error = rms;
    out->max_error = mx;
    return WAVEY_OK;
}
