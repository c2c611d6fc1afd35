// cplx.hpp -- complex arithmetic with the exact formulas of num-complex 0.4
// (the reference's complex type, pinned at 0.4.6 in Cargo.lock), so that the
// host-side FP64 restatements round the same way: plain (a c + b d)/|w|^2
// division without scaling, real-complex mixed operations that keep the real
// side exact.  std::complex is not used because its division scales.
#pragma once
#include <cmath>

namespace wh {

struct cx {
    double re, im;
};

inline cx operator+(cx a, cx b) { return {a.re + b.re, a.im + b.im}; }
inline cx operator-(cx a, cx b) { return {a.re - b.re, a.im - b.im}; }
inline cx operator*(cx a, cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cx operator/(cx a, cx b) {
    double n = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / n, (a.im * b.re - a.re * b.im) / n};
}
// Complex (op) real
inline cx operator*(cx a, double r) { return {a.re * r, a.im * r}; }
inline cx operator/(cx a, double r) { return {a.re / r, a.im / r}; }
inline cx operator+(cx a, double r) { return {a.re + r, a.im}; }
inline cx operator-(cx a, double r) { return {a.re - r, a.im}; }
// real (op) Complex
inline cx operator+(double r, cx a) { return {r + a.re, a.im}; }
inline cx operator-(double r, cx a) { return {r - a.re, 0.0 - a.im}; }
inline cx operator*(double r, cx a) { return {r * a.re, r * a.im}; }
inline cx operator/(double r, cx a) { return cx{r, 0.0} / a; }

inline double norm_sqr(cx a) { return a.re * a.re + a.im * a.im; }
inline double norm(cx a) { return std::hypot(a.re, a.im); }
inline double arg(cx a) { return std::atan2(a.im, a.re); }
inline cx from_polar(double r, double th) { return {r * std::cos(th), r * std::sin(th)}; }

}  // namespace wh
