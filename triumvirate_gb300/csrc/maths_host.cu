// Host maths: Wigner 3-j symbols, spherical Bessel functions and the natural
// cubic spline tables the kernels evaluate.
#include <algorithm>
#include <cmath>
#include <vector>

#include "maths_host.h"

namespace trvg {

namespace {

double factorial(int n) {
  double f = 1.;
  for (int i = 2; i <= n; ++i) f *= double(i);
  return f;
}

// Power series of j_l(x) = x^l / (2l+1)!! sum_k (-x^2/2)^k /
// (k! (2l+3)(2l+5)...(2l+2k+1)); used where its first term dominates.
double sph_bessel_series(int ell, double x) {
  double pref = 1.;
  for (int i = 1; i <= ell; ++i) pref *= x / double(2 * i + 1);
  const double y = -0.5 * x * x;
  double term = 1., sum = 1.;
  for (int k = 1; k < 200; ++k) {
    term *= y / (double(k) * double(2 * ell + 2 * k + 1));
    sum += term;
    if (std::fabs(term) < 1e-18 * std::fabs(sum)) break;
  }
  return pref * sum;
}

// Miller's downward recurrence normalised to j_0 (or j_1 near zeros of j_0).
double sph_bessel_miller(int ell, double x) {
  const int start = ell + 40 + int(x);
  double jp1 = 0., j = 1e-250, jl = 0., j1 = 0.;
  for (int l = start; l >= 0; --l) {
    const double jm1 = (2.0 * l + 1.0) / x * j - jp1;
    jp1 = j;
    j = jm1;  // j now holds j_{l-1}
    if (l - 1 == ell) jl = j;
    if (l - 1 == 1) j1 = j;
    if (std::fabs(j) > 1e200) {  // rescale
      j *= 1e-200;
      jp1 *= 1e-200;
      jl *= 1e-200;
      j1 *= 1e-200;
    }
  }
  // After the loop `jp1` holds the unnormalised j_0.
  const double j0u = jp1;
  const double j0 = std::sin(x) / x;
  const double j1t = std::sin(x) / (x * x) - std::cos(x) / x;
  if (std::fabs(j0) >= std::fabs(j1t)) return jl * (j0 / j0u);
  return jl * (j1t / j1);
}

}  // namespace

double wigner_3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.;
  if (j3 < std::abs(j1 - j2) || j3 > j1 + j2) return 0.;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.;
  // Racah's formula.
  const double tri = factorial(j1 + j2 - j3) * factorial(j1 - j2 + j3) *
                     factorial(-j1 + j2 + j3) / factorial(j1 + j2 + j3 + 1);
  const double pref = tri * factorial(j1 + m1) * factorial(j1 - m1) *
                      factorial(j2 + m2) * factorial(j2 - m2) *
                      factorial(j3 + m3) * factorial(j3 - m3);
  const int kmin = std::max({0, j2 - j3 - m1, j1 - j3 + m2});
  const int kmax = std::min({j1 + j2 - j3, j1 - m1, j2 + m2});
  double s = 0.;
  for (int k = kmin; k <= kmax; ++k) {
    const double den = factorial(k) * factorial(j1 + j2 - j3 - k) *
                       factorial(j1 - m1 - k) * factorial(j2 + m2 - k) *
                       factorial(j3 - j2 + m1 + k) *
                       factorial(j3 - j1 - m2 + k);
    s += ((k & 1) ? -1. : 1.) / den;
  }
  const double sign = ((j1 - j2 - m3) % 2 != 0) ? -1. : 1.;
  return sign * std::sqrt(pref) * s;
}

double calc_coupling_coeff_3pt(int ell1, int ell2, int ELL, int m1, int m2,
                               int M) {
  return double(2 * ell1 + 1) * double(2 * ell2 + 1) * double(2 * ELL + 1) *
         wigner_3j(ell1, ell2, ELL, 0, 0, 0) *
         wigner_3j(ell1, ell2, ELL, m1, m2, M);
}

double calc_coupling_coeff_2pt(int ell, int ELL, int m, int M) {
  return double((2 * ell + 1) * (2 * ELL + 1)) *
         wigner_3j(ell, 0, ELL, 0, 0, 0) * wigner_3j(ell, 0, ELL, m, 0, M);
}

double sph_bessel(int ell, double x) {
  if (x == 0.) return ell == 0 ? 1. : 0.;
  if (x < 0.) return ((ell & 1) ? -1. : 1.) * sph_bessel(ell, -x);
  if (x * x < 4.0 * ell + 6.0) return sph_bessel_series(ell, x);
  if (ell == 0) return std::sin(x) / x;
  if (x > double(ell)) {
    const double sx = std::sin(x), cx = std::cos(x);
    double jm = sx / x;
    double j = sx / (x * x) - cx / x;
    for (int l = 1; l < ell; ++l) {
      const double jn = (2.0 * l + 1.0) / x * j - jm;
      jm = j;
      j = jn;
    }
    return j;
  }
  return sph_bessel_miller(ell, x);
}

// SphericalBesselCalculator (maths.cpp:309-343): nodes x_i = 0 + 0.05 i on
// [0, max(1000, ell^2)], natural cubic spline through j_ell(x_i).
SplineHost::SplineHost(int ell_) : ell(ell_) {
  split = (1000. >= double(ell) * ell) ? 1000. : double(ell) * ell;
  const double xmin = 0.;
  const double dx = kSplineStep;
  const int n = int((split - xmin) / dx) + 1;
  y.resize(n);
  c.assign(n, 0.);
  for (int i = 0; i < n; ++i) y[i] = sph_bessel(ell, xmin + dx * i);
  // Natural spline: c_0 = c_{n-1} = 0 and for 0 < i < n-1
  //   c_{i-1} + 4 c_i + c_{i+1} = 3 (y_{i+1} - 2 y_i + y_{i-1}) / h^2
  // (c = half the second derivative), solved by the Thomas algorithm.
  if (n >= 3) {
    const int m = n - 2;
    std::vector<double> cp(m), dp(m);
    const double h2 = dx * dx;
    for (int q = 0; q < m; ++q) {
      const int i = q + 1;
      const double rhs = 3. * (y[i + 1] - 2. * y[i] + y[i - 1]) / h2;
      const double b = 4.;
      if (q == 0) {
        cp[q] = 1. / b;
        dp[q] = rhs / b;
      } else {
        const double den = b - cp[q - 1];
        cp[q] = 1. / den;
        dp[q] = (rhs - dp[q - 1]) / den;
      }
    }
    c[m] = dp[m - 1];
    for (int q = m - 2; q >= 0; --q) c[q + 1] = dp[q] - cp[q] * c[q + 2];
  }
  // Interval polynomials: b_i = (y_{i+1} - y_i)/h - h (c_{i+1} + 2 c_i)/3,
  // d_i = (c_{i+1} - c_i) / (3 h), with h the node spacing of interval i.
  b.assign(n, 0.);
  d.assign(n, 0.);
  for (int i = 0; i + 1 < n; ++i) {
    const double hh = (xmin + dx * (i + 1)) - (xmin + dx * i);
    b[i] = (y[i + 1] - y[i]) / hh - hh * (c[i + 1] + 2.0 * c[i]) / 3.0;
    d[i] = (c[i + 1] - c[i]) / (3.0 * hh);
  }
}

SplineTable SplineHost::table(const double* dy, const double* db,
                              const double* dc, const double* dd) const {
  SplineTable t;
  t.y = dy;
  t.b = db;
  t.c = dc;
  t.d = dd;
  t.n = int(y.size());
  t.ell = ell;
  t.split = split;
  return t;
}

}  // namespace trvg
