// Shared host/device arithmetic of the mesh estimators.
//
// The same functions run inside the CUDA kernels and in the host-side test
// hooks of the C ABI, so the host tests exercise the device arithmetic.
#pragma once

#include <cmath>
#include <cstdint>

#include <cuda_runtime.h>

#define TRVG_HD __host__ __device__ __forceinline__

namespace trvg {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// Complex double arithmetic.
// ---------------------------------------------------------------------------

struct cd {
  double re, im;
};

TRVG_HD cd cmk(double re, double im) { return cd{re, im}; }
TRVG_HD cd operator+(cd a, cd b) { return cd{a.re + b.re, a.im + b.im}; }
TRVG_HD cd operator-(cd a, cd b) { return cd{a.re - b.re, a.im - b.im}; }
TRVG_HD cd operator*(cd a, cd b) {
  return cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
TRVG_HD cd operator*(double s, cd a) { return cd{s * a.re, s * a.im}; }
TRVG_HD cd conjg(cd a) { return cd{a.re, -a.im}; }
// a / b for real b, component-wise as std::complex<double> operator/=(double).
TRVG_HD cd cdivr(cd a, double b) { return cd{a.re / b, a.im / b}; }

// ---------------------------------------------------------------------------
// Round-to-nearest FP64 primitives.  Wavevector magnitudes decide integer
// mode counts, so they are evaluated with the reference's operation order
// and no fused multiply-add (maths.cpp:57-59, field.cpp:555-562).  Host code
// is compiled with -ffp-contract=off for the same reason.
// ---------------------------------------------------------------------------

TRVG_HD double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
TRVG_HD double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
TRVG_HD double ddiv(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
TRVG_HD double dsqrt(double a) {
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}

// sqrt(x*x + y*y + z*z) summed left to right.
TRVG_HD double vec3_mag(double x, double y, double z) {
  return dsqrt(dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z)));
}

// FFT-ordered index -> signed frequency / offset (field.cpp:538-542).
TRVG_HD int shift_index(int i, int n) { return (i < n / 2) ? i : i - n; }

// y_lm for m = 0..ell at once (y[m]), for the fused field passes: with
// mu = z / r and Q_l^m(mu) = P_l^m(mu) / sin^m(theta) (Condon-Shortley
// phase included), a polynomial,
//   y_lm = sqrt((l-m)! / (l+m)!) Q_l^m(mu) ((x - i y) / r)^m,
// since sin^m(theta) exp(-i m phi) = ((x - i y) / r)^m: one square root
// and one division per vector.  Q_m^m = (-1)^m (2m-1)!!,
// Q_{m+1}^m = (2m+1) mu Q_m^m and
// Q_l^m = ((2l-1) mu Q_{l-1}^m - (l+m-1) Q_{l-2}^m) / (l-m).
// cnorm[m] = (-1)^m (2m-1)!! sqrt((l-m)! / (l+m)!) (ylm_all_norms).  The
// values agree with reduced_ylm to FP64 rounding; y_lm = 0 at |v| < 1e-9.
TRVG_HD void reduced_ylm_all(int ell, const double* cnorm, double x, double y,
                             double z, cd* out) {
  if (ell == 0) {
    out[0] = cmk(1.0, 0.0);
    return;
  }
  const double r = dsqrt(dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z)));
  if (fabs(r) < 1.e-9) {
    for (int m = 0; m <= ell; ++m) out[m] = cmk(0.0, 0.0);
    return;
  }
  const double inv = 1.0 / r;
  const double mu = z * inv;
  const cd u = cmk(x * inv, -y * inv);
  cd e = cmk(1.0, 0.0);  // ((x - i y) / r)^m
  for (int m = 0; m <= ell; ++m) {
    if (m > 0) e = e * u;
    double q2 = 1.0, q1 = 0.0, q = 1.0;  // Q_m^m / ((-1)^m (2m-1)!!)
    if (ell > m) {
      q1 = q2;
      q = double(2 * m + 1) * mu * q1;  // Q_{m+1}^m
      for (int l = m + 2; l <= ell; ++l) {
        const double qn =
            (double(2 * l - 1) * mu * q - double(l + m - 1) * q1) /
            double(l - m);
        q1 = q;
        q = qn;
      }
    }
    out[m] = (cnorm[m] * q) * e;
  }
}

// One order of the same form: y_lm with cnorm_am = cnorm[|m|] of
// ylm_all_norms(ell), mu = z / r and u = (x - i y) / r of a vector with
// |r| >= 1e-9 (y_l,-m = (-1)^m conj(y_lm)).
TRVG_HD cd ylm_lean(int ell, int m, double cnorm_am, double mu, cd u) {
  if (ell == 0) return cmk(1.0, 0.0);
  const int am = m < 0 ? -m : m;
  cd e = cmk(1.0, 0.0);
  for (int i = 0; i < am; ++i) e = e * u;
  double q1 = 0.0, q = 1.0;
  if (ell > am) {
    q1 = 1.0;
    q = double(2 * am + 1) * mu;
    for (int l = am + 2; l <= ell; ++l) {
      const double qn =
          (double(2 * l - 1) * mu * q - double(l + am - 1) * q1) /
          double(l - am);
      q1 = q;
      q = qn;
    }
  }
  cd v = (cnorm_am * q) * e;
  if (m < 0) {
    v = conjg(v);
    if (am & 1) v = -1.0 * v;
  }
  return v;
}

// ylm_lean in FP32 (cnm = cnorm[|m|] of ylm_all_norms).
__device__ __forceinline__ float2 ylm_lean_f(int ell, int m, float cnm,
                                             float mu, float2 u) {
  const int am = m < 0 ? -m : m;
  float2 e = make_float2(1.f, 0.f);
  for (int i = 0; i < am; ++i)
    e = make_float2(e.x * u.x - e.y * u.y, e.x * u.y + e.y * u.x);
  float q1 = 0.f, q = 1.f;
  if (ell > am) {
    q1 = 1.f;
    q = float(2 * am + 1) * mu;
    for (int l = am + 2; l <= ell; ++l) {
      const float qn =
          (float(2 * l - 1) * mu * q - float(l + am - 1) * q1) / float(l - am);
      q1 = q;
      q = qn;
    }
  }
  const float c = cnm * q;
  float2 v = make_float2(c * e.x, c * e.y);
  if (m < 0) {
    v.y = -v.y;
    if (am & 1) v = make_float2(-v.x, -v.y);
  }
  return v;
}

// cnorm[m] of reduced_ylm_all for degree ell (host or device).
TRVG_HD void ylm_all_norms(int ell, double* cnorm) {
  for (int m = 0; m <= ell; ++m) {
    double ratio = 1.0;  // (l-m)! / (l+m)!
    for (int k = ell - m + 1; k <= ell + m; ++k) ratio /= double(k);
    double df = 1.0;  // (2m-1)!!
    for (int k = 2 * m - 1; k > 1; k -= 2) df *= double(k);
    cnorm[m] = ((m & 1) ? -df : df) * sqrt(ratio);
  }
}

// ---------------------------------------------------------------------------
// Reduced spherical harmonics (maths.cpp:171-220):
//   y_lm(v) = (-1)^m [m < 0] conj(Y_l^m(v)) sqrt(4 pi / (2l + 1)),
// Y_l^m with the normalised associated Legendre function and the
// Condon-Shortley phase; y_00 = 1 and y_lm = 0 for |v| < 1e-9.  Formed as
// sqrt((l-|m|)! / (l+|m|)!) Q_l^|m|(mu) ((x - i y) / r)^|m| (conjugated,
// with (-1)^m, for m < 0), where Q_l^m = P_l^m / sin^m(theta) comes from the
// rational three-term recurrence: one square root and one division for the
// vector, one for the norm, instead of the reference's arccos and the
// square roots of the normalised recurrence.
// ---------------------------------------------------------------------------
TRVG_HD cd reduced_ylm(int ell, int m, double x, double y, double z) {
  if (ell == 0 && m == 0) return cmk(1.0, 0.0);
  const double r = dsqrt(dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z)));
  if (fabs(r) < 1.e-9) return cmk(0.0, 0.0);
  const int am = m < 0 ? -m : m;
  double ratio = 1.0;  // (l-m)! / (l+m)!
  for (int k = ell - am + 1; k <= ell + am; ++k) ratio /= double(k);
  double df = 1.0;  // (2m-1)!!
  for (int k = 2 * am - 1; k > 1; k -= 2) df *= double(k);
  const double cn = ((am & 1) ? -df : df) * sqrt(ratio);
  const double inv = 1.0 / r;
  return ylm_lean(ell, m, cn, z * inv, cmk(x * inv, -y * inv));
}

// y_lm of any order from the non-negative orders of reduced_ylm_all.
TRVG_HD cd ylm_of(const cd* ypos, int m) {
  if (m >= 0) return ypos[m];
  const cd v = conjg(ypos[-m]);
  return (m & 1) ? -1.0 * v : v;
}

// ---------------------------------------------------------------------------
// Spherical Bessel functions (maths.cpp:309-375).
// ---------------------------------------------------------------------------

// j_l(x) by upward recurrence from j_0 and j_1; stable for x > l (used at
// and beyond the spline split point max(1000, l^2)).
TRVG_HD double sph_bessel_upward(int ell, double x) {
  const double sx = sin(x), cx = cos(x);
  const double j0 = sx / x;
  if (ell == 0) return j0;
  double j1 = sx / (x * x) - cx / x;
  double jm = j0;
  for (int l = 1; l < ell; ++l) {
    const double jn = (2.0 * l + 1.0) / x * j1 - jm;
    jm = j1;
    j1 = jn;
  }
  return j1;
}

// Natural cubic spline of j_l on the nodes x_i = 0.05 i, i = 0..n-1, as
// the per-interval polynomial y_i + b_i dx + c_i dx^2 + d_i dx^3
// (c: half the second derivative at the nodes).
struct SplineTable {
  const double* y;
  const double* b;
  const double* c;
  const double* d;
  int n;
  int ell;
  double split;
  // FP32 copy for the FP32-mixed kernels: per interval (y hi, y lo, b, c)
  // and d (null when not uploaded).
  const float4* q = nullptr;
  const float* dq = nullptr;
};

constexpr double kSplineStep = 0.05;

// The interval is the one with x_i <= x < x_{i+1} (the last interval for
// x at the last node), found from x / 0.05 and corrected against the node
// values themselves.
TRVG_HD double spline_eval(const SplineTable& t, double x) {
  if (x >= t.split) return sph_bessel_upward(t.ell, x);
  const double h = kSplineStep;
  int i = int(x * (1. / h));
  if (i > t.n - 2) i = t.n - 2;
  if (i < 0) i = 0;
  double xlo = dmul(h, double(i));
  if (x < xlo && i > 0) {
    --i;
    xlo = dmul(h, double(i));
  } else if (i < t.n - 2 && x >= dmul(h, double(i + 1))) {
    ++i;
    xlo = dmul(h, double(i));
  }
  const double dx = x - xlo;
  return t.y[i] + dx * (t.b[i] + dx * (t.c[i] + dx * t.d[i]));
}

// ---------------------------------------------------------------------------
// Per-axis Fourier-space factors (field.cpp:1114-1146, 3440-3520).
// Products over the three axes are formed in the kernels.
// ---------------------------------------------------------------------------

struct AxisTables {
  const double* sinc[3];   // sin(u)/u (1 at u = 0), u = pi * i_shift / n
  const double* alias[3];  // per-axis shot-noise aliasing polynomial of sin^2
  const double* u[3];      // u itself (interlaced isotropic approximation)
  const double* inv_alias[3];  // 1 / alias
};

// ---------------------------------------------------------------------------
// Float-float accumulation.  GB300 issues FP64 (adds, and even conversions
// from FP32) at a small fraction of its FP32 rate, so long FP32 sums are
// carried as an unevaluated pair hi + lo updated with Knuth's TwoSum (the
// rounding error of each addition is recovered exactly and kept in lo).
// The pair holds a sum to about 2^-44 relative using FP32 operations only;
// it becomes a double once, at the end.
// ---------------------------------------------------------------------------

struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_zero() { return FF{0.f, 0.f}; }

// a += x.
__device__ __forceinline__ void ff_add(FF& a, float x) {
  const float s = a.hi + x;
  const float bv = s - a.hi;
  const float err = (a.hi - (s - bv)) + (x - bv);
  a.hi = s;
  a.lo += err;
}

// a += b.
__device__ __forceinline__ void ff_merge(FF& a, const FF& b) {
  const float s = a.hi + b.hi;
  const float bv = s - a.hi;
  const float err = (a.hi - (s - bv)) + (b.hi - bv) + (a.lo + b.lo);
  const float t = s + err;
  a.lo = err - (t - s);
  a.hi = t;
}

__device__ __forceinline__ double ff_value(const FF& a) {
  return double(a.hi) + double(a.lo);
}

// Warp-wide float-float sum; the total is valid in lane 0.
__device__ __forceinline__ FF ff_warp_sum(FF a) {
  for (int o = 16; o > 0; o >>= 1) {
    FF b;
    b.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
    b.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
    ff_merge(a, b);
  }
  return a;
}

}  // namespace trvg
