// Fourier-space kernels: mode counting, shell-filtered field spectra on the
// evaluation grid, fine-binned two-point statistics and the shot-noise
// two-point field.
//
// Spectra of real meshes are stored as cuFFT half spectra
// (n0 x n1 x (n2/2 + 1)); a complex field is the pair (re, im) of the half
// spectra of its real and imaginary part meshes, read back at any full-grid
// index through Hermitian symmetry.  Interlacing (field.cpp:1615-1653) is
// applied on read from the raw main and shadow spectra.
#include <algorithm>
#include <type_traits>

#include "kernels.h"

namespace trvg {

namespace {

template <class C>
__device__ __forceinline__ cd ld(const C* p, int64_t i) {
  const C v = p[i];
  return cd{double(v.x), double(v.y)};
}

template <class C>
__device__ __forceinline__ cd half_value(const C* h, const Geom& g, int i,
                                         int j, int k) {
  if (k < g.nzh) return ld(h, (int64_t(i) * g.n[1] + j) * g.nzh + k);
  const int ii = (i == 0) ? 0 : g.n[0] - i;
  const int jj = (j == 0) ? 0 : g.n[1] - j;
  const int kk = g.n[2] - k;
  return conjg(ld(h, (int64_t(ii) * g.n[1] + jj) * g.nzh + kk));
}

template <class C>
__device__ __forceinline__ cd pair_value(const C* re, const C* im,
                                         const Geom& g, int i, int j, int k,
                                         double im_sign) {
  cd v = half_value(re, g, i, j, k);
  if (im != nullptr) {
    const cd b = half_value(im, g, i, j, k);
    v = v + cd{-im_sign * b.im, im_sign * b.re};  // v + i im_sign b
  }
  return v;
}

// Value of field `f` at full-grid index (i, j, k).
template <class Real>
__device__ __forceinline__ cd field_value(const FieldSpec<Real>& f,
                                          const Geom& g, int i, int j,
                                          int k) {
  if (f.k0_set && i == 0 && j == 0 && k == 0) return f.k0;
  cd v = pair_value(f.re, f.im, g, i, j, k, f.im_sign);
  if (f.re_s != nullptr) {
    const cd vs = pair_value(f.re_s, f.im_s, g, i, j, k, f.im_sign);
    const double mx = (i < g.n[0] / 2) ? double(i) / g.n[0]
                                       : double(i) / g.n[0] - 1;
    const double my = (j < g.n[1] / 2) ? double(j) / g.n[1]
                                       : double(j) / g.n[1] - 1;
    const double mz = (k < g.n[2] / 2) ? double(k) / g.n[2]
                                       : double(k) / g.n[2] - 1;
    const double arg = kPi * (mx + my + mz);
    double sa, ca;
    sincos(arg, &sa, &ca);
    v = cd{(v.re + (ca * vs.re - sa * vs.im)) / 2.,
           (v.im + (sa * vs.re + ca * vs.im)) / 2.};
  }
  if (f.sign != 1.) v = cd{f.sign * v.re, f.sign * v.im};
  return v;
}

// field_value for FP32 spectra without interlacing, in FP32.
template <class Real>
__device__ __forceinline__ float2 field_value_f(const FieldSpec<Real>& f,
                                               const Geom& g, int i, int j,
                                               int k) {
  if (f.k0_set && i == 0 && j == 0 && k == 0)
    return make_float2(float(f.k0.re), float(f.k0.im));
  auto half = [&](const float2* h) {
    if (k < g.nzh) return h[(int64_t(i) * g.n[1] + j) * g.nzh + k];
    const int ii = (i == 0) ? 0 : g.n[0] - i;
    const int jj = (j == 0) ? 0 : g.n[1] - j;
    const float2 v = h[(int64_t(ii) * g.n[1] + jj) * g.nzh + (g.n[2] - k)];
    return make_float2(v.x, -v.y);
  };
  float2 v = half(reinterpret_cast<const float2*>(f.re));
  if (f.im != nullptr) {
    float2 b = half(reinterpret_cast<const float2*>(f.im));
    if (f.im_sign != 1.) b = make_float2(-b.x, -b.y);
    v = make_float2(v.x - b.y, v.y + b.x);  // v + i b
  }
  if (f.sign != 1.) v = make_float2(-v.x, -v.y);
  return v;
}

// Per-axis FP32 factors of 1 / W (1 / sinc^order).
struct InvWinF {
  const float* w[3];
};

// Shot-noise aliasing C_1(k) (field.cpp:3463-3509).
__device__ __forceinline__ double alias_sn(const AxisTablesDev& ax, int i,
                                           int j, int k) {
  if (!ax.interlace)
    return ax.t.alias[0][i] * ax.t.alias[1][j] * ax.t.alias[2][k];
  const double ux = ax.t.u[0][i], uy = ax.t.u[1][j], uz = ax.t.u[2][k];
  const double uhalf = sqrt(ux * ux + uy * uy + uz * uz) / 2.;
  const double sh = sin(uhalf), ch = cos(uhalf);
  const double s2h = sh * sh, c2h = ch * ch;
  double cc = 1.;
  for (int q = 0; q < ax.order; ++q) cc *= c2h;
  double cs = 1.;
  if (ax.order == 2) {
    cs = 1. - 2. / 3. * s2h;
  } else if (ax.order == 3) {
    cs = 1. - s2h + 2. / 15. * s2h * s2h;
  } else if (ax.order == 4) {
    cs = 1. - 4. / 3. * s2h + 2. / 5. * s2h * s2h -
         4. / 315. * s2h * s2h * s2h;
  }
  return cc * cs;
}

__device__ __forceinline__ int wrap(int s, int n) { return s < 0 ? s + n : s; }

int grid_for(int64_t work, int block, int64_t cap = 152 * 16) {
  int64_t g = (work + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return int(g);
}

// ---------------------------------------------------------------------------

__global__ void count_modes_kernel(Geom g, Cube cube, BinsDev bins,
                                   long long* nmodes, double* ksum) {
  extern __shared__ unsigned char smem_raw[];
  double* s_k = reinterpret_cast<double*>(smem_raw);
  long long* s_n = reinterpret_cast<long long*>(s_k + bins.nbins);
  for (int b = threadIdx.x; b < bins.nbins; b += blockDim.x) {
    s_k[b] = 0.;
    s_n[b] = 0;
  }
  __syncthreads();
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       t < cube.count; t += int64_t(gridDim.x) * blockDim.x) {
    const int c = int(t % cube.ext[2]);
    const int b = int((t / cube.ext[2]) % cube.ext[1]);
    const int a = int(t / (int64_t(cube.ext[2]) * cube.ext[1]));
    const int sx = cube.dense[0] ? shift_index(a, g.n[0]) : a - cube.K[0];
    const int sy = cube.dense[1] ? shift_index(b, g.n[1]) : b - cube.K[1];
    const int sz = cube.dense[2] ? shift_index(c, g.n[2]) : c - cube.K[2];
    const double k = vec3_mag(dmul(double(sx), g.dk[0]),
                              dmul(double(sy), g.dk[1]),
                              dmul(double(sz), g.dk[2]));
    for (int q = 0; q < bins.nbins; ++q) {
      if (bins.lo[q] <= k && k < bins.hi[q]) {
        atomicAdd(reinterpret_cast<unsigned long long*>(s_n + q), 1ull);
        atomicAdd(s_k + q, k);
      }
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < bins.nbins; q += blockDim.x) {
    if (s_n[q] != 0) {
      atomicAdd(reinterpret_cast<unsigned long long*>(nmodes + q),
                (unsigned long long)s_n[q]);
      atomicAdd(ksum + q, s_k[q]);
    }
  }
}

// G on the evaluation grid: dn(k) / W(k) / V for |s| <= Kg on pruned axes,
// every mode on dense axes (G_LM: threept.cpp:1665-1670, field.cpp:1657-1785).
template <class Real, class FR>
__global__ void build_G_kernel(Geom g, int M0, int M1, int M2, int Kg0,
                               int Kg1, int Kg2, FieldSpec<Real> f,
                               AxisTablesDev ax,
                               typename CplxOf<FR>::type* out) {
  using C = typename CplxOf<FR>::type;
  const uint32_t count = uint32_t(M0) * M1 * M2;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(M2));
    const uint32_t row = t / uint32_t(M2);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const bool in = (M0 == g.n[0] || abs(sx) <= Kg0) &&
                    (M1 == g.n[1] || abs(sy) <= Kg1) &&
                    (M2 == g.n[2] || abs(sz) <= Kg2);
    C o;
    o.x = 0;
    o.y = 0;
    if (in) {
      const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
                k = wrap(sz, g.n[2]);
      const cd v = field_value(f, g, i, j, k);
      const double w = window_pow(ax, i, j, k);
      const cd r = cdivr(cdivr(v, w), g.vol);
      o.x = FR(r.re);
      o.y = FR(r.im);
    }
    out[t] = o;
  }
}

// build_G_kernel for FP32 spectra without interlacing, in FP32 (1 / W from
// the per-axis tables).
__global__ void build_G_f32_kernel(Geom g, int M0, int M1, int M2, int Kg0,
                                   int Kg1, int Kg2, FieldSpec<float> f,
                                   InvWinF iw, float inv_vol, float2* out) {
  const uint32_t count = uint32_t(M0) * M1 * M2;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(M2));
    const uint32_t row = t / uint32_t(M2);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const bool in = (M0 == g.n[0] || abs(sx) <= Kg0) &&
                    (M1 == g.n[1] || abs(sy) <= Kg1) &&
                    (M2 == g.n[2] || abs(sz) <= Kg2);
    float2 o = make_float2(0.f, 0.f);
    if (in) {
      const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
                k = wrap(sz, g.n[2]);
      const float2 v = field_value_f(f, g, i, j, k);
      const float w = iw.w[0][i] * iw.w[1][j] * iw.w[2][k] * inv_vol;
      o = make_float2(v.x * w, v.y * w);
    }
    out[t] = o;
  }
}

// Shell-filtered spectra y_lm(k) f(k) / W(k), one per bin, on the
// evaluation grid (field.cpp:1812-1847).  The 1/nmodes of the reference is
// applied to the reduced sums instead of the fields.
template <class Real, class FR>
__global__ void build_F_kernel(Geom g, int M0, int M1, int M2, int K0, int K1,
                               int K2, FieldSpec<Real> f, AxisTablesDev ax,
                               int ell, int m, float cnm, const double* lo,
                               const double* hi, int nb, double hi_max,
                               bool sparse, typename CplxOf<FR>::type* out) {
  using C = typename CplxOf<FR>::type;
  // FP32 fields without interlacing: only |k| (shell membership) in FP64.
  constexpr bool f32 = sizeof(FR) == 4 && sizeof(Real) == 4;
  const bool fast = f32 && f.re_s == nullptr && ell <= kMaxYlmDegree;
  const uint32_t count = uint32_t(M0) * M1 * M2;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(M2));
    const uint32_t row = t / uint32_t(M2);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const bool in = (M0 == g.n[0] || abs(sx) <= K0) &&
                    (M1 == g.n[1] || abs(sy) <= K1) &&
                    (M2 == g.n[2] || abs(sz) <= K2);
    double k = -1.;
    cd val = {0., 0.};
    float2 valf = make_float2(0.f, 0.f);
    if (in) {
      const double kx = dmul(double(sx), g.dk[0]);
      const double ky = dmul(double(sy), g.dk[1]);
      const double kz = dmul(double(sz), g.dk[2]);
      k = vec3_mag(kx, ky, kz);
      if (k < hi_max) {
        const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
                  kk = wrap(sz, g.n[2]);
        if (fast) {
          const float2 v = field_value_f(f, g, i, j, kk);
          const float iw = 1.f / float(window_pow(ax, i, j, kk));
          float2 y = make_float2(ell == 0 ? 1.f : 0.f, 0.f);
          if (ell > 0 && k >= 1.e-9) {
            const float ik = 1.f / float(k);
            y = ylm_lean_f(ell, m, cnm, float(kz) * ik,
                           make_float2(float(kx) * ik, -float(ky) * ik));
          }
          const float2 vw = make_float2(v.x * iw, v.y * iw);
          valf = make_float2(y.x * vw.x - y.y * vw.y, y.x * vw.y + y.y * vw.x);
        } else {
          const cd v = field_value(f, g, i, j, kk);
          const double w = window_pow(ax, i, j, kk);
          const cd y = reduced_ylm(ell, m, kx, ky, kz);
          val = y * cdivr(v, w);
        }
      }
    }
    if (sparse) {
      // Disjoint bins, output zeroed: only the bin holding k is written.
      if (in && k < hi_max)
        for (int q = 0; q < nb; ++q)
          if (lo[q] <= k && k < hi[q]) {
            C o;
            o.x = fast ? FR(valf.x) : FR(val.re);
            o.y = fast ? FR(valf.y) : FR(val.im);
            out[int64_t(q) * count + t] = o;
            break;
          }
      continue;
    }
    for (int q = 0; q < nb; ++q) {
      C o;
      const bool sel = in && (lo[q] <= k) && (k < hi[q]);
      o.x = sel ? (fast ? FR(valf.x) : FR(val.re)) : FR(0);
      o.y = sel ? (fast ? FR(valf.y) : FR(val.im)) : FR(0);
      out[int64_t(q) * count + t] = o;
    }
  }
}

// Half-spectrum variants (M0 x M1 x (M2/2 + 1)) of the builders for fields
// that are real: y_lm real with even ell and a real source field make the
// spectrum Hermitian, so the field is the C2R transform of its half.
template <class Real, class FR>
__global__ void build_G_half_kernel(Geom g, int M0, int M1, int M2, int Kg0,
                                    int Kg1, int Kg2, FieldSpec<Real> f,
                                    AxisTablesDev ax,
                                    typename CplxOf<FR>::type* out) {
  using C = typename CplxOf<FR>::type;
  const int Mh = M2 / 2 + 1;
  const uint32_t count = uint32_t(M0) * M1 * Mh;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(Mh));
    const uint32_t row = t / uint32_t(Mh);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const bool in = (M0 == g.n[0] || abs(sx) <= Kg0) &&
                    (M1 == g.n[1] || abs(sy) <= Kg1) &&
                    (M2 == g.n[2] || abs(sz) <= Kg2);
    C o;
    o.x = 0;
    o.y = 0;
    if (in) {
      const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
                k = wrap(sz, g.n[2]);
      const cd v = field_value(f, g, i, j, k);
      const double w = window_pow(ax, i, j, k);
      const cd r = cdivr(cdivr(v, w), g.vol);
      o.x = FR(r.re);
      o.y = FR(r.im);
    }
    out[t] = o;
  }
}

template <class Real, class FR>
__global__ void build_F_half_kernel(Geom g, int M0, int M1, int M2, int K0,
                                    int K1, int K2, FieldSpec<Real> f,
                                    AxisTablesDev ax, int ell, int m,
                                    const double* lo, const double* hi,
                                    int nb, double hi_max,
                                    typename CplxOf<FR>::type* out) {
  using C = typename CplxOf<FR>::type;
  const int Mh = M2 / 2 + 1;
  const uint32_t count = uint32_t(M0) * M1 * Mh;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(Mh));
    const uint32_t row = t / uint32_t(Mh);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const bool in = (M0 == g.n[0] || abs(sx) <= K0) &&
                    (M1 == g.n[1] || abs(sy) <= K1) &&
                    (M2 == g.n[2] || abs(sz) <= K2);
    double k = -1.;
    cd val = {0., 0.};
    if (in) {
      const double kx = dmul(double(sx), g.dk[0]);
      const double ky = dmul(double(sy), g.dk[1]);
      const double kz = dmul(double(sz), g.dk[2]);
      k = vec3_mag(kx, ky, kz);
      if (k < hi_max) {
        const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
                  kk = wrap(sz, g.n[2]);
        const cd v = field_value(f, g, i, j, kk);
        const double w = window_pow(ax, i, j, kk);
        const cd y = reduced_ylm(ell, m, kx, ky, kz);
        val = y * cdivr(v, w);
      }
    }
    for (int q = 0; q < nb; ++q) {
      C o;
      const bool sel = in && (lo[q] <= k) && (k < hi[q]);
      o.x = sel ? FR(val.re) : FR(0);
      o.y = sel ? FR(val.im) : FR(0);
      out[int64_t(q) * count + t] = o;
    }
  }
}

// ---- Fine-binned two-point statistics from a cached mode list ------------
//
// What twopt_stats_kernel computes per mode apart from the field product --
// sample-rule membership, |k|, y_lm(k) / W_pk and the shot-noise weight
// C1 y_lm / W_sn -- depends on the mesh, the binning and the degrees only.
// stats_plan_kernel evaluates it once (same exact FP64 arithmetic),
// stats_fill_kernel lists the member modes bin by bin, and per call
// stats_pk_kernel sums fa conj(fb) coef over each bin's list, one block row
// per bin, with no shared-memory atomics.

__device__ __forceinline__ void cube_mode(const Geom& g, const Cube& cube,
                                          uint32_t t, int& sx, int& sy,
                                          int& sz) {
  const int c = int(t % uint32_t(cube.ext[2]));
  const uint32_t r = t / uint32_t(cube.ext[2]);
  const int b = int(r % uint32_t(cube.ext[1]));
  const int a = int(r / uint32_t(cube.ext[1]));
  sx = cube.dense[0] ? shift_index(a, g.n[0]) : a - cube.K[0];
  sy = cube.dense[1] ? shift_index(b, g.n[1]) : b - cube.K[1];
  sz = cube.dense[2] ? shift_index(c, g.n[2]) : c - cube.K[2];
}

// Bins must be disjoint in sample index (each mode in at most one bin).
__global__ void stats_plan_kernel(Geom g, Cube cube, int ell, int m,
                                  AxisTablesDev ax, BinsDev bins,
                                  int16_t* qtab, double2* coef, double* kmode,
                                  double2* snmode) {
  const int n_sample = 1000000;
  const double dk_sample = 1.e-5;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
       t < uint32_t(cube.count); t += gridDim.x * blockDim.x) {
    int sx, sy, sz;
    cube_mode(g, cube, t, sx, sy, sz);
    const double kx = dmul(double(sx), g.dk[0]);
    const double ky = dmul(double(sy), g.dk[1]);
    const double kz = dmul(double(sz), g.dk[2]);
    const double k = vec3_mag(kx, ky, kz);
    const int idx_k = int(ddiv(k, dk_sample));
    int q = -1;
    if (idx_k >= 0 && idx_k < n_sample)
      for (int b = 0; b < bins.nbins; ++b)
        if (bins.smin[b] <= idx_k && idx_k < bins.smax[b]) q = b;
    qtab[t] = int16_t(q);
    if (q < 0) continue;
    kmode[t] = k;
    const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
              kk = wrap(sz, g.n[2]);
    const double al = alias_sn(ax, i, j, kk);
    double win_pk, win_sn;
    if (ax.interlace) {
      const double w = window_pow(ax, i, j, kk);
      win_pk = w * w;
      win_sn = win_pk;
    } else {
      win_pk = al;
      win_sn = al;
    }
    const cd y = reduced_ylm(ell, m, kx, ky, kz);
    const cd c = cdivr(y, win_pk);
    coef[t] = make_double2(c.re, c.im);
    const cd sn = cdivr(al * y, win_sn);
    snmode[t] = make_double2(sn.re, sn.im);
  }
}

__global__ void stats_fill_kernel(uint32_t nmode, const int16_t* qtab,
                                  const int* off, int* cursor,
                                  uint32_t* list) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nmode;
       t += gridDim.x * blockDim.x) {
    const int q = qtab[t];
    if (q >= 0) list[off[q] + atomicAdd(cursor + q, 1)] = t;
  }
}

// Mode values of the two legs: the (FP32 or FP64) spectra of the fields.
template <class Real>
struct SpectrumModes {
  FieldSpec<Real> fa, fb;
  __device__ __forceinline__ void values(const Geom& g, int sx, int sy,
                                         int sz, cd& va, cd& vb) const {
    const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
              kk = wrap(sz, g.n[2]);
    va = field_value(fa, g, i, j, kk);
    vb = field_value(fb, g, i, j, kk);
  }
};

// Mode values from the float-float spectrum cube |s| <= Kc of one real
// source mesh (both legs), cube[sx + Kc][sy + Kc][sz] for sz >= 0 and the
// conjugate mirror below; k = 0 from each leg's exact sum.
struct CubeModes {
  const float4* cube;
  int Kc;
  cd k0a, k0b;
  const double* k0a_dev;  // device k = 0 values of a replayed batch
  const double* k0b_dev;
  __device__ __forceinline__ void values(const Geom&, int sx, int sy, int sz,
                                         cd& va, cd& vb) const {
    if (sx == 0 && sy == 0 && sz == 0) {
      va = k0a_dev ? cd{k0a_dev[0], k0a_dev[1]} : k0a;
      vb = k0b_dev ? cd{k0b_dev[0], k0b_dev[1]} : k0b;
      return;
    }
    const bool neg = sz < 0;
    const int ax = neg ? -sx : sx, ay = neg ? -sy : sy, az = neg ? -sz : sz;
    const float4 c =
        cube[(int64_t(ax + Kc) * (2 * Kc + 1) + (ay + Kc)) * (Kc + 1) + az];
    const double im = double(c.z) + double(c.w);
    va = cd{double(c.x) + double(c.y), neg ? -im : im};
    vb = va;
  }
};

template <class Modes>
__global__ void __launch_bounds__(256)
stats_pk_kernel(Geom g, Cube cube, Modes modes, const int* off,
                const uint32_t* list, const double2* coef, double* pk) {
  const int q = blockIdx.y;
  const int e0 = off[q], e1 = off[q + 1];
  cd acc = {0., 0.};
  for (int e = e0 + blockIdx.x * blockDim.x + threadIdx.x; e < e1;
       e += gridDim.x * blockDim.x) {
    const uint32_t t = list[e];
    int sx, sy, sz;
    cube_mode(g, cube, t, sx, sy, sz);
    cd va, vb;
    modes.values(g, sx, sy, sz, va, vb);
    const double2 c = coef[t];
    acc = acc + (va * conjg(vb)) * cd{c.x, c.y};
  }
  __shared__ double red[2][32];
  double v[2] = {acc.re, acc.im};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int r = 0; r < 2; ++r) {
    double x = v[r];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[r][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double x = 0.;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) x += red[threadIdx.x][w];
    if (e1 > e0) atomicAdd(pk + 2 * q + threadIdx.x, x);
  }
}

// ---- FP32-mixed builders of real fields ---------------------------------
//
// For an FP32 real field without interlacing the values stay FP32: the
// half spectrum is read as float2 (Hermitian reconstruction for k >= nzh,
// the exact k = 0 value), and 1 / W is a product of per-axis FP32 tables.
// The shell a mode belongs to -- the exact FP64 |k| test of
// build_F_half_kernel -- comes from a table built once per mesh, grid and
// binning.

__device__ __forceinline__ float2 half_value_f(const float2* h, const Geom& g,
                                               int i, int j, int k) {
  if (k < g.nzh) return h[(int64_t(i) * g.n[1] + j) * g.nzh + k];
  const int ii = (i == 0) ? 0 : g.n[0] - i;
  const int jj = (j == 0) ? 0 : g.n[1] - j;
  float2 v = h[(int64_t(ii) * g.n[1] + jj) * g.nzh + (g.n[2] - k)];
  v.y = -v.y;
  return v;
}


// Shell index of every half-spectrum mode of the evaluation grid (-1: in
// no shell), bins disjoint.
__global__ void shell_table_kernel(Geom g, int M0, int M1, int M2, int K0,
                                   int K1, int K2, const double* lo,
                                   const double* hi, int nb, double hi_max,
                                   int16_t* tab) {
  const int Mh = M2 / 2 + 1;
  const uint32_t count = uint32_t(M0) * M1 * Mh;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(Mh));
    const uint32_t row = t / uint32_t(Mh);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const bool in = (M0 == g.n[0] || abs(sx) <= K0) &&
                    (M1 == g.n[1] || abs(sy) <= K1) &&
                    (M2 == g.n[2] || abs(sz) <= K2);
    int16_t bin = -1;
    if (in) {
      const double kx = dmul(double(sx), g.dk[0]);
      const double ky = dmul(double(sy), g.dk[1]);
      const double kz = dmul(double(sz), g.dk[2]);
      const double k = vec3_mag(kx, ky, kz);
      if (k < hi_max)
        for (int q = 0; q < nb; ++q)
          if (lo[q] <= k && k < hi[q]) bin = int16_t(q);
    }
    tab[t] = bin;
  }
}

__global__ void build_G_half_f32_kernel(Geom g, int M0, int M1, int M2,
                                        int Kg0, int Kg1, int Kg2,
                                        const float2* f, float2 k0, InvWinF iw,
                                        float inv_vol, float2* out) {
  const int Mh = M2 / 2 + 1;
  const uint32_t count = uint32_t(M0) * M1 * Mh;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(Mh));
    const uint32_t row = t / uint32_t(Mh);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const bool in = (M0 == g.n[0] || abs(sx) <= Kg0) &&
                    (M1 == g.n[1] || abs(sy) <= Kg1) &&
                    (M2 == g.n[2] || abs(sz) <= Kg2);
    float2 o = make_float2(0.f, 0.f);
    if (in) {
      const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
                k = wrap(sz, g.n[2]);
      const float2 v = (i == 0 && j == 0 && k == 0) ? k0
                                                   : half_value_f(f, g, i, j, k);
      const float s = iw.w[0][i] * iw.w[1][j] * iw.w[2][k] * inv_vol;
      o = make_float2(v.x * s, v.y * s);
    }
    out[t] = o;
  }
}

// Writes only the modes inside a shell: `out` is zeroed beforehand.
__global__ void build_F_half_f32_kernel(Geom g, int M0, int M1, int M2,
                                        const int16_t* tab, const float2* f,
                                        float2 k0, InvWinF iw, int ell,
                                        float2* out) {
  const int Mh = M2 / 2 + 1;
  const uint32_t count = uint32_t(M0) * M1 * Mh;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int q = tab[t];
    if (q < 0) continue;
    const int c = int(t % uint32_t(Mh));
    const uint32_t row = t / uint32_t(Mh);
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
              k = wrap(sz, g.n[2]);
    const float2 v = (i == 0 && j == 0 && k == 0) ? k0
                                                 : half_value_f(f, g, i, j, k);
    float s = iw.w[0][i] * iw.w[1][j] * iw.w[2][k];
    if (ell != 0) {
      const double kx = dmul(double(sx), g.dk[0]);
      const double ky = dmul(double(sy), g.dk[1]);
      const double kz = dmul(double(sz), g.dk[2]);
      s *= float(reduced_ylm(ell, 0, kx, ky, kz).re);
    }
    out[int64_t(q) * count + t] = make_float2(v.x * s, v.y * s);
  }
}

// Complex FP32 shell spectra on the full evaluation grid from the half-grid
// shell table: |k| depends on sz only through sz^2, so mode (a, b, c) with
// c > M2 / 2 reads entry (a, b, M2 - c).  Modes of shell q get
// y_lm(k) f(k) / W(k) with FP32 factors (1 / W from the per-axis tables);
// the others stay zero (`out` is zeroed beforehand).
__global__ void build_F_tab_f32_kernel(Geom g, int M0, int M1, int M2,
                                       const int16_t* tab,
                                       FieldSpec<float> f, InvWinF iw,
                                       int ell, int m, float cnm,
                                       float2* out) {
  const int Mh = M2 / 2 + 1;
  const uint32_t count = uint32_t(M0) * M1 * M2;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const int c = int(t % uint32_t(M2));
    const uint32_t row = t / uint32_t(M2);
    const int q = tab[int64_t(row) * Mh + (c < Mh ? c : M2 - c)];
    if (q < 0) continue;
    const int b = int(row % uint32_t(M1));
    const int a = int(row / uint32_t(M1));
    const int sx = shift_index(a, M0), sy = shift_index(b, M1),
              sz = shift_index(c, M2);
    const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
              kk = wrap(sz, g.n[2]);
    const float2 v = field_value_f(f, g, i, j, kk);
    const float w = iw.w[0][i] * iw.w[1][j] * iw.w[2][kk];
    float2 y = make_float2(1.f, 0.f);
    if (ell > 0) {
      const float kx = float(sx) * float(g.dk[0]);
      const float ky = float(sy) * float(g.dk[1]);
      const float kz = float(sz) * float(g.dk[2]);
      const float k = sqrtf(kx * kx + ky * ky + kz * kz);
      y = make_float2(0.f, 0.f);
      if (k > 0.f) {
        const float ik = 1.f / k;
        y = ylm_lean_f(ell, m, cnm, kz * ik, make_float2(kx * ik, -ky * ik));
      }
    }
    const float2 vw = make_float2(v.x * w, v.y * w);
    out[int64_t(q) * count + t] =
        make_float2(y.x * vw.x - y.y * vw.y, y.x * vw.y + y.y * vw.x);
  }
}

struct SjlArgs {
  SplineTable sj;
  const double* radii;
  int nb;
};

// j_l(k r) y_lm(k) f(k) / W(k) / V on the full mesh, one per radius
// (field.cpp:1908-2010).
template <class Real, class FR>
__global__ void build_F_sjl_kernel(Geom g, FieldSpec<Real> f,
                                   AxisTablesDev ax, int ell, int m,
                                   SjlArgs sa,
                                   typename CplxOf<FR>::type* out) {
  using C = typename CplxOf<FR>::type;
  const int64_t count = g.nmesh;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < count;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int kk = int(t % g.n[2]);
    const int j = int((t / g.n[2]) % g.n[1]);
    const int i = int(t / (int64_t(g.n[2]) * g.n[1]));
    const double kx = dmul(double(shift_index(i, g.n[0])), g.dk[0]);
    const double ky = dmul(double(shift_index(j, g.n[1])), g.dk[1]);
    const double kz = dmul(double(shift_index(kk, g.n[2])), g.dk[2]);
    const double k = vec3_mag(kx, ky, kz);
    const cd v = field_value(f, g, i, j, kk);
    const double w = window_pow(ax, i, j, kk);
    const cd y = reduced_ylm(ell, m, kx, ky, kz);
    const cd val = y * cdivr(v, w);
    for (int q = 0; q < sa.nb; ++q) {
      const double jl = spline_eval(sa.sj, k * sa.radii[q]);
      C o;
      o.x = FR(jl * val.re / g.vol);
      o.y = FR(jl * val.im / g.vol);
      out[int64_t(q) * count + t] = o;
    }
  }
}

template <class Real, class FR>
__global__ void build_F_sjl_half_kernel(Geom g, FieldSpec<Real> f,
                                        AxisTablesDev ax, int ell, int m,
                                        SjlArgs sa,
                                        typename CplxOf<FR>::type* out) {
  using C = typename CplxOf<FR>::type;
  const int64_t count = g.nhalf;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < count;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int kk = int(t % g.nzh);
    const int j = int((t / g.nzh) % g.n[1]);
    const int i = int(t / (int64_t(g.nzh) * g.n[1]));
    const double kx = dmul(double(shift_index(i, g.n[0])), g.dk[0]);
    const double ky = dmul(double(shift_index(j, g.n[1])), g.dk[1]);
    const double kz = dmul(double(shift_index(kk, g.n[2])), g.dk[2]);
    const double k = vec3_mag(kx, ky, kz);
    const cd v = field_value(f, g, i, j, kk);
    const double w = window_pow(ax, i, j, kk);
    const cd y = reduced_ylm(ell, m, kx, ky, kz);
    const cd val = y * cdivr(v, w);
    for (int q = 0; q < sa.nb; ++q) {
      const double jl = spline_eval(sa.sj, k * sa.radii[q]);
      C o;
      o.x = FR(jl * val.re / g.vol);
      o.y = FR(jl * val.im / g.vol);
      out[int64_t(q) * count + t] = o;
    }
  }
}

// FP32 fields of meshes whose three axes share one fundamental frequency
// dk: |k| = dk sqrt(key), key = sx^2 + sy^2 + sz^2, so j_l(k r_q) is one
// table entry per (key, radius) instead of one spline evaluation (FP64,
// with the upward recurrence beyond the spline) per mode and radius.
__global__ void sjl_key_table_kernel(double dk, int64_t nkeys, SjlArgs sa,
                                     float* jt /* [nkeys][nb] */) {
  const int64_t count = nkeys * sa.nb;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < count;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t key = t / sa.nb;
    const int q = int(t - key * sa.nb);
    const double k = dk * sqrt(double(key));
    jt[t] = float(spline_eval(sa.sj, k * sa.radii[q]));
  }
}

// j_l(k r_q) y_lm(k) f(k) / W(k) / V from the key table, each field entry
// one FP32 product.  With F32 (FP32 spectra without interlacing) the
// mode's value is formed in FP32 (1 / W from the per-axis tables, y_lm from
// the FP32 direction), otherwise in FP64 and rounded once.
template <class Real, bool HALF, bool F32>
__global__ void build_F_sjl_key_kernel(Geom g, FieldSpec<Real> f,
                                       AxisTablesDev ax, InvWinF iw,
                                       float cnm, int ell, int m, int nb,
                                       const float* __restrict__ jt,
                                       double inv_vol, float2* out) {
  const int64_t count = HALF ? g.nhalf : g.nmesh;
  const int nz = HALF ? g.nzh : g.n[2];
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < count;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int kk = int(t % nz);
    const int j = int((t / nz) % g.n[1]);
    const int i = int(t / (int64_t(nz) * g.n[1]));
    const int sx = shift_index(i, g.n[0]), sy = shift_index(j, g.n[1]),
              sz = shift_index(kk, g.n[2]);
    float vr, vi;
    if constexpr (F32) {
      const float2 v = field_value_f(f, g, i, j, kk);
      const float w =
          iw.w[0][i] * iw.w[1][j] * iw.w[2][kk] * float(inv_vol);
      float2 y = make_float2(1.f, 0.f);
      if (ell > 0) {
        const float kx = float(sx) * float(g.dk[0]);
        const float ky = float(sy) * float(g.dk[1]);
        const float kz = float(sz) * float(g.dk[2]);
        const float k = sqrtf(kx * kx + ky * ky + kz * kz);
        y = make_float2(0.f, 0.f);
        if (k > 0.f) {
          const float ik = 1.f / k;
          y = ylm_lean_f(ell, m, cnm, kz * ik,
                         make_float2(kx * ik, -ky * ik));
        }
      }
      vr = (y.x * v.x - y.y * v.y) * w;
      vi = (y.x * v.y + y.y * v.x) * w;
    } else {
      const double kx = dmul(double(sx), g.dk[0]);
      const double ky = dmul(double(sy), g.dk[1]);
      const double kz = dmul(double(sz), g.dk[2]);
      const cd v = field_value(f, g, i, j, kk);
      const double w = window_pow(ax, i, j, kk);
      const cd y = reduced_ylm(ell, m, kx, ky, kz);
      const cd val = y * cdivr(v, w);
      vr = float(val.re * inv_vol);
      vi = float(val.im * inv_vol);
    }
    const int64_t key = int64_t(sx) * sx + int64_t(sy) * sy + int64_t(sz) * sz;
    const float* row = jt + key * nb;
    for (int q = 0; q < nb; ++q) {
      const float jl = row[q];
      out[int64_t(q) * count + t] = make_float2(vr * jl, vi * jl);
    }
  }
}

// Key-table form: FP32 fields, one fundamental frequency on all axes.
template <class Real, class FR>
bool sjl_key_form(Context& ctx, const Geom& g, const SplineTable& sj,
                  const double* radii, int nb, int64_t& nkeys, float*& jt) {
  if constexpr (sizeof(FR) != 4) {
    return false;
  } else {
    if (g.dk[0] != g.dk[1] || g.dk[1] != g.dk[2]) return false;
    nkeys = 1;
    for (int a = 0; a < 3; ++a) nkeys += int64_t(g.n[a] / 2) * (g.n[a] / 2);
    if (nkeys * nb > (int64_t(1) << 30)) return false;
    jt = ctx.buf<float>("sjl.keys", size_t(nkeys) * nb);
    SjlArgs sa{sj, radii, nb};
    TRVG_KBEGIN(ctx, "sjl_key_table_kernel");
    sjl_key_table_kernel<<<grid_for(nkeys * nb, 256), 256, 0, ctx.stream>>>(
        g.dk[0], nkeys, sa, jt);
    TRVG_LAUNCHED(ctx);
    return true;
  }
}

// Fine-binned two-point statistics (field.cpp:2586-2702).  Each mode goes
// to fine sample int(k / 1e-5); bin b collects samples i with
// lo_b <= i * 1e-5 < hi_b (precomputed as [smin_b, smax_b)).
template <class Real>
__global__ void twopt_stats_kernel(Geom g, Cube cube, FieldSpec<Real> fa,
                                   FieldSpec<Real> fb, cd shot, int ell,
                                   int m, AxisTablesDev ax, BinsDev bins,
                                   long long* nmodes, double* ksum,
                                   double* pk, double* sn) {
  extern __shared__ unsigned char smem_raw[];
  double* s_k = reinterpret_cast<double*>(smem_raw);
  double* s_pk = s_k + bins.nbins;          // 2 * nbins
  double* s_sn = s_pk + 2 * bins.nbins;     // 2 * nbins
  long long* s_n = reinterpret_cast<long long*>(s_sn + 2 * bins.nbins);
  for (int q = threadIdx.x; q < bins.nbins; q += blockDim.x) {
    s_k[q] = 0.;
    s_pk[2 * q] = s_pk[2 * q + 1] = 0.;
    s_sn[2 * q] = s_sn[2 * q + 1] = 0.;
    s_n[q] = 0;
  }
  __syncthreads();
  const int n_sample = 1000000;
  const double dk_sample = 1.e-5;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       t < cube.count; t += int64_t(gridDim.x) * blockDim.x) {
    const int c = int(t % cube.ext[2]);
    const int b = int((t / cube.ext[2]) % cube.ext[1]);
    const int a = int(t / (int64_t(cube.ext[2]) * cube.ext[1]));
    const int sx = cube.dense[0] ? shift_index(a, g.n[0]) : a - cube.K[0];
    const int sy = cube.dense[1] ? shift_index(b, g.n[1]) : b - cube.K[1];
    const int sz = cube.dense[2] ? shift_index(c, g.n[2]) : c - cube.K[2];
    const double kx = dmul(double(sx), g.dk[0]);
    const double ky = dmul(double(sy), g.dk[1]);
    const double kz = dmul(double(sz), g.dk[2]);
    const double k = vec3_mag(kx, ky, kz);
    const int idx_k = int(ddiv(k, dk_sample));
    if (idx_k < 0 || idx_k >= n_sample) continue;
    bool any = false;
    for (int q = 0; q < bins.nbins; ++q)
      any |= (bins.smin[q] <= idx_k && idx_k < bins.smax[q]);
    if (!any) continue;
    const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
              kk = wrap(sz, g.n[2]);
    const cd va = field_value(fa, g, i, j, kk);
    const cd vb = field_value(fb, g, i, j, kk);
    const double al = alias_sn(ax, i, j, kk);
    double win_pk, win_sn;
    if (ax.interlace) {
      const double w = window_pow(ax, i, j, kk);
      win_pk = w * w;
      win_sn = win_pk;
    } else {
      win_pk = al;
      win_sn = al;
    }
    const cd y = reduced_ylm(ell, m, kx, ky, kz);
    const cd pkm = cdivr(va * conjg(vb), win_pk) * y;
    const cd snm = cdivr(al * shot, win_sn) * y;
    for (int q = 0; q < bins.nbins; ++q) {
      if (bins.smin[q] <= idx_k && idx_k < bins.smax[q]) {
        atomicAdd(reinterpret_cast<unsigned long long*>(s_n + q), 1ull);
        atomicAdd(s_k + q, k);
        atomicAdd(s_pk + 2 * q, pkm.re);
        atomicAdd(s_pk + 2 * q + 1, pkm.im);
        atomicAdd(s_sn + 2 * q, snm.re);
        atomicAdd(s_sn + 2 * q + 1, snm.im);
      }
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < bins.nbins; q += blockDim.x) {
    if (s_n[q] == 0) continue;
    atomicAdd(reinterpret_cast<unsigned long long*>(nmodes + q),
              (unsigned long long)s_n[q]);
    atomicAdd(ksum + q, s_k[q]);
    atomicAdd(pk + 2 * q, s_pk[2 * q]);
    atomicAdd(pk + 2 * q + 1, s_pk[2 * q + 1]);
    atomicAdd(sn + 2 * q, s_sn[2 * q]);
    atomicAdd(sn + 2 * q + 1, s_sn[2 * q + 1]);
  }
}

// Shot-noise two-point field spectrum (fa fb^* / win_pk - S C_1 / win_sn) / V
// (field.cpp:3273-3298) on the half-spectrum grid.  Without interlacing
// win_pk = win_sn = C_1, so the mode is fa fb^* / C_1 - S, formed with the
// reciprocal tables (no division).  When `out_im` is given the spectrum is
// split into its Hermitian parts so that both halves transform with C2R:
// P = H_re + i H_im.
template <class Real>
__device__ __forceinline__ cd twopt_mode(const Geom& g, const FieldSpec<Real>& fa,
                                         const FieldSpec<Real>& fb, cd shot,
                                         const AxisTablesDev& ax, int i,
                                         int j, int k) {
  const cd va = field_value(fa, g, i, j, k);
  const cd vb = field_value(fb, g, i, j, k);
  const cd pr = va * conjg(vb);
  if (!ax.interlace) {
    const double inv = ax.t.inv_alias[0][i] * ax.t.inv_alias[1][j] *
                       ax.t.inv_alias[2][k];
    return cd{pr.re * inv - shot.re, pr.im * inv - shot.im};
  }
  const double al = alias_sn(ax, i, j, k);
  const double w = window_pow(ax, i, j, k);
  const double win = w * w;
  return cdivr(pr, win) - cdivr(al * shot, win);
}

// One block per (i, j) row of the half spectrum; threads run along k.
template <class Real, class XR>
__global__ void __launch_bounds__(256)
twopt_field_kernel(Geom g, FieldSpec<Real> fa, FieldSpec<Real> fb, cd shot,
                   AxisTablesDev ax, typename CplxOf<XR>::type* out_re,
                   typename CplxOf<XR>::type* out_im) {
  using C = typename CplxOf<XR>::type;
  const double inv_vol = 1. / g.vol;
  const int row = blockIdx.x;
  const int i = row / g.n[1], j = row - (row / g.n[1]) * g.n[1];
  for (int k = threadIdx.x; k < g.nzh; k += blockDim.x) {
    const int64_t t = int64_t(row) * g.nzh + k;
    const cd p = twopt_mode(g, fa, fb, shot, ax, i, j, k);
    C o;
    if (out_im == nullptr) {
      o.x = XR(p.re * inv_vol);
      o.y = XR(p.im * inv_vol);
      out_re[t] = o;
    } else {
      const int ii = (i == 0) ? 0 : g.n[0] - i;
      const int jj = (j == 0) ? 0 : g.n[1] - j;
      const int kk = (k == 0) ? 0 : g.n[2] - k;
      const cd q = conjg(twopt_mode(g, fa, fb, shot, ax, ii, jj, kk));
      const cd s = p + q, d = p - q;
      const double h = 0.5 * inv_vol;
      o.x = XR(s.re * h);
      o.y = XR(s.im * h);
      out_re[t] = o;
      C oi;
      oi.x = XR(d.im * h);
      oi.y = XR(-d.re * h);
      out_im[t] = oi;
    }
  }
}

// twopt_field_kernel for FP32 spectra without interlacing, in FP32 (1 / C_1
// from the per-axis FP32 tables): the complex survey fields.
__device__ __forceinline__ float2 twopt_mode_f32(const Geom& g,
                                                 const FieldSpec<float>& fa,
                                                 const FieldSpec<float>& fb,
                                                 float2 shot, const InvWinF& ia,
                                                 int i, int j, int k) {
  const float2 va = field_value_f(fa, g, i, j, k);
  const float2 vb = field_value_f(fb, g, i, j, k);
  const float inv = ia.w[0][i] * ia.w[1][j] * ia.w[2][k];
  return make_float2((va.x * vb.x + va.y * vb.y) * inv - shot.x,
                     (va.y * vb.x - va.x * vb.y) * inv - shot.y);
}

__global__ void __launch_bounds__(256)
twopt_field_f32_kernel(Geom g, FieldSpec<float> fa, FieldSpec<float> fb,
                       float2 shot, InvWinF ia, float inv_vol, float2* out_re,
                       float2* out_im) {
  const int row = blockIdx.x;
  const int i = row / g.n[1], j = row - (row / g.n[1]) * g.n[1];
  for (int k = threadIdx.x; k < g.nzh; k += blockDim.x) {
    const int64_t t = int64_t(row) * g.nzh + k;
    const float2 p = twopt_mode_f32(g, fa, fb, shot, ia, i, j, k);
    if (out_im == nullptr) {
      out_re[t] = make_float2(p.x * inv_vol, p.y * inv_vol);
    } else {
      const int ii = (i == 0) ? 0 : g.n[0] - i;
      const int jj = (j == 0) ? 0 : g.n[1] - j;
      const int kk = (k == 0) ? 0 : g.n[2] - k;
      float2 q = twopt_mode_f32(g, fa, fb, shot, ia, ii, jj, kk);
      q.y = -q.y;
      const float h = 0.5f * inv_vol;
      out_re[t] = make_float2((p.x + q.x) * h, (p.y + q.y) * h);
      out_im[t] = make_float2((p.y - q.y) * h, -(p.x - q.x) * h);
    }
  }
}

// FP32 fast path for two real-mesh spectra without interlacing:
// P = (fa fb^* / C_1 - S) / V in float, the k = 0 mode given exactly.
// One element of the FP32 shot-noise field at flat half-spectrum index t.
__device__ __forceinline__ float2 twopt_elem_f32(uint32_t t, int n1, int nzh,
                                                 float2 a, float2 b,
                                                 const float* iax,
                                                 const float* iay,
                                                 const float* iaz, float shot,
                                                 float inv_vol, float2 p0) {
  if (t == 0) return p0;
  const uint32_t row = t / uint32_t(nzh);
  const int k = int(t - row * uint32_t(nzh));
  const int i = int(row / uint32_t(n1)), j = int(row - uint32_t(i) * n1);
  const float inv = iax[i] * iay[j] * iaz[k];
  float2 o;
  o.x = ((a.x * b.x + a.y * b.y) * inv - shot) * inv_vol;
  o.y = ((a.y * b.x - a.x * b.y) * inv) * inv_vol;
  return o;
}

// Flat over the half spectrum, two elements per 16-byte load and store.
__global__ void __launch_bounds__(256)
twopt_field_real_f32_kernel(uint32_t nhalf, int n1, int nzh, const float2* fa,
                            const float2* fb, const float* iax,
                            const float* iay, const float* iaz, float shot,
                            float inv_vol, float2 p0, const double* k0a,
                            const double* k0b, const double* shotp,
                            double vol, float2* out) {
  if (k0a != nullptr) {
    // The k = 0 modes and S of the current mock, from device memory:
    // (a0 conj(b0) - S) / V as for the host values.
    const double ar = k0a[0], ai = k0a[1], br = k0b[0], bi = k0b[1];
    shot = float(shotp[0]);
    p0 = make_float2(float((ar * br + ai * bi - shotp[0]) / vol),
                     float((ai * br - ar * bi - shotp[1]) / vol));
  }
  const bool same = fa == fb;  // |f|^2: one read of the spectrum
  const uint32_t npair = nhalf / 2;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < npair;
       u += gridDim.x * blockDim.x) {
    const float4 a = reinterpret_cast<const float4*>(fa)[u];
    const float4 b = same ? a : reinterpret_cast<const float4*>(fb)[u];
    const float2 o0 = twopt_elem_f32(2 * u, n1, nzh, make_float2(a.x, a.y),
                                     make_float2(b.x, b.y), iax, iay, iaz,
                                     shot, inv_vol, p0);
    const float2 o1 = twopt_elem_f32(2 * u + 1, n1, nzh, make_float2(a.z, a.w),
                                     make_float2(b.z, b.w), iax, iay, iaz,
                                     shot, inv_vol, p0);
    reinterpret_cast<float4*>(out)[u] = make_float4(o0.x, o0.y, o1.x, o1.y);
  }
  if ((nhalf & 1u) && blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t t = nhalf - 1;
    out[t] = twopt_elem_f32(t, n1, nzh, fa[t], fb[t], iax, iay, iaz, shot,
                            inv_vol, p0);
  }
}

// ---- Shot-noise field on one octant -----------------------------------------
//
// For weights symmetric under every sign flip of r (m = 0 legs of even
// total degree) the shot-noise sums need only xi averaged over the flips,
//   xi_s(a, b, c) = sum_k P(k) cos(k_x a dr) cos(k_y b dr) cos(k_z c dr),
// on 0 <= a, b, c <= n/2: the sum over the half-mesh octant of the flip-
// averaged spectrum with weights 1 (index 0 or n/2) or 2, i.e. three
// DCT-I passes of length n/2 + 1.  Each pass is a real FFT of length n of
// the even extension e[j] = e[n - j] of a line (the real parts of its
// first n/2 + 1 outputs).

// P averaged over (+-k_x, +-k_y), k_z >= 0 (its real part: the imaginary
// parts cancel in xi_s), written as the even extensions of the z lines:
// ext[(p (hy + 1) + q) n_z + j], j and n_z - j both holding k_z index r.
__global__ void __launch_bounds__(256)
xi_octant_spectrum_kernel(int n0, int n1, int nzh, const float2* fa,
                          const float2* fb, const float* iax,
                          const float* iay, const float* iaz, float shot,
                          float inv_vol, float2 p0, const double* k0a,
                          const double* k0b, const double* shotp, double vol,
                          float* ext) {
  if (k0a != nullptr) {
    const double ar = k0a[0], ai = k0a[1], br = k0b[0], bi = k0b[1];
    shot = float(shotp[0]);
    p0 = make_float2(float((ar * br + ai * bi - shotp[0]) / vol),
                     float((ai * br - ar * bi - shotp[1]) / vol));
  }
  const int hx = n0 / 2, hy = n1 / 2, hz = nzh - 1, nz = 2 * hz;
  const int64_t total = int64_t(hx + 1) * (hy + 1) * (hz + 1);
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < total;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int r = int(t % (hz + 1));
    const int64_t pq = t / (hz + 1);
    const int q = int(pq % (hy + 1)), pp = int(pq / (hy + 1));
    const int is[2] = {pp, (n0 - pp) % n0};
    const int js[2] = {q, (n1 - q) % n1};
    // The four images' loads first (one field when both legs share it).
    float2 av[4], bv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      av[u] = fa[(int64_t(is[u >> 1]) * n1 + js[u & 1]) * nzh + r];
    if (fa != fb) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        bv[u] = fb[(int64_t(is[u >> 1]) * n1 + js[u & 1]) * nzh + r];
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u) bv[u] = av[u];
    }
    float acc = 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = is[u >> 1], j = js[u & 1];
      if (i == 0 && j == 0 && r == 0) {
        acc += p0.x;
      } else {
        const float inv = iax[i] * iay[j] * iaz[r];
        acc += ((av[u].x * bv[u].x + av[u].y * bv[u].y) * inv - shot) *
               inv_vol;
      }
    }
    const float v = 0.25f * acc;
    float* line = ext + pq * nz;
    line[r] = v;
    if (r != 0 && r != hz) line[nz - r] = v;
  }
}

// The same flip-averaged spectrum of one field from its FP32 planes
// planes[r][x][y] (the mesh's z transform completed along x and y, before
// any transpose into the R2C layout): per p a 32 (q) x 32 (r) tile is
// read along y, averaged over the four (+-x, +-y) images and written along
// z through shared memory.
__global__ void __launch_bounds__(256)
xi_octant_planes_kernel(int n0, int n1, int nzh, const float2* planes,
                        const float* iax, const float* iay, const float* iaz,
                        float shot, float inv_vol, float2 p0,
                        const double* k0a, const double* k0b,
                        const double* shotp, double vol, float* ext) {
  __shared__ float tile[32][33];
  if (k0a != nullptr) {
    const double ar = k0a[0], ai = k0a[1], br = k0b[0], bi = k0b[1];
    shot = float(shotp[0]);
    p0 = make_float2(float((ar * br + ai * bi - shotp[0]) / vol),
                     float((ai * br - ar * bi - shotp[1]) / vol));
  }
  const int hy = n1 / 2, hz = nzh - 1, nz = 2 * hz;
  const int pp = blockIdx.z;
  const int q0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t plane = int64_t(n0) * n1;
  const int is[2] = {pp, (n0 - pp) % n0};
  for (int k = ty; k < 32; k += 8) {
    const int r = r0 + k, q = q0 + tx;
    float v = 0.f;
    if (r <= hz && q <= hy) {
      const int js[2] = {q, (n1 - q) % n1};
      float acc = 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = is[u >> 1], j = js[u & 1];
        if (i == 0 && j == 0 && r == 0) {
          acc += p0.x;
        } else {
          const float2 a = planes[int64_t(r) * plane + int64_t(i) * n1 + j];
          const float inv = iax[i] * iay[j] * iaz[r];
          acc += ((a.x * a.x + a.y * a.y) * inv - shot) * inv_vol;
        }
      }
      v = 0.25f * acc;
    }
    tile[k][tx] = v;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int q = q0 + k, r = r0 + tx;
    if (q <= hy && r <= hz) {
      float* line = ext + (int64_t(pp) * (hy + 1) + q) * nz;
      const float v = tile[tx][k];
      line[r] = v;
      if (r != 0 && r != hz) line[nz - r] = v;
    }
  }
}

// Real parts of R2C outputs, transposed into the even extensions of the
// next axis: for slab s, src row r and column k,
//   dst[s dS + k dK + r] = dst[s dS + k dK + (len - r)] = src[s sS + r sR + k].x
// (rows r = 0 .. len/2, columns k = 0 .. ncol - 1), through 32 x 32 tiles.
__global__ void __launch_bounds__(256)
octant_transpose_kernel(const float2* src, int64_t sS, int64_t sR, float* dst,
                        int64_t dS, int64_t dK, int nrow, int ncol, int len) {
  __shared__ float tile[32][33];
  const int s = blockIdx.z;
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows a pass
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, k = k0 + tx;
    if (r < nrow && k < ncol) tile[i][tx] = src[s * sS + r * sR + k].x;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int k = k0 + i, r = r0 + tx;
    if (r < nrow && k < ncol) {
      float* line = dst + s * dS + k * dK;
      const float v = tile[tx][i];
      line[r] = v;
      if (r != 0 && r != len / 2) line[len - r] = v;
    }
  }
}

}  // namespace

void launch_count_modes(Context& ctx, const Geom& g, const Cube& cube,
                        const BinsDev& bins, long long* nmodes,
                        double* ksum) {
  const size_t smem = bins.nbins * (sizeof(double) + sizeof(long long));
  TRVG_KBEGIN(ctx, "count_modes_kernel");
  count_modes_kernel<<<grid_for(cube.count, 256), 256, smem, ctx.stream>>>(
      g, cube, bins, nmodes, ksum);
  TRVG_LAUNCHED(ctx);
}

template <class Real, class FR>
void launch_build_G(Context& ctx, const Geom& g, const int M[3],
                    const int Kg[3], const FieldSpec<Real>& f,
                    const AxisTablesDev& ax,
                    typename CplxOf<FR>::type* out) {
  const int64_t count = int64_t(M[0]) * M[1] * M[2];
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  TRVG_KBEGIN(ctx, "build_G_kernel");
  build_G_kernel<Real, FR><<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, M[0], M[1], M[2], Kg[0], Kg[1], Kg[2], f, ax, out);
  TRVG_LAUNCHED(ctx);
}

template <class Real, class FR>
void launch_build_F(Context& ctx, const Geom& g, const int M[3],
                    const int K[3], const FieldSpec<Real>& f,
                    const AxisTablesDev& ax, int ell, int m,
                    const double* lo, const double* hi, int nb,
                    double hi_max, typename CplxOf<FR>::type* out,
                    bool disjoint_bins) {
  const int64_t count = int64_t(M[0]) * M[1] * M[2];
  if (disjoint_bins)
    TRVG_CUDA(cudaMemsetAsync(
        out, 0, size_t(nb) * size_t(count) * sizeof(typename CplxOf<FR>::type),
        ctx.stream));
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  double cn[kMaxYlmDegree + 1] = {};
  float cnm = 0.f;
  if (ell <= kMaxYlmDegree) {
    ylm_all_norms(ell, cn);
    cnm = float(cn[std::abs(m)]);
  }
  TRVG_KBEGIN(ctx, "build_F_kernel");
  build_F_kernel<Real, FR><<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, M[0], M[1], M[2], K[0], K[1], K[2], f, ax, ell, m, cnm, lo, hi, nb,
      hi_max, disjoint_bins, out);
  TRVG_LAUNCHED(ctx);
}

template <class Real, class FR>
void launch_build_F_sjl(Context& ctx, const Geom& g, const FieldSpec<Real>& f,
                        const AxisTablesDev& ax, int ell, int m,
                        const SplineTable& sj, const double* radii, int nb,
                        typename CplxOf<FR>::type* out,
                        const float* const iw[3]) {
  int64_t nkeys = 0;
  float* jt = nullptr;
  if (sjl_key_form<Real, FR>(ctx, g, sj, radii, nb, nkeys, jt)) {
    InvWinF w{{iw[0], iw[1], iw[2]}};
    double cn[kMaxYlmDegree + 1] = {};
    const bool f32 = sizeof(Real) == 4 && f.re_s == nullptr &&
                     ell <= kMaxYlmDegree && iw[0] != nullptr;
    if (ell <= kMaxYlmDegree) ylm_all_norms(ell, cn);
    const float cnm = ell <= kMaxYlmDegree ? float(cn[std::abs(m)]) : 0.f;
    TRVG_KBEGIN(ctx, "build_F_sjl_kernel");
    if (f32)
      build_F_sjl_key_kernel<Real, false, true>
          <<<grid_for(g.nmesh, 256), 256, 0, ctx.stream>>>(
              g, f, ax, w, cnm, ell, m, nb, jt, 1. / g.vol,
              reinterpret_cast<float2*>(out));
    else
      build_F_sjl_key_kernel<Real, false, false>
          <<<grid_for(g.nmesh, 256), 256, 0, ctx.stream>>>(
              g, f, ax, w, cnm, ell, m, nb, jt, 1. / g.vol,
              reinterpret_cast<float2*>(out));
    TRVG_LAUNCHED(ctx);
    return;
  }
  SjlArgs sa{sj, radii, nb};
  TRVG_KBEGIN(ctx, "build_F_sjl_kernel");
  build_F_sjl_kernel<Real, FR><<<grid_for(g.nmesh, 256), 256, 0, ctx.stream>>>(
      g, f, ax, ell, m, sa, out);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_twopt_stats(Context& ctx, const Geom& g, const Cube& cube,
                        const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                        cd shot, int ell, int m, const AxisTablesDev& ax,
                        const BinsDev& bins, long long* nmodes, double* ksum,
                        double* pk, double* sn) {
  const size_t smem = bins.nbins * (5 * sizeof(double) + sizeof(long long));
  TRVG_KBEGIN(ctx, "twopt_stats_kernel");
  twopt_stats_kernel<Real><<<grid_for(cube.count, 256), 256, smem,
                             ctx.stream>>>(g, cube, fa, fb, shot, ell, m, ax,
                                           bins, nmodes, ksum, pk, sn);
  TRVG_LAUNCHED(ctx);
}

template <class Real, class XR>
void launch_twopt_field(Context& ctx, const Geom& g, const FieldSpec<Real>& fa,
                        const FieldSpec<Real>& fb, cd shot,
                        const AxisTablesDev& ax,
                        typename CplxOf<XR>::type* out_re,
                        typename CplxOf<XR>::type* out_im) {
  TRVG_KBEGIN(ctx, "twopt_field_kernel");
  twopt_field_kernel<Real, XR><<<g.n[0] * g.n[1], 256, 0, ctx.stream>>>(
      g, fa, fb, shot, ax, out_re, out_im);
  TRVG_LAUNCHED(ctx);
}

void launch_twopt_field_f32(Context& ctx, const Geom& g,
                            const FieldSpec<float>& fa,
                            const FieldSpec<float>& fb, float2 shot,
                            const float* const inv_alias[3], float2* out_re,
                            float2* out_im) {
  InvWinF ia{{inv_alias[0], inv_alias[1], inv_alias[2]}};
  TRVG_KBEGIN(ctx, "twopt_field_kernel");
  twopt_field_f32_kernel<<<g.n[0] * g.n[1], 256, 0, ctx.stream>>>(
      g, fa, fb, shot, ia, float(1. / g.vol), out_re, out_im);
  TRVG_LAUNCHED(ctx);
}

void launch_twopt_field_real_f32(Context& ctx, const Geom& g,
                                 const float2* fa, const float2* fb,
                                 const float* const inv_alias[3], float shot,
                                 float2 p0, float2* out, const double* k0a,
                                 const double* k0b, const double* shotp) {
  if (g.nhalf >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Mesh too large.");
  TRVG_KBEGIN(ctx, "twopt_field_kernel");
  twopt_field_real_f32_kernel<<<grid_for(g.nhalf / 2, 256), 256, 0,
                                ctx.stream>>>(
      uint32_t(g.nhalf), g.n[1], g.nzh, fa, fb, inv_alias[0], inv_alias[1],
      inv_alias[2], shot, float(1. / g.vol), p0, k0a, k0b, shotp, g.vol,
      out);
  TRVG_LAUNCHED(ctx);
}

void launch_xi_octant_spectrum(Context& ctx, const Geom& g, const float2* fa,
                               const float2* fb, const float* const inv_alias[3],
                               float shot, float2 p0, const double* k0a,
                               const double* k0b, const double* shotp,
                               float* ext) {
  const int64_t total =
      int64_t(g.n[0] / 2 + 1) * (g.n[1] / 2 + 1) * (g.n[2] / 2 + 1);
  TRVG_KBEGIN(ctx, "xi_octant_kernel");
  xi_octant_spectrum_kernel<<<grid_for(total, 256), 256, 0, ctx.stream>>>(
      g.n[0], g.n[1], g.nzh, fa, fb, inv_alias[0], inv_alias[1], inv_alias[2],
      shot, float(1. / g.vol), p0, k0a, k0b, shotp, g.vol, ext);
  TRVG_LAUNCHED(ctx);
}

void launch_xi_octant_planes(Context& ctx, const Geom& g, const float2* planes,
                             const float* const inv_alias[3], float shot,
                             float2 p0, const double* k0a, const double* k0b,
                             const double* shotp, float* ext) {
  const int hx = g.n[0] / 2, hy = g.n[1] / 2, hz = g.n[2] / 2;
  dim3 grid((hy + 1 + 31) / 32, (hz + 1 + 31) / 32, hx + 1);
  TRVG_KBEGIN(ctx, "xi_octant_kernel");
  xi_octant_planes_kernel<<<grid, 256, 0, ctx.stream>>>(
      g.n[0], g.n[1], g.nzh, planes, inv_alias[0], inv_alias[1],
      inv_alias[2], shot, float(1. / g.vol), p0, k0a, k0b, shotp, g.vol, ext);
  TRVG_LAUNCHED(ctx);
}

void launch_octant_transpose(Context& ctx, const float2* src, int64_t sS,
                             int64_t sR, float* dst, int64_t dS, int64_t dK,
                             int nslab, int nrow, int ncol, int len) {
  dim3 grid((ncol + 31) / 32, (nrow + 31) / 32, nslab);
  TRVG_KBEGIN(ctx, "xi_octant_kernel");
  octant_transpose_kernel<<<grid, 256, 0, ctx.stream>>>(src, sS, sR, dst, dS,
                                                        dK, nrow, ncol, len);
  TRVG_LAUNCHED(ctx);
}

void launch_stats_plan(Context& ctx, const Geom& g, const Cube& cube,
                       int ell, int m, const AxisTablesDev& ax,
                       const BinsDev& bins, int16_t* qtab, double2* coef,
                       double* kmode, double2* snmode) {
  if (cube.count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Mode cube too large.");
  TRVG_KBEGIN(ctx, "stats_plan_kernel");
  stats_plan_kernel<<<grid_for(cube.count, 256), 256, 0, ctx.stream>>>(
      g, cube, ell, m, ax, bins, qtab, coef, kmode, snmode);
  TRVG_LAUNCHED(ctx);
}

void launch_stats_fill(Context& ctx, int64_t nmode, const int16_t* qtab,
                       const int* off, int* cursor, uint32_t* list) {
  TRVG_KBEGIN(ctx, "stats_fill_kernel");
  stats_fill_kernel<<<grid_for(nmode, 256), 256, 0, ctx.stream>>>(
      uint32_t(nmode), qtab, off, cursor, list);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_stats_pk(Context& ctx, const Geom& g, const Cube& cube,
                     const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                     int nbins, int max_count, const int* off,
                     const uint32_t* list, const double2* coef, double* pk) {
  if (nbins <= 0 || max_count <= 0) return;
  const int bx = int(std::min<int64_t>((max_count + 1023) / 1024, 64));
  TRVG_KBEGIN(ctx, "twopt_stats_kernel");
  stats_pk_kernel<<<dim3(bx, nbins), 256, 0, ctx.stream>>>(
      g, cube, SpectrumModes<Real>{fa, fb}, off, list, coef, pk);
  TRVG_LAUNCHED(ctx);
}

// Wide-angle power-law kernel (field.cpp:1727-1760): every cell of a
// configuration-space field on the mesh times r^-p, r = |grid position|
// (the library's shifted cell coordinates), cells with r < 1e-6 unchanged.
template <class T>
__global__ void wide_angle_kernel(Geom g, T* f, double p) {
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       t < g.nmesh; t += int64_t(gridDim.x) * blockDim.x) {
    const int k = int(t % g.n[2]);
    const int j = int((t / g.n[2]) % g.n[1]);
    const int i = int(t / (int64_t(g.n[2]) * g.n[1]));
    const double rx = double(shift_index(i, g.n[0])) * g.dr[0];
    const double ry = double(shift_index(j, g.n[1])) * g.dr[1];
    const double rz = double(shift_index(k, g.n[2])) * g.dr[2];
    const double r = vec3_mag(rx, ry, rz);
    if (r < 1.e-6) continue;
    const double s = pow(r, -p);
    if constexpr (std::is_same_v<T, float2> || std::is_same_v<T, double2>) {
      using E = decltype(f[t].x);
      f[t].x = E(double(f[t].x) * s);
      f[t].y = E(double(f[t].y) * s);
    } else {
      f[t] = T(double(f[t]) * s);
    }
  }
}

template <class T>
void launch_wide_angle(Context& ctx, const Geom& g, T* f, double p) {
  TRVG_KBEGIN(ctx, "wide_angle_kernel");
  wide_angle_kernel<T><<<grid_for(g.nmesh, 256), 256, 0, ctx.stream>>>(
      g, f, p);
  TRVG_LAUNCHED(ctx);
}
template void launch_wide_angle<float>(Context&, const Geom&, float*, double);
template void launch_wide_angle<double>(Context&, const Geom&, double*,
                                        double);
template void launch_wide_angle<float2>(Context&, const Geom&, float2*,
                                        double);
template void launch_wide_angle<double2>(Context&, const Geom&, double2*,
                                         double);

// Adjoint of the single-leg shot-noise terms S_a = sum_{k in a} coef(k)
// fa(k) fb(k)^* / n_a for ell = 0: with fa = fb = delta away from k = 0,
// dS_a / dm(x) = 2 sum_k coef delta_k e^{ikx} / n_a, so every listed mode
// of the half spectrum (kz >= 0) adds 2 fac[a] coef(k) delta_k to U, and
// k = 0 adds fac[a] coef (fa + fb) (the two legs' k = 0 values, which the
// count mesh moves one for one).  Bins list disjoint modes.
template <class Modes, class UR>
__global__ void adjoint_stats_kernel(Geom g, Cube cube, Modes modes,
                                     const int* off, const uint32_t* list,
                                     const double2* coef, const double* fac,
                                     typename CplxOf<UR>::type* U) {
  const int q = blockIdx.y;
  const double f = fac[q];
  if (f == 0.) return;
  for (int e = off[q] + blockIdx.x * blockDim.x + threadIdx.x; e < off[q + 1];
       e += gridDim.x * blockDim.x) {
    const uint32_t t = list[e];
    int sx, sy, sz;
    cube_mode(g, cube, t, sx, sy, sz);
    if (sz < 0) continue;
    cd va, vb;
    modes.values(g, sx, sy, sz, va, vb);
    const double c = coef[t].x;
    const cd d = (sx == 0 && sy == 0 && sz == 0)
                     ? cd{va.re + vb.re, va.im + vb.im}
                     : cd{2. * va.re, 2. * va.im};
    const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]);
    auto& u = U[(int64_t(i) * g.n[1] + j) * g.nzh + sz];
    u.x += UR(f * c * d.re);
    u.y += UR(f * c * d.im);
  }
}

template <class Real, class UR>
void launch_adjoint_stats(Context& ctx, const Geom& g, const Cube& cube,
                          const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                          int nbins, int max_count, const int* off,
                          const uint32_t* list, const double2* coef,
                          const double* fac, typename CplxOf<UR>::type* U) {
  if (nbins <= 0 || max_count <= 0) return;
  const int bx = int(std::min<int64_t>((max_count + 255) / 256, 64));
  TRVG_KBEGIN(ctx, "adjoint_stats_kernel");
  adjoint_stats_kernel<SpectrumModes<Real>, UR>
      <<<dim3(bx, nbins), 256, 0, ctx.stream>>>(
          g, cube, SpectrumModes<Real>{fa, fb}, off, list, coef, fac, U);
  TRVG_LAUNCHED(ctx);
}

template void launch_adjoint_stats<float, float>(
    Context&, const Geom&, const Cube&, const FieldSpec<float>&,
    const FieldSpec<float>&, int, int, const int*, const uint32_t*,
    const double2*, const double*, float2*);
template void launch_adjoint_stats<double, double>(
    Context&, const Geom&, const Cube&, const FieldSpec<double>&,
    const FieldSpec<double>&, int, int, const int*, const uint32_t*,
    const double2*, const double*, double2*);

// U(k) += 2 scale Wh(k) / C_1(k) delta(k) on the half spectrum: the
// adjoint of sum_p mu_p S_ab through xi = IFFT[(|delta|^2 / C_1 - S) / V];
// at k = 0 the two legs' k = 0 values (a0 + b0) replace 2 delta.
template <class Real>
__global__ void adjoint_xi_kernel(Geom g,
                                  const typename CplxOf<Real>::type* Wh,
                                  FieldSpec<Real> fa, FieldSpec<Real> fb,
                                  AxisTablesDev ax, double scale,
                                  typename CplxOf<Real>::type* U) {
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       t < g.nhalf; t += int64_t(gridDim.x) * blockDim.x) {
    const int k = int(t % g.nzh);
    const int j = int((t / g.nzh) % g.n[1]);
    const int i = int(t / (int64_t(g.nzh) * g.n[1]));
    const cd va = field_value(fa, g, i, j, k), vb = field_value(fb, g, i, j, k);
    const cd d = (t == 0) ? cd{va.re + vb.re, va.im + vb.im}
                          : cd{2. * va.re, 2. * va.im};
    const double c = scale * double(Wh[t].x) / alias_sn(ax, i, j, k);
    U[t].x += Real(c * d.re);
    U[t].y += Real(c * d.im);
  }
}

template <class Real>
void launch_adjoint_xi(Context& ctx, const Geom& g,
                       const typename CplxOf<Real>::type* Wh,
                       const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                       const AxisTablesDev& ax, double scale,
                       typename CplxOf<Real>::type* U) {
  TRVG_KBEGIN(ctx, "adjoint_xi_kernel");
  adjoint_xi_kernel<Real><<<grid_for(g.nhalf, 256), 256, 0, ctx.stream>>>(
      g, Wh, fa, fb, ax, scale, U);
  TRVG_LAUNCHED(ctx);
}

template void launch_adjoint_xi<float>(Context&, const Geom&, const float2*,
                                       const FieldSpec<float>&,
                                       const FieldSpec<float>&,
                                       const AxisTablesDev&, double, float2*);
template void launch_adjoint_xi<double>(Context&, const Geom&,
                                        const double2*,
                                        const FieldSpec<double>&,
                                        const FieldSpec<double>&,
                                        const AxisTablesDev&, double,
                                        double2*);

void launch_stats_pk_cube(Context& ctx, const Geom& g, const Cube& cube,
                          const float4* ffcube, int Kc, cd k0a, cd k0b,
                          int nbins, int max_count, const int* off,
                          const uint32_t* list, const double2* coef,
                          double* pk, const double* k0a_dev,
                          const double* k0b_dev) {
  if (nbins <= 0 || max_count <= 0) return;
  const int bx = int(std::min<int64_t>((max_count + 1023) / 1024, 64));
  TRVG_KBEGIN(ctx, "twopt_stats_kernel");
  stats_pk_kernel<<<dim3(bx, nbins), 256, 0, ctx.stream>>>(
      g, cube, CubeModes{ffcube, Kc, k0a, k0b, k0a_dev, k0b_dev}, off, list,
      coef, pk);
  TRVG_LAUNCHED(ctx);
}

void launch_shell_table(Context& ctx, const Geom& g, const int M[3],
                        const int K[3], const double* lo, const double* hi,
                        int nb, double hi_max, int16_t* tab) {
  const int64_t count = int64_t(M[0]) * M[1] * (M[2] / 2 + 1);
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  TRVG_KBEGIN(ctx, "shell_table_kernel");
  shell_table_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, M[0], M[1], M[2], K[0], K[1], K[2], lo, hi, nb, hi_max, tab);
  TRVG_LAUNCHED(ctx);
}

void launch_build_G_half_f32(Context& ctx, const Geom& g, const int M[3],
                             const int Kg[3], const float2* f, cd k0,
                             const float* const iw[3], float2* out) {
  const int64_t count = int64_t(M[0]) * M[1] * (M[2] / 2 + 1);
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  InvWinF w{{iw[0], iw[1], iw[2]}};
  TRVG_KBEGIN(ctx, "build_G_kernel");
  build_G_half_f32_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, M[0], M[1], M[2], Kg[0], Kg[1], Kg[2], f,
      make_float2(float(k0.re), float(k0.im)), w, float(1. / g.vol), out);
  TRVG_LAUNCHED(ctx);
}

void launch_build_F_half_f32(Context& ctx, const Geom& g, const int M[3],
                             const int16_t* tab, const float2* f, cd k0,
                             const float* const iw[3], int ell, int nb,
                             float2* out) {
  const int64_t count = int64_t(M[0]) * M[1] * (M[2] / 2 + 1);
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  TRVG_CUDA(cudaMemsetAsync(out, 0, size_t(nb) * count * sizeof(float2),
                            ctx.stream));
  InvWinF w{{iw[0], iw[1], iw[2]}};
  TRVG_KBEGIN(ctx, "build_F_kernel");
  build_F_half_f32_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, M[0], M[1], M[2], tab, f, make_float2(float(k0.re), float(k0.im)), w,
      ell, out);
  TRVG_LAUNCHED(ctx);
}

void launch_build_G_f32(Context& ctx, const Geom& g, const int M[3],
                        const int Kg[3], const FieldSpec<float>& f,
                        const float* const iw[3], float2* out) {
  const int64_t count = int64_t(M[0]) * M[1] * M[2];
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  InvWinF w{{iw[0], iw[1], iw[2]}};
  TRVG_KBEGIN(ctx, "build_G_kernel");
  build_G_f32_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, M[0], M[1], M[2], Kg[0], Kg[1], Kg[2], f, w, float(1. / g.vol), out);
  TRVG_LAUNCHED(ctx);
}

void launch_build_F_tab_f32(Context& ctx, const Geom& g, const int M[3],
                            const int16_t* tab, const FieldSpec<float>& f,
                            const float* const iw[3], int ell, int m, int nb,
                            float2* out) {
  const int64_t count = int64_t(M[0]) * M[1] * M[2];
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  if (ell > kMaxYlmDegree)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Degree above the FP32 builder.");
  TRVG_CUDA(cudaMemsetAsync(out, 0, size_t(nb) * count * sizeof(float2),
                            ctx.stream));
  double cn[kMaxYlmDegree + 1] = {};
  ylm_all_norms(ell, cn);
  InvWinF w{{iw[0], iw[1], iw[2]}};
  TRVG_KBEGIN(ctx, "build_F_kernel");
  build_F_tab_f32_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, M[0], M[1], M[2], tab, f, w, ell, m, float(cn[std::abs(m)]), out);
  TRVG_LAUNCHED(ctx);
}

template <class Real, class FR>
void launch_build_G_half(Context& ctx, const Geom& g, const int M[3],
                         const int Kg[3], const FieldSpec<Real>& f,
                         const AxisTablesDev& ax,
                         typename CplxOf<FR>::type* out) {
  const int64_t count = int64_t(M[0]) * M[1] * (M[2] / 2 + 1);
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  TRVG_KBEGIN(ctx, "build_G_kernel");
  build_G_half_kernel<Real, FR><<<grid_for(count, 256), 256, 0,
                                  ctx.stream>>>(g, M[0], M[1], M[2], Kg[0],
                                                Kg[1], Kg[2], f, ax, out);
  TRVG_LAUNCHED(ctx);
}

template <class Real, class FR>
void launch_build_F_half(Context& ctx, const Geom& g, const int M[3],
                         const int K[3], const FieldSpec<Real>& f,
                         const AxisTablesDev& ax, int ell, int m,
                         const double* lo, const double* hi, int nb,
                         double hi_max, typename CplxOf<FR>::type* out) {
  const int64_t count = int64_t(M[0]) * M[1] * (M[2] / 2 + 1);
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  TRVG_KBEGIN(ctx, "build_F_kernel");
  build_F_half_kernel<Real, FR><<<grid_for(count, 256), 256, 0,
                                  ctx.stream>>>(g, M[0], M[1], M[2], K[0],
                                                K[1], K[2], f, ax, ell, m, lo,
                                                hi, nb, hi_max, out);
  TRVG_LAUNCHED(ctx);
}

template <class Real, class FR>
void launch_build_F_sjl_half(Context& ctx, const Geom& g,
                             const FieldSpec<Real>& f, const AxisTablesDev& ax,
                             int ell, int m, const SplineTable& sj,
                             const double* radii, int nb,
                             typename CplxOf<FR>::type* out,
                             const float* const iw[3]) {
  int64_t nkeys = 0;
  float* jt = nullptr;
  if (sjl_key_form<Real, FR>(ctx, g, sj, radii, nb, nkeys, jt)) {
    InvWinF w{{iw[0], iw[1], iw[2]}};
    double cn[kMaxYlmDegree + 1] = {};
    const bool f32 = sizeof(Real) == 4 && f.re_s == nullptr &&
                     ell <= kMaxYlmDegree && iw[0] != nullptr;
    if (ell <= kMaxYlmDegree) ylm_all_norms(ell, cn);
    const float cnm = ell <= kMaxYlmDegree ? float(cn[std::abs(m)]) : 0.f;
    TRVG_KBEGIN(ctx, "build_F_sjl_kernel");
    if (f32)
      build_F_sjl_key_kernel<Real, true, true>
          <<<grid_for(g.nhalf, 256), 256, 0, ctx.stream>>>(
              g, f, ax, w, cnm, ell, m, nb, jt, 1. / g.vol,
              reinterpret_cast<float2*>(out));
    else
      build_F_sjl_key_kernel<Real, true, false>
          <<<grid_for(g.nhalf, 256), 256, 0, ctx.stream>>>(
              g, f, ax, w, cnm, ell, m, nb, jt, 1. / g.vol,
              reinterpret_cast<float2*>(out));
    TRVG_LAUNCHED(ctx);
    return;
  }
  SjlArgs sa{sj, radii, nb};
  TRVG_KBEGIN(ctx, "build_F_sjl_kernel");
  build_F_sjl_half_kernel<Real, FR><<<grid_for(g.nhalf, 256), 256, 0,
                                      ctx.stream>>>(g, f, ax, ell, m, sa, out);
  TRVG_LAUNCHED(ctx);
}

#define TRVG_INST2(R, F)                                                     \
  template void launch_build_G<R, F>(Context&, const Geom&, const int*,      \
                                     const int*, const FieldSpec<R>&,        \
                                     const AxisTablesDev&, CplxOf<F>::type*);\
  template void launch_build_F<R, F>(                                        \
      Context&, const Geom&, const int*, const int*, const FieldSpec<R>&,    \
      const AxisTablesDev&, int, int, const double*, const double*, int,     \
      double, CplxOf<F>::type*, bool);                                       \
  template void launch_build_F_sjl<R, F>(                                    \
      Context&, const Geom&, const FieldSpec<R>&, const AxisTablesDev&, int, \
      int, const SplineTable&, const double*, int, CplxOf<F>::type*,         \
      const float* const*);                                                  \
  template void launch_build_G_half<R, F>(                                   \
      Context&, const Geom&, const int*, const int*, const FieldSpec<R>&,    \
      const AxisTablesDev&, CplxOf<F>::type*);                               \
  template void launch_build_F_half<R, F>(                                   \
      Context&, const Geom&, const int*, const int*, const FieldSpec<R>&,    \
      const AxisTablesDev&, int, int, const double*, const double*, int,     \
      double, CplxOf<F>::type*);                                             \
  template void launch_build_F_sjl_half<R, F>(                               \
      Context&, const Geom&, const FieldSpec<R>&, const AxisTablesDev&, int, \
      int, const SplineTable&, const double*, int, CplxOf<F>::type*,         \
      const float* const*);                                                  \
  template void launch_twopt_field<R, F>(                                    \
      Context&, const Geom&, const FieldSpec<R>&, const FieldSpec<R>&, cd,   \
      const AxisTablesDev&, CplxOf<F>::type*, CplxOf<F>::type*);
TRVG_INST2(float, float)
TRVG_INST2(float, double)
TRVG_INST2(double, double)
#undef TRVG_INST2

#define TRVG_INST(R)                                                         \
  template void launch_stats_pk<R>(Context&, const Geom&, const Cube&,       \
                                   const FieldSpec<R>&, const FieldSpec<R>&, \
                                   int, int, const int*, const uint32_t*,    \
                                   const double2*, double*);                 \
  template void launch_twopt_stats<R>(                                       \
      Context&, const Geom&, const Cube&, const FieldSpec<R>&,               \
      const FieldSpec<R>&, cd, int, int, const AxisTablesDev&,               \
      const BinsDev&, long long*, double*, double*, double*);
TRVG_INST(float)
TRVG_INST(double)
#undef TRVG_INST

}  // namespace trvg
