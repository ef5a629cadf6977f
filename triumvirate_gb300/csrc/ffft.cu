// Float-float transforms of the shell fields (FP32-mixed path).
//
// The FP32 cuFFT transforms round about 2.3e-7 (rms, relative) per mode,
// and the bispectrum bins whose value is ~1e-4 of sum |F_a F_b G| amplify
// that to ~1e-5.  These transforms keep float-float precision (ff.cuh),
// for just the modes the shell fields use:
//   forward: the FP32 mesh -> its spectrum on the cube |s| <= Kg (three
//            line passes z, y, x; only the kept frequencies are stored);
//   inverse: each evaluation-grid field from its half spectrum (passes
//            x, y over the lines that can be nonzero, then C2R along z).
// Each pass loads a group of lines into shared memory and runs a
// self-sorting (Stockham) mixed-radix FFT over them (radices 8, 4, 2, 3,
// 5; the indexing of Govindaraju et al., SC 2008).  The results are
// rounded to FP32 once, at the end.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ff.cuh"
#include "kernels.h"

namespace trvg {

namespace {

int grid_for(int64_t work, int block, int64_t cap = 152 * 16) {
  int64_t g = (work + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return int(g);
}

__device__ __forceinline__ int wrapi(int s, int n) { return s < 0 ? s + n : s; }

// Frequency of index i on the evaluation grid, symmetric for odd m (the
// largest index of the positive half is (m - 1) / 2).  When the band
// |s| <= Kg fills an odd grid (m = 2 Kg + 1), the library's own mapping
// would drop +Kg while keeping -Kg, and the kz = 0 plane would lose its
// Hermitian symmetry.
__device__ __forceinline__ int sym_shift(int i, int m) {
  return i < (m + 1) / 2 ? i : i - m;
}

__device__ __forceinline__ int min_lines(int64_t a, int64_t b) {
  return int(a < b ? a : b);
}

// Float-float constants (hi, lo of the double values).
__device__ __forceinline__ FF k_rsqrt2() { return FF{0x1.6a09e6p-1f, 0x1.9fcef4p-27f}; }
__device__ __forceinline__ FF k_sqrt3_2() { return FF{0x1.bb67aep-1f, 0x1.0b0996p-26f}; }
__device__ __forceinline__ FF k_c1_5() { return FF{0x1.3c6ef4p-2f, -0x1.1a02d6p-27f}; }
__device__ __forceinline__ FF k_c2_5() { return FF{-0x1.9e377ap-1f, 0x1.1a02d6p-27f}; }
__device__ __forceinline__ FF k_s1_5() { return FF{0x1.e6f0e2p-1f, -0x1.97756p-26f}; }
__device__ __forceinline__ FF k_s2_5() { return FF{0x1.2cf23p-1f, 0x1.1d5698p-27f}; }

// In-place DFT of size R with root exp(d 2 pi i / R).
template <int R>
__device__ __forceinline__ void small_dft(FFC* v, int d);

template <>
__device__ __forceinline__ void small_dft<2>(FFC* v, int) {
  const FFC a = v[0], b = v[1];
  v[0] = ffc_add(a, b);
  v[1] = ffc_sub(a, b);
}

template <>
__device__ __forceinline__ void small_dft<4>(FFC* v, int d) {
  const FFC t0 = ffc_add(v[0], v[2]), t1 = ffc_sub(v[0], v[2]);
  const FFC t2 = ffc_add(v[1], v[3]);
  const FFC t3 = ffc_muli(ffc_sub(v[1], v[3]), d);
  v[0] = ffc_add(t0, t2);
  v[2] = ffc_sub(t0, t2);
  v[1] = ffc_add(t1, t3);
  v[3] = ffc_sub(t1, t3);
}

template <>
__device__ __forceinline__ void small_dft<8>(FFC* v, int d) {
  FFC e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  small_dft<4>(e, d);
  small_dft<4>(o, d);
  // o_k *= exp(d 2 pi i k / 8)
  const FF c = k_rsqrt2();
  auto w1 = [&](FFC x) {
    const FF re = (d > 0) ? ffsub(x.re, x.im) : ffadd(x.re, x.im);
    const FF im = (d > 0) ? ffadd(x.im, x.re) : ffsub(x.im, x.re);
    return FFC{ffmul(re, c), ffmul(im, c)};
  };
  o[1] = w1(o[1]);
  o[2] = ffc_muli(o[2], d);
  o[3] = ffc_muli(w1(o[3]), d);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = ffc_add(e[k], o[k]);
    v[k + 4] = ffc_sub(e[k], o[k]);
  }
}

template <>
__device__ __forceinline__ void small_dft<3>(FFC* v, int d) {
  const FFC t = ffc_add(v[1], v[2]);
  const FFC m = ffc_sub(v[0], ffc_scale2(t, 0.5f));
  const FFC u = ffc_mulr(ffc_muli(ffc_sub(v[1], v[2]), d), k_sqrt3_2());
  v[0] = ffc_add(v[0], t);
  v[1] = ffc_add(m, u);
  v[2] = ffc_sub(m, u);
}

template <>
__device__ __forceinline__ void small_dft<5>(FFC* v, int d) {
  const FFC t1 = ffc_add(v[1], v[4]), t2 = ffc_add(v[2], v[3]);
  const FFC t3 = ffc_sub(v[1], v[4]), t4 = ffc_sub(v[2], v[3]);
  const FF c1 = k_c1_5(), c2 = k_c2_5(), s1 = k_s1_5(), s2 = k_s2_5();
  const FFC b1 = ffc_add(v[0], ffc_add(ffc_mulr(t1, c1), ffc_mulr(t2, c2)));
  const FFC b2 = ffc_add(v[0], ffc_add(ffc_mulr(t1, c2), ffc_mulr(t2, c1)));
  const FFC b3 =
      ffc_muli(ffc_add(ffc_mulr(t3, s1), ffc_mulr(t4, s2)), d);
  const FFC b4 =
      ffc_muli(ffc_sub(ffc_mulr(t3, s2), ffc_mulr(t4, s1)), d);
  v[0] = ffc_add(v[0], ffc_add(t1, t2));
  v[1] = ffc_add(b1, b3);
  v[4] = ffc_sub(b1, b3);
  v[2] = ffc_add(b2, b4);
  v[3] = ffc_sub(b2, b4);
}

// Shared-memory slot of element i of a line: one pad slot per 8 elements,
// so that the stride-R accesses of a stage spread over the bank groups of
// the 16-byte elements.
__host__ __device__ __forceinline__ int pidx(int i) { return i + (i >> 3); }
__host__ __device__ __forceinline__ int padded_len(int n) {
  return pidx(n - 1) + 1;
}

// Butterflies one thread keeps in registers per stage.
template <int R>
struct StageItems {
  static constexpr int value = R == 8 || R == 5 ? 1 : 2;
};

// One Stockham stage of radix R over the nl lines of A (padded line length
// ln), in place: every thread loads and transforms its butterflies, the
// block synchronises, then every thread writes its results.
template <int R>
__device__ __noinline__ void ff_stage(float4* A, int nl, int n, int ln,
                                         int Ns, const float4* tw, int d) {
  constexpr int IMAX = StageItems<R>::value;
  const int nb = n / R;
  const int items = nl * nb;
  FFC v[IMAX][R];
#pragma unroll
  for (int it = 0; it < IMAX; ++it) {
    const int w = threadIdx.x + it * blockDim.x;
    if (w >= items) break;
    const int l = w / nb, j = w - l * nb;
    const float4* in = A + l * ln;
    const int k = j % Ns;
    const int step = (n / (Ns * R)) * k;  // r * step < n
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[it][r] = ffc_load(in + pidx(j + r * nb));
      if (r > 0 && k > 0) {
        const float4 t = tw[r * step];
        FFC wv{FF{t.x, t.y}, FF{t.z, t.w}};
        if (d < 0) wv.im = ffneg(wv.im);
        v[it][r] = ffc_mul(v[it][r], wv);
      }
    }
    small_dft<R>(v[it], d);
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IMAX; ++it) {
    const int w = threadIdx.x + it * blockDim.x;
    if (w >= items) break;
    const int l = w / nb, j = w - l * nb;
    float4* out = A + l * ln;
    const int k = j % Ns;
    const int idx = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) ffc_store(out + pidx(idx + r * Ns), v[it][r]);
  }
  __syncthreads();
}

// Transforms the nl lines of A (padded line length ln) in place.
__device__ void ff_fft_lines(float4* A, int nl, int ln, const FFPlan& P,
                             int d) {
  __syncthreads();
  int Ns = 1;
  for (int s = 0; s < P.nstage; ++s) {
    switch (P.radix[s]) {
      case 8: ff_stage<8>(A, nl, P.n, ln, Ns, P.tw, d); break;
      case 4: ff_stage<4>(A, nl, P.n, ln, Ns, P.tw, d); break;
      case 2: ff_stage<2>(A, nl, P.n, ln, Ns, P.tw, d); break;
      case 3: ff_stage<3>(A, nl, P.n, ln, Ns, P.tw, d); break;
      default: ff_stage<5>(A, nl, P.n, ln, Ns, P.tw, d); break;
    }
    Ns *= P.radix[s];
  }
}

__device__ __forceinline__ float4 ffc_pack(FFC a) {
  return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo);
}

// ---- Forward cube ----------------------------------------------------------

// z lines of the real mesh, two rows per complex line; keeps kz in [0, Kz]
// into T1[x][kz][y].
__global__ void __launch_bounds__(256, 2)
ff_fwd_z_kernel(Geom g, const float* mesh, FFPlan P, int LB, int Kz,
                float4* T1) {
  extern __shared__ float4 smem[];
  const int n2 = g.n[2], ln = padded_len(n2);
  float4* A = smem;
  const int64_t npair = int64_t(g.n[0]) * g.n[1] / 2;
  const int64_t p0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, npair - p0);
  for (int w = threadIdx.x; w < nl * n2; w += blockDim.x) {
    const int l = w / n2, i = w - l * n2;
    const int64_t r0 = 2 * (p0 + l);
    A[l * ln + pidx(i)] =
        make_float4(mesh[r0 * n2 + i], 0.f, mesh[(r0 + 1) * n2 + i], 0.f);
  }
  ff_fft_lines(A, nl, ln, P, -1);
  for (int w = threadIdx.x; w < nl * (Kz + 1); w += blockDim.x) {
    const int l = w / (Kz + 1), kz = w - l * (Kz + 1);
    const FFC z = ffc_load(A + l * ln + pidx(kz));
    const FFC zm = ffc_conj(
        ffc_load(A + l * ln + pidx(kz == 0 ? 0 : n2 - kz)));
    const FFC x0 = ffc_scale2(ffc_add(z, zm), 0.5f);
    const FFC x1 = ffc_scale2(ffc_muli(ffc_sub(z, zm), -1), 0.5f);
    const int64_t r0 = 2 * (p0 + l);
    for (int h = 0; h < 2; ++h) {
      const int64_t r = r0 + h;
      const int x = int(r / g.n[1]), y = int(r - int64_t(x) * g.n[1]);
      T1[(int64_t(x) * (Kz + 1) + kz) * g.n[1] + y] = ffc_pack(h ? x1 : x0);
    }
  }
}

// y lines (x, kz) of T1; keeps sy in [-Ky, Ky] into T2[sy + Ky][kz][x].
__global__ void __launch_bounds__(256, 2)
ff_fwd_y_kernel(Geom g, const float4* T1, FFPlan P, int LB, int Ky, int Kz,
                float4* T2) {
  extern __shared__ float4 smem[];
  const int n1 = g.n[1], ln = padded_len(n1);
  float4* A = smem;
  const int64_t nlines = int64_t(g.n[0]) * (Kz + 1);
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  for (int w = threadIdx.x; w < nl * n1; w += blockDim.x) {
    const int l = w / n1, i = w - l * n1;
    A[l * ln + pidx(i)] = T1[l0 * n1 + w];
  }
  ff_fft_lines(A, nl, ln, P, -1);
  const int ny = 2 * Ky + 1;
  for (int w = threadIdx.x; w < nl * ny; w += blockDim.x) {
    const int l = w / ny, b = w - l * ny;
    const int64_t line = l0 + l;
    const int x = int(line / (Kz + 1)), kz = int(line - int64_t(x) * (Kz + 1));
    T2[(int64_t(b) * (Kz + 1) + kz) * g.n[0] + x] =
        A[l * ln + pidx(wrapi(b - Ky, n1))];
  }
}

// x lines (sy, kz) of T2; keeps sx in [-Kx, Kx] into
// cube[sx + Kx][sy + Ky][kz].
__global__ void __launch_bounds__(256, 2)
ff_fwd_x_kernel(Geom g, const float4* T2, FFPlan P, int LB, int Kx, int Ky,
                int Kz, float4* cube) {
  extern __shared__ float4 smem[];
  const int n0 = g.n[0], ln = padded_len(n0);
  float4* A = smem;
  const int64_t nlines = int64_t(2 * Ky + 1) * (Kz + 1);
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  for (int w = threadIdx.x; w < nl * n0; w += blockDim.x) {
    const int l = w / n0, i = w - l * n0;
    A[l * ln + pidx(i)] = T2[l0 * n0 + w];
  }
  ff_fft_lines(A, nl, ln, P, -1);
  const int nx = 2 * Kx + 1;
  for (int w = threadIdx.x; w < nl * nx; w += blockDim.x) {
    const int l = w / nx, a = w - l * nx;
    const int64_t line = l0 + l;  // = b * (Kz + 1) + kz
    const int b = int(line / (Kz + 1)), kz = int(line - int64_t(b) * (Kz + 1));
    cube[(int64_t(a) * (2 * Ky + 1) + b) * (Kz + 1) + kz] =
        A[l * ln + pidx(wrapi(a - Kx, n0))];
  }
}

// ---- Evaluation-grid half spectra -----------------------------------------

struct FFBuild {
  int M0, M1;
  int Kc;            // cube half extent (all axes)
  const float2* iw[3];  // 1 / W per full-mesh index, float-float
  FF inv_vol;
};

__device__ __forceinline__ FFC cube_value(const float4* cube, int Kc, int sx,
                                          int sy, int sz) {
  return ffc_load(cube + (int64_t(sx + Kc) * (2 * Kc + 1) + (sy + Kc)) *
                             (Kc + 1) + sz);
}

__device__ __forceinline__ FF inv_window(const FFBuild& b, const Geom& g,
                                         int sx, int sy, int sz) {
  const float2 wx = b.iw[0][wrapi(sx, g.n[0])];
  const float2 wy = b.iw[1][wrapi(sy, g.n[1])];
  const float2 wz = b.iw[2][wrapi(sz, g.n[2])];
  return ffmul(ffmul(FF{wx.x, wx.y}, FF{wy.x, wy.y}), FF{wz.x, wz.y});
}

// E[c][b][a] (c in [0, Kg], (a, b) on the M grid) of G: the cube values
// with |sx|, |sy| <= Kg, times 1 / (W V); k = 0 from `k0`.
__global__ void ff_build_G_kernel(Geom g, FFBuild bd, const float4* cube,
                                  int Kg, FFC k0, float4* E) {
  const int64_t count = int64_t(Kg + 1) * bd.M1 * bd.M0;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < count;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int a = int(t % bd.M0);
    const int64_t r = t / bd.M0;
    const int b = int(r % bd.M1), c = int(r / bd.M1);
    const int sx = sym_shift(a, bd.M0), sy = sym_shift(b, bd.M1);
    FFC v = ffc_zero();
    if (abs(sx) <= Kg && abs(sy) <= Kg) {
      v = (sx == 0 && sy == 0 && c == 0) ? k0
                                         : cube_value(cube, bd.Kc, sx, sy, c);
      v = ffc_mulr(v, ffmul(inv_window(bd, g, sx, sy, c), bd.inv_vol));
    }
    E[t] = ffc_pack(v);
  }
}

// E[q][c][b][a] (c in [0, K]) of the shell fields: each mode of shell q
// (from the table on the M half grid) times y_l0(k) / W; E is zeroed first.
__global__ void ff_build_F_kernel(Geom g, FFBuild bd, int M2, const float4* cube,
                                  int K, const int16_t* tab, int ell, FFC k0,
                                  float4* E) {
  const int64_t plane = int64_t(K + 1) * bd.M1 * bd.M0;
  const int Mh = M2 / 2 + 1;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < plane;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int a = int(t % bd.M0);
    const int64_t r = t / bd.M0;
    const int b = int(r % bd.M1), c = int(r / bd.M1);
    const int q = tab[(int64_t(a) * bd.M1 + b) * Mh + c];
    if (q < 0) continue;
    const int sx = sym_shift(a, bd.M0), sy = sym_shift(b, bd.M1);
    FFC v = (sx == 0 && sy == 0 && c == 0) ? k0
                                           : cube_value(cube, bd.Kc, sx, sy, c);
    FF s = inv_window(bd, g, sx, sy, c);
    if (ell != 0) {
      const double kx = dmul(double(sx), g.dk[0]);
      const double ky = dmul(double(sy), g.dk[1]);
      const double kz = dmul(double(c), g.dk[2]);
      s = ffmul(s, ff_from_double(reduced_ylm(ell, 0, kx, ky, kz).re));
    }
    E[int64_t(q) * plane + t] = ffc_pack(ffc_mulr(v, s));
  }
}

// ---- Inverse transforms of a group of fields -------------------------------
// nf fields, each with planes c in [0, Kcf] and band |sx|, |sy| <= Kf.

// x lines (f, c, b in band) of E[f][c][b][a]; writes Y1[f][c][a][b].
__global__ void __launch_bounds__(256, 2)
ff_inv_x_kernel(int M0, int M1, int nf, int Kf, int Kcf, const float4* E,
                FFPlan P, int LB, float4* Y1) {
  extern __shared__ float4 smem[];
  const int ln = padded_len(M0);
  float4* A = smem;
  const int nb = 2 * Kf + 1;
  const int64_t nlines = int64_t(nf) * (Kcf + 1) * nb;
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  for (int w = threadIdx.x; w < nl * M0; w += blockDim.x) {
    const int l = w / M0, a = w - l * M0;
    const int64_t line = l0 + l;
    const int bb = int(line % nb);
    const int64_t fc = line / nb;  // f * (Kcf + 1) + c
    const int b = wrapi(bb - Kf, M1);
    A[l * ln + pidx(a)] = E[(fc * M1 + b) * M0 + a];
  }
  ff_fft_lines(A, nl, ln, P, +1);
  for (int w = threadIdx.x; w < nl * M0; w += blockDim.x) {
    const int l = w / M0, a = w - l * M0;
    const int64_t line = l0 + l;
    const int bb = int(line % nb);
    const int64_t fc = line / nb;
    const int b = wrapi(bb - Kf, M1);
    Y1[(fc * M0 + a) * M1 + b] = A[l * ln + pidx(a)];
  }
}

// y lines (f, c, a) of Y1 (entries outside the band are zero); writes
// Y2[f][a][b][c].
__global__ void __launch_bounds__(256, 2)
ff_inv_y_kernel(int M0, int M1, int nf, int Kf, int Kcf, const float4* Y1,
                FFPlan P, int LB, float4* Y2) {
  extern __shared__ float4 smem[];
  const int ln = padded_len(M1);
  float4* A = smem;
  const int64_t nlines = int64_t(nf) * (Kcf + 1) * M0;
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  for (int w = threadIdx.x; w < nl * M1; w += blockDim.x) {
    const int l = w / M1, b = w - l * M1;
    const int sb = sym_shift(b, M1);
    A[l * ln + pidx(b)] =
        (abs(sb) <= Kf) ? Y1[(l0 + l) * M1 + b] : make_float4(0, 0, 0, 0);
  }
  ff_fft_lines(A, nl, ln, P, +1);
  for (int w = threadIdx.x; w < nl * M1; w += blockDim.x) {
    const int l = w / M1, b = w - l * M1;
    const int64_t line = l0 + l;  // (f * (Kcf + 1) + c) * M0 + a
    const int a = int(line % M0);
    const int64_t fc = line / M0;
    const int c = int(fc % (Kcf + 1));
    const int64_t f = fc / (Kcf + 1);
    Y2[((f * M0 + a) * M1 + b) * (Kcf + 1) + c] = A[l * ln + pidx(b)];
  }
}

// C2R along z of the half lines Y2[f][a][b][0..Kcf] (zero above), two
// lines per complex transform; writes the real fields out[f][a][b][z].
__global__ void __launch_bounds__(256, 2)
ff_inv_z_kernel(int M0, int M1, int M2, int nf, int Kcf, const float4* Y2,
                FFPlan P, int LB, float* out, float* out_lo) {
  extern __shared__ float4 smem[];
  const int ln = padded_len(M2);
  float4* A = smem;
  const int64_t nlines = int64_t(nf) * M0 * M1;
  const int64_t npair = (nlines + 1) / 2;
  const int64_t p0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, npair - p0);
  auto half = [&](int64_t line, int k) -> FFC {
    // Hermitian extension of the half line.
    if (line >= nlines) return ffc_zero();
    const int kk = (k <= M2 / 2) ? k : M2 - k;
    if (kk > Kcf) return ffc_zero();
    const FFC v = ffc_load(Y2 + line * (Kcf + 1) + kk);
    return (k <= M2 / 2) ? v : ffc_conj(v);
  };
  for (int w = threadIdx.x; w < nl * M2; w += blockDim.x) {
    const int l = w / M2, k = w - l * M2;
    const int64_t line0 = 2 * (p0 + l);
    const FFC h1 = half(line0, k), h2 = half(line0 + 1, k);
    // Z = H1 + i H2
    A[l * ln + pidx(k)] =
        ffc_pack(FFC{ffsub(h1.re, h2.im), ffadd(h1.im, h2.re)});
  }
  ff_fft_lines(A, nl, ln, P, +1);
  for (int w = threadIdx.x; w < nl * M2; w += blockDim.x) {
    const int l = w / M2, z = w - l * M2;
    const int64_t line0 = 2 * (p0 + l);
    const float4 v = A[l * ln + pidx(z)];
    out[line0 * M2 + z] = v.x;
    out_lo[line0 * M2 + z] = v.y;
    if (line0 + 1 < nlines) {
      out[(line0 + 1) * M2 + z] = v.z;
      out_lo[(line0 + 1) * M2 + z] = v.w;
    }
  }
}

// Lines per block: every butterfly of a stage must fit the registers the
// stage keeps per thread (StageItems, 256 threads).
int lines_per_block(const FFPlan& P) {
  int lb = 16;
  for (int s = 0; s < P.nstage; ++s) {
    const int R = P.radix[s];
    const int items = (R == 8 || R == 5) ? 1 : 2;
    lb = std::min(lb, items * 256 / (P.n / R));
  }
  return std::max(1, lb);
}

size_t smem_bytes(int n, int lb) {
  return size_t(lb) * padded_len(n) * sizeof(float4);
}

// Opt in to more than 48 KB of dynamic shared memory (per launch: the
// setting belongs to the current device).
template <class K>
void allow_smem(K kernel) {
  TRVG_CUDA(cudaFuncSetAttribute(kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024));
}

}  // namespace

bool ff_length_ok(int n) {
  if (n < 2) return false;
  for (int r : {2, 3, 5})
    while (n % r == 0) n /= r;
  return n == 1;
}

FFPlan ff_plan(Context& ctx, int n) {
  FFPlan P;
  P.n = n;
  P.nstage = 0;
  int m = n;
  while (m % 8 == 0) { P.radix[P.nstage++] = 8; m /= 8; }
  while (m % 4 == 0) { P.radix[P.nstage++] = 4; m /= 4; }
  while (m % 2 == 0) { P.radix[P.nstage++] = 2; m /= 2; }
  while (m % 3 == 0) { P.radix[P.nstage++] = 3; m /= 3; }
  while (m % 5 == 0) { P.radix[P.nstage++] = 5; m /= 5; }
  if (m != 1 || P.nstage > 16)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Float-float transform length %d unsupported.", n);
  const std::string name = "fftw." + std::to_string(n);
  auto it = ctx.buffers.find(name);
  if (it != ctx.buffers.end() && it->second.bytes >= size_t(n) * sizeof(float4)) {
    P.tw = static_cast<const float4*>(it->second.ptr);
    return P;
  }
  std::vector<float4> h(n);
  for (int k = 0; k < n; ++k) {
    const double a = 2. * M_PI * double(k) / double(n);
    const double c = std::cos(a), s = std::sin(a);
    const float ch = float(c), sh = float(s);
    h[k] = make_float4(ch, float(c - double(ch)), sh, float(s - double(sh)));
  }
  float4* d = ctx.buf<float4>(name, n);
  TRVG_CUDA(cudaMemcpyAsync(d, h.data(), n * sizeof(float4),
                            cudaMemcpyHostToDevice, ctx.stream));
  TRVG_CUDA(cudaStreamSynchronize(ctx.stream));
  P.tw = d;
  return P;
}

void launch_ff_forward_cube(Context& ctx, const Geom& g, const float* mesh,
                            int Kg, float4* T1, float4* T2, float4* cube) {
  const FFPlan Pz = ff_plan(ctx, g.n[2]);
  const FFPlan Py = ff_plan(ctx, g.n[1]);
  const FFPlan Px = ff_plan(ctx, g.n[0]);
  {
    const int lb = lines_per_block(Pz);
    const int64_t npair = int64_t(g.n[0]) * g.n[1] / 2;
    allow_smem(ff_fwd_z_kernel);
    TRVG_KBEGIN(ctx, "ff_forward_kernel");
    ff_fwd_z_kernel<<<int((npair + lb - 1) / lb), 256, smem_bytes(g.n[2], lb),
                      ctx.stream>>>(g, mesh, Pz, lb, Kg, T1);
    TRVG_LAUNCHED(ctx);
  }
  {
    const int lb = lines_per_block(Py);
    const int64_t nl = int64_t(g.n[0]) * (Kg + 1);
    allow_smem(ff_fwd_y_kernel);
    TRVG_KBEGIN(ctx, "ff_forward_kernel");
    ff_fwd_y_kernel<<<int((nl + lb - 1) / lb), 256, smem_bytes(g.n[1], lb),
                      ctx.stream>>>(g, T1, Py, lb, Kg, Kg, T2);
    TRVG_LAUNCHED(ctx);
  }
  {
    const int lb = lines_per_block(Px);
    const int64_t nl = int64_t(2 * Kg + 1) * (Kg + 1);
    allow_smem(ff_fwd_x_kernel);
    TRVG_KBEGIN(ctx, "ff_forward_kernel");
    ff_fwd_x_kernel<<<int((nl + lb - 1) / lb), 256, smem_bytes(g.n[0], lb),
                      ctx.stream>>>(g, T2, Px, lb, Kg, Kg, Kg, cube);
    TRVG_LAUNCHED(ctx);
  }
}

void launch_ff_build_G(Context& ctx, const Geom& g, const int M[3],
                       const float4* cube, int Kg, const float2* const iw[3],
                       cd k0, float4* E) {
  FFBuild bd{M[0], M[1], Kg, {iw[0], iw[1], iw[2]},
             FF{float(1. / g.vol), float(1. / g.vol - double(float(1. / g.vol)))}};
  const FFC k0f{FF{float(k0.re), float(k0.re - double(float(k0.re)))},
                FF{float(k0.im), float(k0.im - double(float(k0.im)))}};
  const int64_t count = int64_t(Kg + 1) * M[1] * M[0];
  TRVG_KBEGIN(ctx, "ff_build_kernel");
  ff_build_G_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, bd, cube, Kg, k0f, E);
  TRVG_LAUNCHED(ctx);
}

void launch_ff_build_F(Context& ctx, const Geom& g, const int M[3],
                       const float4* cube, int Kg, int K, const int16_t* tab,
                       int nq, int ell, const float2* const iw[3], cd k0,
                       float4* E) {
  FFBuild bd{M[0], M[1], Kg, {iw[0], iw[1], iw[2]}, FF{0.f, 0.f}};
  const FFC k0f{FF{float(k0.re), float(k0.re - double(float(k0.re)))},
                FF{float(k0.im), float(k0.im - double(float(k0.im)))}};
  const int64_t plane = int64_t(K + 1) * M[1] * M[0];
  TRVG_CUDA(cudaMemsetAsync(E, 0, size_t(nq) * plane * sizeof(float4),
                            ctx.stream));
  TRVG_KBEGIN(ctx, "ff_build_kernel");
  ff_build_F_kernel<<<grid_for(plane, 256), 256, 0, ctx.stream>>>(
      g, bd, M[2], cube, K, tab, ell, k0f, E);
  TRVG_LAUNCHED(ctx);
}

void launch_ff_inverse(Context& ctx, const int M[3], int nf, int Kf, int Kcf,
                       const float4* E, float4* Y1, float4* Y2, float* out,
                       float* out_lo) {
  const FFPlan Px = ff_plan(ctx, M[0]);
  const FFPlan Py = ff_plan(ctx, M[1]);
  const FFPlan Pz = ff_plan(ctx, M[2]);
  {
    const int lb = lines_per_block(Px);
    const int64_t nl = int64_t(nf) * (Kcf + 1) * (2 * Kf + 1);
    allow_smem(ff_inv_x_kernel);
    TRVG_KBEGIN(ctx, "ff_inverse_kernel");
    ff_inv_x_kernel<<<int((nl + lb - 1) / lb), 256, smem_bytes(M[0], lb),
                      ctx.stream>>>(M[0], M[1], nf, Kf, Kcf, E, Px, lb, Y1);
    TRVG_LAUNCHED(ctx);
  }
  {
    const int lb = lines_per_block(Py);
    const int64_t nl = int64_t(nf) * (Kcf + 1) * M[0];
    allow_smem(ff_inv_y_kernel);
    TRVG_KBEGIN(ctx, "ff_inverse_kernel");
    ff_inv_y_kernel<<<int((nl + lb - 1) / lb), 256, smem_bytes(M[1], lb),
                      ctx.stream>>>(M[0], M[1], nf, Kf, Kcf, Y1, Py, lb, Y2);
    TRVG_LAUNCHED(ctx);
  }
  {
    const int lb = lines_per_block(Pz);
    const int64_t np = (int64_t(nf) * M[0] * M[1] + 1) / 2;
    allow_smem(ff_inv_z_kernel);
    TRVG_KBEGIN(ctx, "ff_inverse_kernel");
    ff_inv_z_kernel<<<int((np + lb - 1) / lb), 256, smem_bytes(M[2], lb),
                      ctx.stream>>>(M[0], M[1], M[2], nf, Kcf, Y2, Pz, lb,
                                    out, out_lo);
    TRVG_LAUNCHED(ctx);
  }
}

}  // namespace trvg
