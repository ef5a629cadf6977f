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
#include <type_traits>
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

// In-place DFTs of size R with root exp(D 2 pi i / R), D = +-1.
template <int D>
__device__ __forceinline__ void small_dft2(FFC* v) {
  const FFC a = v[0], b = v[1];
  v[0] = ffc_add(a, b);
  v[1] = ffc_sub(a, b);
}

template <int D>
__device__ __forceinline__ void small_dft4(FFC* v) {
  const FFC t0 = ffc_add(v[0], v[2]), t1 = ffc_sub(v[0], v[2]);
  const FFC t2 = ffc_add(v[1], v[3]);
  const FFC t3 = ffc_muli(ffc_sub(v[1], v[3]), D);
  v[0] = ffc_add(t0, t2);
  v[2] = ffc_sub(t0, t2);
  v[1] = ffc_add(t1, t3);
  v[3] = ffc_sub(t1, t3);
}

template <int D>
__device__ __forceinline__ void small_dft8(FFC* v) {
  FFC e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  small_dft4<D>(e);
  small_dft4<D>(o);
  // o_k *= exp(D 2 pi i k / 8)
  const FF c = k_rsqrt2();
  auto w1 = [&](FFC x) {
    const FF re = (D > 0) ? ffsub(x.re, x.im) : ffadd(x.re, x.im);
    const FF im = (D > 0) ? ffadd(x.im, x.re) : ffsub(x.im, x.re);
    return FFC{ffmul(re, c), ffmul(im, c)};
  };
  o[1] = w1(o[1]);
  o[2] = ffc_muli(o[2], D);
  o[3] = ffc_muli(w1(o[3]), D);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = ffc_add(e[k], o[k]);
    v[k + 4] = ffc_sub(e[k], o[k]);
  }
}

template <int D>
__device__ __forceinline__ void small_dft3(FFC* v) {
  const FFC t = ffc_add(v[1], v[2]);
  const FFC m = ffc_sub(v[0], ffc_scale2(t, 0.5f));
  const FFC u = ffc_mulr(ffc_muli(ffc_sub(v[1], v[2]), D), k_sqrt3_2());
  v[0] = ffc_add(v[0], t);
  v[1] = ffc_add(m, u);
  v[2] = ffc_sub(m, u);
}

template <int D>
__device__ __forceinline__ void small_dft5(FFC* v) {
  const FFC t1 = ffc_add(v[1], v[4]), t2 = ffc_add(v[2], v[3]);
  const FFC t3 = ffc_sub(v[1], v[4]), t4 = ffc_sub(v[2], v[3]);
  const FF c1 = k_c1_5(), c2 = k_c2_5(), s1 = k_s1_5(), s2 = k_s2_5();
  const FFC b1 = ffc_add(v[0], ffc_add(ffc_mulr(t1, c1), ffc_mulr(t2, c2)));
  const FFC b2 = ffc_add(v[0], ffc_add(ffc_mulr(t1, c2), ffc_mulr(t2, c1)));
  const FFC b3 =
      ffc_muli(ffc_add(ffc_mulr(t3, s1), ffc_mulr(t4, s2)), D);
  const FFC b4 =
      ffc_muli(ffc_sub(ffc_mulr(t3, s2), ffc_mulr(t4, s1)), D);
  v[0] = ffc_add(v[0], ffc_add(t1, t2));
  v[1] = ffc_add(b1, b3);
  v[4] = ffc_sub(b1, b3);
  v[2] = ffc_add(b2, b4);
  v[3] = ffc_sub(b2, b4);
}

template <int R, int D>
__device__ __forceinline__ void small_dft(FFC* v) {
  if constexpr (R == 2) small_dft2<D>(v);
  else if constexpr (R == 4) small_dft4<D>(v);
  else if constexpr (R == 8) small_dft8<D>(v);
  else if constexpr (R == 3) small_dft3<D>(v);
  else small_dft5<D>(v);
}

// Shared-memory slot of element i of a line: one pad slot per 8 elements,
// so that the stride-R accesses of a stage spread over the bank groups of
// the 16-byte elements.
__host__ __device__ __forceinline__ int pidx(int i) { return i + (i >> 3); }
__host__ __device__ __forceinline__ int padded_len(int n) {
  return pidx(n - 1) + 1;
}
// Distance between the lines of a block: odd, so that the same element of
// consecutive lines falls in different bank groups.
__host__ __device__ __forceinline__ int line_stride(int n) {
  return padded_len(n) | 1;
}
// Lines per block at most (per-line offsets are kept in shared memory).
constexpr int kMaxLines = 16;

// Radix sets of a plan (bit per radix); kernels specialised for a set
// inline its stages, the generic ones (kRadixAll) call them out of line, so
// that each stage keeps its own register allocation.
constexpr int kRadix8 = 1, kRadix4 = 2, kRadix2 = 4, kRadix3 = 8,
              kRadix5 = 16, kRadixAll = 31;

// Butterflies one thread keeps in registers per stage.
template <int R>
struct StageItems {
  static constexpr int value = R == 8 || R == 5 ? 1 : 2;
};

// Quotient of w by d through the plan's multiplier (w, d small: see FFPlan).
__device__ __forceinline__ int fdiv(int w, int d, unsigned m) {
  return d == 1 ? w : int(__umulhi(unsigned(w), m));
}

// One Stockham stage of radix R (stage s of the plan) over the nl lines of
// A (padded line length ln), in place: every thread loads and transforms
// its butterflies, the block synchronises, then every thread writes its
// results.
template <int R, int D>
__device__ __forceinline__ void ff_stage_body(float4* A, int nl, int ln,
                                      const FFPlan& P, int s,
                                      const float4* tw) {
  constexpr int IMAX = StageItems<R>::value;
  const int nb = P.nb[s], Ns = P.ns[s];
  const unsigned mnb = P.mnb[s], mns = P.mns[s];
  const int items = nl * nb;
  FFC v[IMAX][R];
#pragma unroll
  for (int it = 0; it < IMAX; ++it) {
    const int w = threadIdx.x + it * blockDim.x;
    if (w >= items) break;
    const int l = fdiv(w, nb, mnb), j = w - l * nb;
    const int q = fdiv(j, Ns, mns), k = j - q * Ns;
    const float4* in = A + l * ln;
    const int tb = P.twoff[s] - Ns + k;  // + r Ns: entry (r - 1) Ns + k
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[it][r] = ffc_load(in + pidx(j + r * nb));
      if (r > 0 && k > 0) {
        const float4 t = tw[tb + r * Ns];
        FFC wv{FF{t.x, t.y}, FF{t.z, t.w}};
        if (D < 0) wv.im = ffneg(wv.im);
        v[it][r] = ffc_mul(v[it][r], wv);
      }
    }
    small_dft<R, D>(v[it]);
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IMAX; ++it) {
    const int w = threadIdx.x + it * blockDim.x;
    if (w >= items) break;
    const int l = fdiv(w, nb, mnb), j = w - l * nb;
    const int q = fdiv(j, Ns, mns), k = j - q * Ns;
    float4* out = A + l * ln;
    const int idx = q * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) ffc_store(out + pidx(idx + r * Ns), v[it][r]);
  }
  __syncthreads();
}

// Blocks per SM the inverse passes are compiled for: the radix sets whose
// kernels fit fewer registers without spills (checked with -Xptxas -v:
// {3, 5} in 80 registers, its z pass in 64; {2, 3} in 79) run more warps
// per SM; the others need up to 128 registers.
template <int MASK, bool ZPASS>
constexpr int inv_min_blocks() {
  return MASK == (kRadix3 | kRadix5) ? (ZPASS ? 4 : 3)
         : MASK == (kRadix2 | kRadix3) ? 3
                                       : 2;
}

// Butterflies per lane when one warp transforms a line: two of radix 8 in
// plans of radix 8 alone (n = 512 has 64 per stage), where the kernels
// still fit 128 registers without spills; one in mixed plans.
template <int R, int MASK>
struct WarpItems {
  static constexpr int value =
      R == 8 ? (MASK == kRadix8 ? 2 : 1) : (R == 5 ? 1 : (R == 2 ? 3 : 2));
};

// One stage of radix R over the line L of this warp (same indexing as
// ff_stage, butterfly j = lane + 32 it), synchronised within the warp only.
template <int R, int D, int MASK>
__device__ __forceinline__ void ff_stage_warp_body(float4* L, const FFPlan& P,
                                                   int s, const float4* tw) {
  constexpr int IMAX = WarpItems<R, MASK>::value;
  const int nb = P.nb[s], Ns = P.ns[s];
  const unsigned mns = P.mns[s];
  const int lane = threadIdx.x & 31;
  FFC v[IMAX][R];
#pragma unroll
  for (int it = 0; it < IMAX; ++it) {
    const int j = lane + 32 * it;
    if (j >= nb) break;
    const int k = j - fdiv(j, Ns, mns) * Ns;
    const int tb = P.twoff[s] - Ns + k;  // + r Ns: entry (r - 1) Ns + k
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[it][r] = ffc_load(L + pidx(j + r * nb));
      if (r > 0 && k > 0) {
        const float4 t = tw[tb + r * Ns];
        FFC wv{FF{t.x, t.y}, FF{t.z, t.w}};
        if (D < 0) wv.im = ffneg(wv.im);
        v[it][r] = ffc_mul(v[it][r], wv);
      }
    }
    small_dft<R, D>(v[it]);
  }
  __syncwarp();
#pragma unroll
  for (int it = 0; it < IMAX; ++it) {
    const int j = lane + 32 * it;
    if (j >= nb) break;
    const int q = fdiv(j, Ns, mns), k = j - q * Ns;
    const int idx = q * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) ffc_store(L + pidx(idx + r * Ns), v[it][r]);
  }
  __syncwarp();
}

// Transforms the nl lines of A (line stride ln) in place, direction D,
// with the twiddle table tw (n entries, usually a shared-memory copy).

template <int R, int D>
__device__ __noinline__ void ff_stage_call(float4* A, int nl, int ln,
                                           const FFPlan& P, int s,
                                           const float4* tw) {
  ff_stage_body<R, D>(A, nl, ln, P, s, tw);
}
template <int R, int D>
__device__ __noinline__ void ff_stage_warp_call(float4* L, const FFPlan& P,
                                                int s, const float4* tw) {
  ff_stage_warp_body<R, D, kRadixAll>(L, P, s, tw);
}

template <int R, int D, int MASK>
__device__ __forceinline__ void ff_stage(float4* A, int nl, int ln,
                                         const FFPlan& P, int s,
                                         const float4* tw) {
  if constexpr (MASK == kRadixAll) ff_stage_call<R, D>(A, nl, ln, P, s, tw);
  else ff_stage_body<R, D>(A, nl, ln, P, s, tw);
}
template <int R, int D, int MASK>
__device__ __forceinline__ void ff_stage_warp(float4* L, const FFPlan& P,
                                              int s, const float4* tw) {
  if constexpr (MASK == kRadixAll) ff_stage_warp_call<R, D>(L, P, s, tw);
  else ff_stage_warp_body<R, D, MASK>(L, P, s, tw);
}

// Transforms the nl lines of A (line stride ln) in place, direction D,
// with the twiddle table tw (n entries, a shared-memory copy).  The plan
// orders its stages by radix (8, 4, 2, 3, 5); MASK holds every radix of
// the plan.
template <int D, int MASK>
__device__ void ff_fft_lines(float4* A, int nl, int ln, const FFPlan& P,
                             const float4* tw) {
  __syncthreads();
  if (P.warp_lines) {
    for (int l = threadIdx.x >> 5; l < nl; l += blockDim.x >> 5) {
      float4* L = A + l * ln;
      int s = 0;
      if constexpr ((MASK & kRadix8) != 0)
        for (; s < P.nstage && P.radix[s] == 8; ++s)
          ff_stage_warp<8, D, MASK>(L, P, s, tw);
      if constexpr ((MASK & kRadix4) != 0)
        for (; s < P.nstage && P.radix[s] == 4; ++s)
          ff_stage_warp<4, D, MASK>(L, P, s, tw);
      if constexpr ((MASK & kRadix2) != 0)
        for (; s < P.nstage && P.radix[s] == 2; ++s)
          ff_stage_warp<2, D, MASK>(L, P, s, tw);
      if constexpr ((MASK & kRadix3) != 0)
        for (; s < P.nstage && P.radix[s] == 3; ++s)
          ff_stage_warp<3, D, MASK>(L, P, s, tw);
      if constexpr ((MASK & kRadix5) != 0)
        for (; s < P.nstage; ++s) ff_stage_warp<5, D, MASK>(L, P, s, tw);
    }
    __syncthreads();
    return;
  }
  int s = 0;
  if constexpr ((MASK & kRadix8) != 0)
    for (; s < P.nstage && P.radix[s] == 8; ++s)
      ff_stage<8, D, MASK>(A, nl, ln, P, s, tw);
  if constexpr ((MASK & kRadix4) != 0)
    for (; s < P.nstage && P.radix[s] == 4; ++s)
      ff_stage<4, D, MASK>(A, nl, ln, P, s, tw);
  if constexpr ((MASK & kRadix2) != 0)
    for (; s < P.nstage && P.radix[s] == 2; ++s)
      ff_stage<2, D, MASK>(A, nl, ln, P, s, tw);
  if constexpr ((MASK & kRadix3) != 0)
    for (; s < P.nstage && P.radix[s] == 3; ++s)
      ff_stage<3, D, MASK>(A, nl, ln, P, s, tw);
  if constexpr ((MASK & kRadix5) != 0)
    for (; s < P.nstage; ++s) ff_stage<5, D, MASK>(A, nl, ln, P, s, tw);
}

// Shared-memory copy of the plan's twiddles after the nl lines of a block.
__device__ __forceinline__ const float4* stage_twiddles(float4* smem,
                                                        int LB, int ls,
                                                        const FFPlan& P) {
  float4* tw = smem + LB * ls;
  for (int i = threadIdx.x; i < P.n; i += blockDim.x) tw[i] = P.tw[i];
  return tw;
}

// Global-memory form: canonical float-float words.
__device__ __forceinline__ float4 ffc_pack(FFC a) {
  a = ffc_norm(a);
  return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo);
}

// ---- Forward cube ----------------------------------------------------------

// Element loops of the passes: loads run one warp per line along the
// contiguous axis; stores that transpose run with the line index fastest
// (the lines of a block are consecutive in the output), over the next power
// of two of the line count.  Per-line offsets are computed once per block.
__device__ __forceinline__ int lines_shift(int nl) {
  return nl <= 1 ? 0 : 32 - __clz(nl - 1);
}

// z lines of the real mesh, two rows per complex line; keeps kz in [0, Kz]
// into T1[x][kz][y] and, when `full` is set, every kz in [0, n2 / 2] of
// every row rounded to FP32 into full[kz][x][y] (planes of the mesh's
// transform along z, which batched x-y transforms complete).
template <int MASK>
__global__ void __launch_bounds__(256, 2)
ff_fwd_z_kernel(Geom g, const float* mesh, const float* mesh_lo,
                __grid_constant__ const FFPlan P, int LB, int Kz,
                float4* T1, float2* full) {
  extern __shared__ float4 smem[];
  __shared__ int64_t obase[2 * kMaxLines];
  const int n2 = g.n[2], ls = line_stride(n2);
  float4* A = smem;
  const float4* tw = stage_twiddles(smem, LB, ls, P);
  const int64_t npair = int64_t(g.n[0]) * g.n[1] / 2;
  const int64_t p0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, npair - p0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  if (threadIdx.x < 2 * nl) {
    const int64_t r = 2 * p0 + threadIdx.x;  // row = x n1 + y
    const int64_t x = r / g.n[1], y = r - x * g.n[1];
    obase[threadIdx.x] = x * (Kz + 1) * g.n[1] + y;
  }
  for (int l = warp; l < nl; l += nw) {
    const float* row = mesh + 2 * (p0 + l) * n2;
    if (mesh_lo != nullptr) {
      // Compensated mesh: each cell is the float-float value hi + lo.
      const float* rlo = mesh_lo + 2 * (p0 + l) * n2;
      for (int i = lane; i < n2; i += 32)
        A[l * ls + pidx(i)] =
            make_float4(row[i], rlo[i], row[n2 + i], rlo[n2 + i]);
    } else {
      for (int i = lane; i < n2; i += 32)
        A[l * ls + pidx(i)] = make_float4(row[i], 0.f, row[n2 + i], 0.f);
    }
  }
  ff_fft_lines<-1, MASK>(A, nl, ls, P, tw);
  const int sh = lines_shift(2 * nl);
  for (int w = threadIdx.x; w < (Kz + 1) << sh; w += blockDim.x) {
    const int t = w & ((1 << sh) - 1), kz = w >> sh;
    if (t >= 2 * nl) continue;
    const int l = t >> 1;
    const FFC z = ffc_load(A + l * ls + pidx(kz));
    const FFC zm = ffc_conj(
        ffc_load(A + l * ls + pidx(kz == 0 ? 0 : n2 - kz)));
    // rows 2l and 2l + 1: (Z(k) + conj Z(-k)) / 2 and (Z(k) - conj Z(-k)) / 2i
    const FFC v = (t & 1) ? ffc_scale2(ffc_muli(ffc_sub(z, zm), -1), 0.5f)
                          : ffc_scale2(ffc_add(z, zm), 0.5f);
    T1[obase[t] + int64_t(kz) * g.n[1]] = ffc_pack(v);
  }
  if (full != nullptr) {
    // Both rows of line l at kz, from Z(k) and conj Z(-k) rounded to FP32,
    // plane by plane: full[kz][row].  The two rows are adjacent in a plane
    // (one 16-byte store); consecutive threads write the block's
    // consecutive lines of one plane.
    const int nzh = n2 / 2 + 1;
    const int64_t nrows = int64_t(g.n[0]) * g.n[1];
    const int shl = lines_shift(nl);
    for (int w = threadIdx.x; w < nzh << shl; w += blockDim.x) {
      const int l = w & ((1 << shl) - 1), kz = w >> shl;
      if (l >= nl) continue;
      const float4 a = A[l * ls + pidx(kz)];
      const float4 b = A[l * ls + pidx(kz == 0 ? 0 : n2 - kz)];
      const float zr = a.x + a.y, zi = a.z + a.w;
      const float mr = b.x + b.y, mi = -(b.z + b.w);
      reinterpret_cast<float4*>(full + int64_t(kz) * nrows)[p0 + l] =
          make_float4(0.5f * (zr + mr), 0.5f * (zi + mi), 0.5f * (zi - mi),
                      -0.5f * (zr - mr));
    }
  }
}

// y lines of T1, ordered kz * n0 + x; keeps sy in [-Ky, Ky] into
// T2[sy + Ky][kz][x].
template <int MASK>
__global__ void __launch_bounds__(256, 2)
ff_fwd_y_kernel(Geom g, const float4* T1, __grid_constant__ const FFPlan P,
                int LB, int Ky, int Kz, float4* T2) {
  extern __shared__ float4 smem[];
  __shared__ int64_t ibase[kMaxLines], obase[kMaxLines];
  const int n1 = g.n[1], ls = line_stride(n1);
  float4* A = smem;
  const float4* tw = stage_twiddles(smem, LB, ls, P);
  const int64_t nlines = int64_t(g.n[0]) * (Kz + 1);
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  if (threadIdx.x < nl) {
    const int64_t line = l0 + threadIdx.x;
    const int64_t kz = line / g.n[0], x = line - kz * g.n[0];
    ibase[threadIdx.x] = (x * (Kz + 1) + kz) * n1;
    obase[threadIdx.x] = line;  // kz * n0 + x
  }
  __syncthreads();
  for (int l = warp; l < nl; l += nw) {
    const float4* src = T1 + ibase[l];
    for (int i = lane; i < n1; i += 32) A[l * ls + pidx(i)] = src[i];
  }
  ff_fft_lines<-1, MASK>(A, nl, ls, P, tw);
  const int sh = lines_shift(nl);
  const int64_t plane = int64_t(Kz + 1) * g.n[0];
  for (int w = threadIdx.x; w < (2 * Ky + 1) << sh; w += blockDim.x) {
    const int l = w & ((1 << sh) - 1), b = w >> sh;
    if (l >= nl) continue;
    T2[obase[l] + b * plane] = A[l * ls + pidx(wrapi(b - Ky, n1))];
  }
}

// x lines (sy, kz) of T2; keeps sx in [-Kx, Kx] into
// cube[sx + Kx][sy + Ky][kz].
template <int MASK>
__global__ void __launch_bounds__(256, 2)
ff_fwd_x_kernel(Geom g, const float4* T2, __grid_constant__ const FFPlan P,
                int LB, int Kx, int Ky, int Kz, float4* cube) {
  extern __shared__ float4 smem[];
  const int n0 = g.n[0], ls = line_stride(n0);
  float4* A = smem;
  const float4* tw = stage_twiddles(smem, LB, ls, P);
  const int64_t nlines = int64_t(2 * Ky + 1) * (Kz + 1);
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  for (int l = warp; l < nl; l += nw) {
    const float4* src = T2 + (l0 + l) * n0;
    for (int i = lane; i < n0; i += 32) A[l * ls + pidx(i)] = src[i];
  }
  ff_fft_lines<-1, MASK>(A, nl, ls, P, tw);
  const int sh = lines_shift(nl);
  for (int w = threadIdx.x; w < (2 * Kx + 1) << sh; w += blockDim.x) {
    const int l = w & ((1 << sh) - 1), a = w >> sh;
    if (l >= nl) continue;
    // line = (sy + Ky) (Kz + 1) + kz
    cube[int64_t(a) * nlines + l0 + l] = A[l * ls + pidx(wrapi(a - Kx, n0))];
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
__device__ __forceinline__ FFC k0_value(FFC k0, const double* k0_dev) {
  return k0_dev != nullptr
             ? FFC{ff_from_double(k0_dev[0]), ff_from_double(k0_dev[1])}
             : k0;
}

__global__ void ff_build_G_kernel(Geom g, FFBuild bd, const float4* cube,
                                  int Kg, FFC k0h, const double* k0_dev,
                                  float4* E) {
  const FFC k0 = k0_value(k0h, k0_dev);
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
                                  int K, const int16_t* tab, int ell, FFC k0h,
                                  const double* k0_dev, float4* E) {
  const FFC k0 = k0_value(k0h, k0_dev);
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

// x lines (f, c, b in band; only the listed ones when band.xl is set) of
// E[f][c][b][a]; writes Y1[f][c][a][b].
template <int MASK>
__global__ void __launch_bounds__(256, inv_min_blocks<MASK, false>())
ff_inv_x_kernel(int M0, int M1, int nf, int Kf, int Kcf, const float4* E,
                __grid_constant__ const FFPlan P, int LB, float4* Y1,
                FFBand band) {
  extern __shared__ float4 smem[];
  __shared__ int64_t ibase[kMaxLines], obase[kMaxLines];
  const int ls = line_stride(M0);
  float4* A = smem;
  const float4* tw = stage_twiddles(smem, LB, ls, P);
  const int nb = 2 * Kf + 1;
  const int64_t nlines =
      band.xl != nullptr ? band.nxl : int64_t(nf) * (Kcf + 1) * nb;
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  if (threadIdx.x < nl) {
    const int64_t line = band.xl != nullptr
                             ? int64_t(band.xl[l0 + threadIdx.x])
                             : l0 + threadIdx.x;
    const int64_t fc = line / nb;  // f (Kcf + 1) + c
    const int b = wrapi(int(line - fc * nb) - Kf, M1);
    ibase[threadIdx.x] = (fc * M1 + b) * M0;
    obase[threadIdx.x] = fc * M0 * M1 + b;
  }
  __syncthreads();
  for (int l = warp; l < nl; l += nw) {
    const float4* src = E + ibase[l];
    for (int a = lane; a < M0; a += 32) A[l * ls + pidx(a)] = src[a];
  }
  ff_fft_lines<+1, MASK>(A, nl, ls, P, tw);
  const int sh = lines_shift(nl);
  for (int w = threadIdx.x; w < M0 << sh; w += blockDim.x) {
    const int l = w & ((1 << sh) - 1), a = w >> sh;
    if (l >= nl) continue;
    Y1[obase[l] + int64_t(a) * M1] = A[l * ls + pidx(a)];
  }
}

// y lines of Y1 (entries outside the band, or outside the x lines that
// band lists, are zero), ordered (f M0 + a) (Kcf + 1) + c, or with
// band.yoff set field by field over the planes c <= kz[f]; writes
// Y2[f][a][b][c].
template <int MASK>
__global__ void __launch_bounds__(256, inv_min_blocks<MASK, false>())
ff_inv_y_kernel(int M0, int M1, int nf, int Kf, int Kcf, const float4* Y1,
                __grid_constant__ const FFPlan P, int LB, float4* Y2,
                FFBand band) {
  extern __shared__ float4 smem[];
  __shared__ int64_t ibase[kMaxLines], obase[kMaxLines];
  __shared__ int lbm[kMaxLines];
  const int ls = line_stride(M1);
  float4* A = smem;
  const float4* tw = stage_twiddles(smem, LB, ls, P);
  const int64_t nlines =
      band.yoff != nullptr ? band.nyl : int64_t(nf) * (Kcf + 1) * M0;
  const int64_t l0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, nlines - l0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  if (threadIdx.x < nl) {
    const int64_t line = l0 + threadIdx.x;
    int64_t f, a, c;
    int bmax = Kf;
    if (band.yoff != nullptr) {
      // The last field whose lines start at or before this one (a field
      // has at least its plane c = 0, so it owns the line).
      int lo = 0, hi = nf;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (band.yoff[mid] <= line) lo = mid;
        else hi = mid;
      }
      f = lo;
      const int64_t r = line - band.yoff[f];
      const int64_t kc = band.kz[f] + 1;
      a = r / kc;
      c = r - a * kc;
      bmax = band.bm[f * (Kcf + 1) + c];
    } else {
      const int64_t fa = line / (Kcf + 1);
      c = line - fa * (Kcf + 1);
      f = fa / M0;
      a = fa - f * M0;
    }
    ibase[threadIdx.x] = ((f * (Kcf + 1) + c) * M0 + a) * M1;
    obase[threadIdx.x] = (f * M0 + a) * M1 * (Kcf + 1) + c;
    lbm[threadIdx.x] = bmax;
  }
  __syncthreads();
  for (int l = warp; l < nl; l += nw) {
    const float4* src = Y1 + ibase[l];
    const int bmax = lbm[l];
    for (int b = lane; b < M1; b += 32)
      A[l * ls + pidx(b)] = (abs(sym_shift(b, M1)) <= bmax)
                                ? src[b]
                                : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  ff_fft_lines<+1, MASK>(A, nl, ls, P, tw);
  const int sh = lines_shift(nl);
  for (int w = threadIdx.x; w < M1 << sh; w += blockDim.x) {
    const int l = w & ((1 << sh) - 1), b = w >> sh;
    if (l >= nl) continue;
    Y2[obase[l] + int64_t(b) * (Kcf + 1)] = A[l * ls + pidx(b)];
  }
}

// C2R along z of the half lines Y2[f][a][b][0..Kcf] (zero above), two
// lines per complex transform; writes the real fields out[f][a][b][z]
// (hi words, correctly rounded) and their lo words unless out_lo is null.
template <int MASK>
__global__ void __launch_bounds__(256, inv_min_blocks<MASK, true>())
ff_inv_z_kernel(int M0, int M1, int M2, int nf, int Kcf, const float4* Y2,
                __grid_constant__ const FFPlan P, int LB, float* out,
                float* out_lo, int64_t ld, const int* kz) {
  extern __shared__ float4 smem[];
  const int ls = line_stride(M2);
  float4* A = smem;
  const float4* tw = stage_twiddles(smem, LB, ls, P);
  const int64_t nlines = int64_t(nf) * M0 * M1;
  const int64_t npair = (nlines + 1) / 2;
  const int64_t p0 = int64_t(blockIdx.x) * LB;
  const int nl = min_lines(LB, npair - p0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int64_t plane = int64_t(M0) * M1;  // lines per field
  for (int l = warp; l < nl; l += nw) {
    const int64_t line0 = 2 * (p0 + l);
    const bool two = line0 + 1 < nlines;
    const float4* h1 = Y2 + line0 * (Kcf + 1);
    const float4* h2 = h1 + (Kcf + 1);
    // Planes above a field's last shell plane were not written (zero).
    int kz1 = Kcf, kz2 = Kcf;
    if (kz != nullptr) {
      kz1 = kz[line0 / plane];
      if (two) kz2 = kz[(line0 + 1) / plane];
    }
    for (int k = lane; k < M2; k += 32) {
      // Hermitian extension of the half lines; Z = H1 + i H2.
      const bool up = k <= M2 / 2;
      const int kk = up ? k : M2 - k;
      FFC a = ffc_zero(), b = ffc_zero();
      if (kk <= Kcf) {
        if (kk <= kz1) a = ffc_load(h1 + kk);
        if (two && kk <= kz2) b = ffc_load(h2 + kk);
        if (!up) {
          a = ffc_conj(a);
          b = ffc_conj(b);
        }
      }
      A[l * ls + pidx(k)] =
          ffc_pack(FFC{ffsub(a.re, b.im), ffadd(a.im, b.re)});
    }
  }
  ff_fft_lines<+1, MASK>(A, nl, ls, P, tw);
  auto offset = [&](int64_t line) {
    const int64_t f = line / plane;
    return f * ld + (line - f * plane) * M2;
  };
  for (int l = warp; l < nl; l += nw) {
    const int64_t line0 = 2 * (p0 + l);
    const bool two = line0 + 1 < nlines;
    const int64_t o0 = offset(line0), o1 = two ? offset(line0 + 1) : 0;
    for (int z = lane; z < M2; z += 32) {
      const float4 v = A[l * ls + pidx(z)];
      const FF re = ffnorm(FF{v.x, v.y}), im = ffnorm(FF{v.z, v.w});
      out[o0 + z] = re.hi;
      if (out_lo != nullptr) out_lo[o0 + z] = re.lo;
      if (two) {
        out[o1 + z] = im.hi;
        if (out_lo != nullptr) out_lo[o1 + z] = im.lo;
      }
    }
  }
}

// Lines per block: every butterfly of a stage must fit the registers the
// stage keeps per thread (StageItems, 256 threads).
int lines_per_block(const FFPlan& P) {
  if (P.warp_lines) return 8;  // one line per warp of the 256 threads
  int lb = kMaxLines;
  for (int s = 0; s < P.nstage; ++s) {
    const int R = P.radix[s];
    const int items = (R == 8 || R == 5) ? 1 : 2;
    lb = std::min(lb, items * 256 / (P.n / R));
  }
  return std::max(1, lb);
}

size_t smem_bytes(int n, int lb) {
  return (size_t(lb) * line_stride(n) + n) * sizeof(float4);
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
  auto magic = [](int dv) {
    return dv <= 1 ? 0u : unsigned((uint64_t(1) << 32) / uint64_t(dv) + 1);
  };
  for (int s = 0, ns = 1; s < P.nstage; ns *= P.radix[s], ++s) {
    P.nb[s] = n / P.radix[s];
    P.ns[s] = ns;
    P.tstep[s] = n / (ns * P.radix[s]);
    P.mnb[s] = magic(P.nb[s]);
    P.mns[s] = magic(ns);
  }
  P.warp_lines = true;
  bool pure8 = true;
  for (int s = 0; s < P.nstage; ++s) pure8 = pure8 && P.radix[s] == 8;
  for (int s = 0; s < P.nstage; ++s) {
    const int R = P.radix[s];
    // WarpItems of the kernel this plan's radix set selects.
    const int items = R == 8 ? (pure8 ? 2 : 1) : (R == 5 ? 1 : (R == 2 ? 3 : 2));
    if (P.nb[s] > 32 * items) P.warp_lines = false;
  }
  // Stage-major twiddle table: sum over stages of (radix - 1) ns = n - 1
  // entries.
  int off = 0;
  for (int s = 0; s < P.nstage; ++s) {
    P.twoff[s] = off;
    off += (P.radix[s] - 1) * P.ns[s];
  }
  const std::string name = "fftw.staged." + std::to_string(n);
  auto it = ctx.buffers.find(name);
  if (it != ctx.buffers.end() && it->second.bytes >= size_t(n) * sizeof(float4)) {
    P.tw = static_cast<const float4*>(it->second.ptr);
    return P;
  }
  std::vector<float4> h(n, make_float4(1.f, 0.f, 0.f, 0.f));
  for (int s = 0; s < P.nstage; ++s)
    for (int r = 1; r < P.radix[s]; ++r)
      for (int k = 0; k < P.ns[s]; ++k) {
        // exp(2 pi i e / n) with e = r k tstep < n; direction D < 0 takes
        // the conjugate in the stage bodies.
        const int64_t e = int64_t(r) * k * P.tstep[s];
        const double a = 2. * M_PI * double(e) / double(n);
        const double c = std::cos(a), sn = std::sin(a);
        const float ch = float(c), sh = float(sn);
        h[P.twoff[s] + (r - 1) * P.ns[s] + k] =
            make_float4(ch, float(c - double(ch)), sh, float(sn - double(sh)));
      }
  float4* d = ctx.buf<float4>(name, n);
  TRVG_CUDA(cudaMemcpyAsync(d, h.data(), n * sizeof(float4),
                            cudaMemcpyHostToDevice, ctx.stream));
  TRVG_CUDA(cudaStreamSynchronize(ctx.stream));
  P.tw = d;
  return P;
}

namespace {

int radix_mask(const FFPlan& P) {
  int m = 0;
  for (int s = 0; s < P.nstage; ++s)
    switch (P.radix[s]) {
      case 8: m |= kRadix8; break;
      case 4: m |= kRadix4; break;
      case 2: m |= kRadix2; break;
      case 3: m |= kRadix3; break;
      default: m |= kRadix5; break;
    }
  return m;
}

template <int M>
using RadixSet = std::integral_constant<int, M>;

// Calls f with the specialised radix set that holds all radices of P, or
// the generic kernels.  Mesh passes (forward) see power-of-two lengths and
// 3 * 2^k; evaluation-grid passes (inverse) the 5-smooth lengths of
// good_fft_size.
template <int... SETS>
struct RadixSets {};

template <class F, int FIRST, int... REST>
void dispatch_radix(int m, F&& f, RadixSets<FIRST, REST...>) {
  if ((m & ~FIRST) == 0) f(RadixSet<FIRST>{});
  else dispatch_radix(m, f, RadixSets<REST...>{});
}
template <class F>
void dispatch_radix(int, F&& f, RadixSets<>) {
  f(RadixSet<kRadixAll>{});
}

template <class F>
void with_mesh_radix_set(const FFPlan& P, F&& f) {
  dispatch_radix(radix_mask(P), f,
                 RadixSets<kRadix8, kRadix8 | kRadix4, kRadix8 | kRadix2,
                           kRadix8 | kRadix2 | kRadix3>{});
}

template <class F>
void with_grid_radix_set(const FFPlan& P, F&& f) {
  // Plans of radix 8 alone take the kRadix8 kernels here too: their warp
  // form keeps two butterflies per lane (WarpItems), which ff_plan assumes.
  dispatch_radix(radix_mask(P), f,
                 RadixSets<kRadix8, kRadix3 | kRadix5, kRadix2 | kRadix3,
                           kRadix8 | kRadix4 | kRadix5,
                           kRadix8 | kRadix2 | kRadix5,
                           kRadix4 | kRadix3 | kRadix5,
                           kRadix8 | kRadix2 | kRadix3,
                           kRadix2 | kRadix3 | kRadix5>{});
}

}  // namespace

// spec[x][y][kz] = planes[kz][x][y] (kz < nz): 32 x 32 tiles of (kz, y)
// per x through shared memory, both sides coalesced.
__global__ void __launch_bounds__(256)
planes_to_half_kernel(int n0, int n1, int nz, const float2* __restrict__ planes,
                      float2* __restrict__ spec) {
  __shared__ float2 tile[32][33];
  const int x = blockIdx.z;
  const int y0 = blockIdx.x * 32, z0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int64_t plane = int64_t(n0) * n1;
  for (int j = ty; j < 32; j += 8) {
    const int z = z0 + j, y = y0 + tx;
    if (z < nz && y < n1)
      tile[j][tx] = planes[int64_t(z) * plane + int64_t(x) * n1 + y];
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int y = y0 + j, z = z0 + tx;
    if (z < nz && y < n1)
      spec[(int64_t(x) * n1 + y) * nz + z] = tile[tx][j];
  }
}

void launch_planes_to_half(Context& ctx, const Geom& g, const float2* planes,
                           float2* spec) {
  const int nz = g.n[2] / 2 + 1;
  dim3 grid((g.n[1] + 31) / 32, (nz + 31) / 32, g.n[0]);
  TRVG_KBEGIN(ctx, "planes_to_half_kernel");
  planes_to_half_kernel<<<grid, 256, 0, ctx.stream>>>(g.n[0], g.n[1], nz,
                                                      planes, spec);
  TRVG_LAUNCHED(ctx);
}

void launch_ff_forward_cube(Context& ctx, const Geom& g, const float* mesh,
                            const float* mesh_lo, int Kg, float4* T1,
                            float4* T2, float4* cube, float2* full,
                            cudaEvent_t after_z) {
  const FFPlan Pz = ff_plan(ctx, g.n[2]);
  const FFPlan Py = ff_plan(ctx, g.n[1]);
  const FFPlan Px = ff_plan(ctx, g.n[0]);
  with_mesh_radix_set(Pz, [&](auto set) {
    constexpr int MASK = decltype(set)::value;
    const int lb = lines_per_block(Pz);
    const int64_t npair = int64_t(g.n[0]) * g.n[1] / 2;
    allow_smem(ff_fwd_z_kernel<MASK>);
    TRVG_KBEGIN(ctx, "ff_fwd_z_kernel");
    ff_fwd_z_kernel<MASK><<<int((npair + lb - 1) / lb), 256,
                            smem_bytes(g.n[2], lb), ctx.stream>>>(
        g, mesh, mesh_lo, Pz, lb, Kg, T1, full);
    TRVG_LAUNCHED(ctx);
  });
  if (after_z != nullptr) TRVG_CUDA(cudaEventRecord(after_z, ctx.stream));
  with_mesh_radix_set(Py, [&](auto set) {
    constexpr int MASK = decltype(set)::value;
    const int lb = lines_per_block(Py);
    const int64_t nl = int64_t(g.n[0]) * (Kg + 1);
    allow_smem(ff_fwd_y_kernel<MASK>);
    TRVG_KBEGIN(ctx, "ff_fwd_y_kernel");
    ff_fwd_y_kernel<MASK><<<int((nl + lb - 1) / lb), 256,
                            smem_bytes(g.n[1], lb), ctx.stream>>>(
        g, T1, Py, lb, Kg, Kg, T2);
    TRVG_LAUNCHED(ctx);
  });
  with_mesh_radix_set(Px, [&](auto set) {
    constexpr int MASK = decltype(set)::value;
    const int lb = lines_per_block(Px);
    const int64_t nl = int64_t(2 * Kg + 1) * (Kg + 1);
    allow_smem(ff_fwd_x_kernel<MASK>);
    TRVG_KBEGIN(ctx, "ff_fwd_x_kernel");
    ff_fwd_x_kernel<MASK><<<int((nl + lb - 1) / lb), 256,
                            smem_bytes(g.n[0], lb), ctx.stream>>>(
        g, T2, Px, lb, Kg, Kg, Kg, cube);
    TRVG_LAUNCHED(ctx);
  });
}

// The cube's modes rounded once to FP32, written at their places in a half
// spectrum of the mesh (the R2C output layout); entries off the cube are
// left as they are.
__global__ void ff_cube_to_half_kernel(Geom g, const float4* cube, int Kg,
                                       float2* h) {
  const int w = 2 * Kg + 1;
  const int64_t count = int64_t(w) * w * (Kg + 1);
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < count;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int sz = int(t % (Kg + 1));
    const int64_t r = t / (Kg + 1);
    const int sy = int(r % w) - Kg, sx = int(r / w) - Kg;
    const float4 v = cube[t];
    h[(int64_t(wrapi(sx, g.n[0])) * g.n[1] + wrapi(sy, g.n[1])) * g.nzh +
      sz] = make_float2(v.x + v.y, v.z + v.w);
  }
}

void launch_ff_cube_to_half(Context& ctx, const Geom& g, const float4* cube,
                            int Kg, float2* h) {
  const int64_t count = int64_t(2 * Kg + 1) * (2 * Kg + 1) * (Kg + 1);
  TRVG_KBEGIN(ctx, "ff_cube_to_half_kernel");
  ff_cube_to_half_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, cube, Kg, h);
  TRVG_LAUNCHED(ctx);
}

void launch_ff_build_G(Context& ctx, const Geom& g, const int M[3],
                       const float4* cube, int Kg, const float2* const iw[3],
                       cd k0, float4* E, const double* k0_dev) {
  FFBuild bd{M[0], M[1], Kg, {iw[0], iw[1], iw[2]},
             FF{float(1. / g.vol), float(1. / g.vol - double(float(1. / g.vol)))}};
  const FFC k0f{FF{float(k0.re), float(k0.re - double(float(k0.re)))},
                FF{float(k0.im), float(k0.im - double(float(k0.im)))}};
  const int64_t count = int64_t(Kg + 1) * M[1] * M[0];
  TRVG_KBEGIN(ctx, "ff_build_kernel");
  ff_build_G_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(
      g, bd, cube, Kg, k0f, k0_dev, E);
  TRVG_LAUNCHED(ctx);
}

void launch_ff_build_F(Context& ctx, const Geom& g, const int M[3],
                       const float4* cube, int Kg, int K, const int16_t* tab,
                       int nq, int ell, const float2* const iw[3], cd k0,
                       float4* E, const double* k0_dev) {
  FFBuild bd{M[0], M[1], Kg, {iw[0], iw[1], iw[2]}, FF{0.f, 0.f}};
  const FFC k0f{FF{float(k0.re), float(k0.re - double(float(k0.re)))},
                FF{float(k0.im), float(k0.im - double(float(k0.im)))}};
  const int64_t plane = int64_t(K + 1) * M[1] * M[0];
  TRVG_CUDA(cudaMemsetAsync(E, 0, size_t(nq) * plane * sizeof(float4),
                            ctx.stream));
  TRVG_KBEGIN(ctx, "ff_build_kernel");
  ff_build_F_kernel<<<grid_for(plane, 256), 256, 0, ctx.stream>>>(
      g, bd, M[2], cube, K, tab, ell, k0f, k0_dev, E);
  TRVG_LAUNCHED(ctx);
}

void launch_ff_inverse(Context& ctx, const int M[3], int nf, int Kf, int Kcf,
                       const float4* E, float4* Y1, float4* Y2, float* out,
                       float* out_lo, int64_t ld, const FFBand& band) {
  const FFPlan Px = ff_plan(ctx, M[0]);
  const FFPlan Py = ff_plan(ctx, M[1]);
  const FFPlan Pz = ff_plan(ctx, M[2]);
  with_grid_radix_set(Px, [&](auto set) {
    constexpr int MASK = decltype(set)::value;
    const int lb = lines_per_block(Px);
    const int64_t nl = band.xl != nullptr
                           ? band.nxl
                           : int64_t(nf) * (Kcf + 1) * (2 * Kf + 1);
    if (nl == 0) return;
    allow_smem(ff_inv_x_kernel<MASK>);
    TRVG_KBEGIN(ctx, "ff_inv_x_kernel");
    ff_inv_x_kernel<MASK><<<int((nl + lb - 1) / lb), 256,
                            smem_bytes(M[0], lb), ctx.stream>>>(
        M[0], M[1], nf, Kf, Kcf, E, Px, lb, Y1, band);
    TRVG_LAUNCHED(ctx);
  });
  with_grid_radix_set(Py, [&](auto set) {
    constexpr int MASK = decltype(set)::value;
    const int lb = lines_per_block(Py);
    const int64_t nl = band.yoff != nullptr
                           ? band.nyl
                           : int64_t(nf) * (Kcf + 1) * M[0];
    if (nl == 0) return;
    allow_smem(ff_inv_y_kernel<MASK>);
    TRVG_KBEGIN(ctx, "ff_inv_y_kernel");
    ff_inv_y_kernel<MASK><<<int((nl + lb - 1) / lb), 256,
                            smem_bytes(M[1], lb), ctx.stream>>>(
        M[0], M[1], nf, Kf, Kcf, Y1, Py, lb, Y2, band);
    TRVG_LAUNCHED(ctx);
  });
  with_grid_radix_set(Pz, [&](auto set) {
    constexpr int MASK = decltype(set)::value;
    const int lb = lines_per_block(Pz);
    const int64_t np = (int64_t(nf) * M[0] * M[1] + 1) / 2;
    allow_smem(ff_inv_z_kernel<MASK>);
    TRVG_KBEGIN(ctx, "ff_inv_z_kernel");
    ff_inv_z_kernel<MASK><<<int((np + lb - 1) / lb), 256,
                            smem_bytes(M[2], lb), ctx.stream>>>(
        M[0], M[1], M[2], nf, Kcf, Y2, Pz, lb, out, out_lo, ld, band.kz);
    TRVG_LAUNCHED(ctx);
  });
}

}  // namespace trvg
