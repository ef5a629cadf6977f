// Configuration-space reductions.
//
//  * reduce_pairs: sum_x F_a(x) F_b(x) G(x) for many bin pairs in one launch
//    (the triple-product loops of threept.cpp:1703-1723 and its copies),
//    accumulated in FP64 for FP64 fields and as float-float pairs (FP32
//    operations only) for FP32 fields.
//  * radial_hist + pair_bessel_sums: the uncoupled shot noise of the
//    bispectrum, vol_cell sum_x j_la(k_a r) j_lb(k_b r) y_a(r) y_b(r) xi(x)
//    (field.cpp:3349-3396).  With cubic cells r depends on x only through
//    the integer key s_x^2 + s_y^2 + s_z^2, so xi * y_a * y_b is first
//    summed per key and the Bessel weights are applied per key and pair.
//  * octant_cell_hist: the same sums for cells of unequal sides, keyed by
//    (|s_x|, |s_y|, |s_z|), which fixes |r|; pair_bessel_sums then reads
//    each key's radius from a table.
//  * shotnoise_3pcf_bins: r-binned sums of the 3PCF shot noise
//    (field.cpp:3090-3196) with exact per-cell separations.
#include <algorithm>
#include <cmath>
#include <string>
#include <type_traits>
#include <vector>

#include "ff.cuh"
#include "kernels.h"

namespace trvg {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

int grid_for(int64_t work, int block, int64_t cap = 152 * 16) {
  int64_t g = (work + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return int(g);
}

// Block-wide sum of `n` per-thread values, atomically added to out[0..n).
// Only the first `limit` sums are written (the tail of the last chunk of
// pairs has no output slots).
template <int N>
__device__ __forceinline__ void block_add(double (&v)[N], double* out,
                                          double* red /* [N][32] */,
                                          int limit = N) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const double s = warp_sum(v[q]);
    if (lane == 0) red[q * 32 + wid] = s;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < N; q += blockDim.x) {
    double s = 0.;
    for (int w = 0; w < nw; ++w) s += red[q * 32 + w];
    if (out != nullptr && q < limit) atomicAdd(out + q, s);
  }
  __syncthreads();
}

template <class C>
__device__ __forceinline__ C cmulc(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

constexpr int kPairChunk = 8;

// Per-thread sum: float-float for FP32 fields, FP64 for FP64 fields.
template <class Real>
struct Acc;
template <>
struct Acc<float> {
  FF v = {0.f, 0.f};
  __device__ __forceinline__ void add(float x) { ff_add(v, x); }
  // The warp's total, valid in lane 0 (the only lane that converts).
  __device__ __forceinline__ double warp_total(int lane) {
    const FF t = ff_warp_sum(v);
    double r = 0.;
    if (lane == 0) r = ff_value(t);
    return r;
  }
};
template <>
struct Acc<double> {
  double v = 0.;
  __device__ __forceinline__ void add(double x) { v += x; }
  __device__ __forceinline__ double warp_total(int) { return warp_sum(v); }
};

// Block-wide sums of N accumulators, atomically added to out[q * stride]
// for q < limit.  Warps sum in the accumulators' own arithmetic; the
// (at most 32) warp totals are added in FP64.
template <int N, class Real>
__device__ __forceinline__ void block_add_acc(Acc<Real> (&a)[N], double* out,
                                              int stride, int limit,
                                              double* red /* [N][32] */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const double s = a[q].warp_total(lane);
    if (lane == 0) red[q * 32 + wid] = s;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < N && q < limit; q += blockDim.x) {
    double s = 0.;
    for (int w = 0; w < nw; ++w) s += red[q * 32 + w];
    atomicAdd(out + int64_t(q) * stride, s);
  }
}

template <class Real>
__global__ void __launch_bounds__(256)
reduce_pairs_kernel(int64_t ncell, const typename CplxOf<Real>::type* G,
                    const typename CplxOf<Real>::type* Fa,
                    const typename CplxOf<Real>::type* Fb, const int* pa,
                    const int* pb, int npairs, double* out, bool conj_b) {
  using C = typename CplxOf<Real>::type;
  __shared__ double red[2 * kPairChunk * 32];
  const int p0 = blockIdx.y * kPairChunk;
  int ia[kPairChunk], ib[kPairChunk];
  bool ok[kPairChunk];
#pragma unroll
  for (int q = 0; q < kPairChunk; ++q) {
    ok[q] = (p0 + q) < npairs;
    ia[q] = ok[q] ? pa[p0 + q] : 0;
    ib[q] = ok[q] ? pb[p0 + q] : 0;
  }
  Acc<Real> acc[2 * kPairChunk];
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < ncell;
       t += int64_t(gridDim.x) * blockDim.x) {
    const C g = G[t];
#pragma unroll
    for (int q = 0; q < kPairChunk; ++q) {
      if (!ok[q]) continue;
      const C a = Fa[int64_t(ia[q]) * ncell + t];
      C b = Fb[int64_t(ib[q]) * ncell + t];
      if (conj_b) b.y = -b.y;
      const C p = cmulc(cmulc(a, b), g);
      acc[2 * q].add(p.x);
      acc[2 * q + 1].add(p.y);
    }
  }
  block_add_acc<2 * kPairChunk, Real>(acc, out + 2 * p0, 1, 2 * (npairs - p0),
                                      red);
}

// FP32 complex fields as a Gram product: a block loads a tile of cells of
// every leg-a field and of every leg-b field times G into shared memory
// (each field is read once per launch instead of once per pair) and
// accumulates sum_x F_a (F_b G) for its pairs from there in float-float.
constexpr int kRedTile = 64;
constexpr int kRedRow = kRedTile + 1;  // padded: rows fall in other banks
constexpr int kRedPairsPerThread = 2;

__global__ void __launch_bounds__(256)
reduce_pairs_gram_kernel(int64_t ncell, const float2* G, const float2* Fa,
                         int na, const float2* Fb, int nb, const int* pa,
                         const int* pb, int npairs, double* out) {
  extern __shared__ float2 rsm[];
  float2* A = rsm;                  // [na][kRedRow]: F_a
  float2* B = rsm + na * kRedRow;   // [nb][kRedRow]: F_b G
  const int pbase = blockIdx.y * blockDim.x * kRedPairsPerThread;
  int ia[kRedPairsPerThread], ib[kRedPairsPerThread];
  bool on[kRedPairsPerThread];
  FF acc[2 * kRedPairsPerThread];
#pragma unroll
  for (int u = 0; u < kRedPairsPerThread; ++u) {
    const int pp = pbase + u * blockDim.x + threadIdx.x;
    on[u] = pp < npairs;
    ia[u] = on[u] ? pa[pp] : 0;
    ib[u] = on[u] ? pb[pp] : 0;
    acc[2 * u] = acc[2 * u + 1] = FF{0.f, 0.f};
  }
  const int nrows = na + nb;
  for (int64_t c0 = int64_t(blockIdx.x) * kRedTile; c0 < ncell;
       c0 += int64_t(gridDim.x) * kRedTile) {
    __syncthreads();  // the previous tile is consumed
    for (int w = threadIdx.x; w < nrows * kRedTile; w += blockDim.x) {
      const int row = w / kRedTile, c = w - row * kRedTile;
      const int64_t cell = c0 + c;
      float2 v = make_float2(0.f, 0.f);
      if (cell < ncell) {
        if (row < na) {
          v = Fa[int64_t(row) * ncell + cell];
        } else {
          v = cmulc(Fb[int64_t(row - na) * ncell + cell], G[cell]);
        }
      }
      if (row < na) A[row * kRedRow + c] = v;
      else B[(row - na) * kRedRow + c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kRedPairsPerThread; ++u) {
      if (!on[u]) continue;
      const float2* ra = A + ia[u] * kRedRow;
      const float2* rb = B + ib[u] * kRedRow;
      for (int c = 0; c < kRedTile; ++c) {
        const float2 q = cmulc(ra[c], rb[c]);
        ff_add(acc[2 * u], q.x);
        ff_add(acc[2 * u + 1], q.y);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < kRedPairsPerThread; ++u) {
    if (!on[u]) continue;
    const int pp = pbase + u * blockDim.x + threadIdx.x;
    atomicAdd(out + 2 * pp, ff_value(acc[2 * u]));
    atomicAdd(out + 2 * pp + 1, ff_value(acc[2 * u + 1]));
  }
}

// The same tiled Gram form for FP32 real fields (imaginary output zero).
__global__ void __launch_bounds__(256)
reduce_pairs_gram_real_kernel(int64_t ncell, const float* G, const float* Fa,
                              int na, const float* Fb, int nb, const int* pa,
                              const int* pb, int npairs, double* out) {
  extern __shared__ float rsr[];
  float* A = rsr;                  // [na][kRedRow]: F_a
  float* B = rsr + na * kRedRow;   // [nb][kRedRow]: F_b G
  const int pbase = blockIdx.y * blockDim.x * kRedPairsPerThread;
  int ia[kRedPairsPerThread], ib[kRedPairsPerThread];
  bool on[kRedPairsPerThread];
  FF acc[kRedPairsPerThread];
#pragma unroll
  for (int u = 0; u < kRedPairsPerThread; ++u) {
    const int pp = pbase + u * blockDim.x + threadIdx.x;
    on[u] = pp < npairs;
    ia[u] = on[u] ? pa[pp] : 0;
    ib[u] = on[u] ? pb[pp] : 0;
    acc[u] = FF{0.f, 0.f};
  }
  const int nrows = na + nb;
  for (int64_t c0 = int64_t(blockIdx.x) * kRedTile; c0 < ncell;
       c0 += int64_t(gridDim.x) * kRedTile) {
    __syncthreads();
    for (int w = threadIdx.x; w < nrows * kRedTile; w += blockDim.x) {
      const int row = w / kRedTile, c = w - row * kRedTile;
      const int64_t cell = c0 + c;
      float v = 0.f;
      if (cell < ncell)
        v = (row < na) ? Fa[int64_t(row) * ncell + cell]
                       : Fb[int64_t(row - na) * ncell + cell] * G[cell];
      if (row < na) A[row * kRedRow + c] = v;
      else B[(row - na) * kRedRow + c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kRedPairsPerThread; ++u) {
      if (!on[u]) continue;
      const float* ra = A + ia[u] * kRedRow;
      const float* rb = B + ib[u] * kRedRow;
      for (int c = 0; c < kRedTile; ++c) ff_add(acc[u], ra[c] * rb[c]);
    }
  }
#pragma unroll
  for (int u = 0; u < kRedPairsPerThread; ++u) {
    if (!on[u]) continue;
    const int pp = pbase + u * blockDim.x + threadIdx.x;
    atomicAdd(out + 2 * pp, ff_value(acc[u]));
  }
}

// Register-tiled Gram form of the pair sums for FP32 fields.  A block
// stages CELLS cells of every leg-a field (F_a), of every leg-b field (F_b)
// and of G in shared memory, cell-major, with asynchronous copies
// (cp.async) into one of two buffers while it reduces the other; F_b is
// then multiplied by G in shared memory (when both legs are one field set,
// F_b G is formed from the staged F_a and nothing more is read).  A thread
// reads the TI leg-a and TJ leg-b values of one cell as 16-byte vectors and
// updates a TI x TJ tile of field pairs from them (TI + TJ loads for TI TJ
// products).  Every field is read from HBM once per launch.  The products
// of kGramRun (16) cells are summed in FP32 and then added to float-float
// accumulators (TwoSum), so the accumulated sum keeps the error of an FP32
// sum of kGramRun terms per run rather than of the whole grid.  The
// threads of a tile split the chunk's cells into slices; the slices are
// summed in FP64 at the end and each data-vector entry gets one atomic add
// per block.
constexpr int kGramRun = 16;
constexpr int kGramThreads = 256;

__device__ __forceinline__ void cp_async_val(float* s, const float* g) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(s));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a),
               "l"(g)
               : "memory");
}
__device__ __forceinline__ void cp_async_val(float2* s, const float2* g) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(s));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(a),
               "l"(g)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ float gram_zero(float) { return 0.f; }
__device__ __forceinline__ float2 gram_zero(float2) {
  return make_float2(0.f, 0.f);
}
__device__ __forceinline__ float gram_mul(float a, float b) { return a * b; }
__device__ __forceinline__ float2 gram_mul(float2 a, float2 b) {
  return cmulc(a, b);
}

template <bool CPLX, int TI, int TJ, int CELLS>
__global__ void __launch_bounds__(kGramThreads, 2)
reduce_pairs_tiled_kernel(int64_t ncell, const float* __restrict__ G,
                          const float* __restrict__ Fa, int na, int rsa,
                          const float* __restrict__ Fb, int nb, int rsb,
                          unsigned mrsb, bool same,
                          const int2* __restrict__ tiles, int ntiles,
                          const int* __restrict__ slot, double* out,
                          int64_t ld) {
  using V = typename std::conditional<CPLX, float2, float>::type;
  constexpr int W = CPLX ? 2 : 1;  // floats per value
  constexpr int NP = TI * TJ * W;  // partial sums per thread
  extern __shared__ float4 gsm4[];
  V* const sbase = reinterpret_cast<V*>(gsm4);
  const int stage = CELLS * (rsa + rsb + 1);  // values per buffer
  const V* fa = reinterpret_cast<const V*>(Fa);
  const V* fb = reinterpret_cast<const V*>(Fb);
  const V* gv = reinterpret_cast<const V*>(G);
  const int g0 = blockIdx.y * kGramThreads;  // this block's tile group
  const int T = min(kGramThreads, ntiles - g0);
  const int S = kGramThreads / T;
  const int tid = threadIdx.x;
  const bool active = tid < S * T;
  const int tile = tid % T, slice = tid / T;
  int i0 = 0, j0 = 0;
  if (active) {
    const int2 tl = tiles[g0 + tile];
    i0 = tl.x * TI;
    j0 = tl.y * TJ;
  }
  float p[NP];
  FF acc[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    p[q] = 0.f;
    acc[q] = ff_zero();
  }
  int run = 0;
  // Rows fetched per chunk: leg a, leg b (unless one field set), G.
  const int nfetch = rsa + (same ? 0 : rsb) + 1;
  auto issue = [&](int64_t c0, int buf) {
    V* As = sbase + buf * stage;
    V* Bs = As + CELLS * rsa;
    V* Gs = Bs + CELLS * rsb;
    for (int w = tid; w < nfetch * CELLS; w += kGramThreads) {
      const int row = w / CELLS, c = w - row * CELLS;
      const int64_t cell = c0 + c;
      V* dst;
      const V* src = nullptr;
      if (row < rsa) {
        dst = As + c * rsa + row;
        if (row < na && cell < ncell) src = fa + int64_t(row) * ld + cell;
      } else if (row == nfetch - 1) {
        dst = Gs + c;
        if (cell < ncell) src = gv + cell;
      } else {
        const int r = row - rsa;
        dst = Bs + c * rsb + r;
        if (r < nb && cell < ncell) src = fb + int64_t(r) * ld + cell;
      }
      if (src != nullptr) cp_async_val(dst, src);
      else *dst = gram_zero(V());
    }
    cp_async_commit();
  };
  const int64_t step = int64_t(gridDim.x) * CELLS;
  int64_t c0 = int64_t(blockIdx.x) * CELLS;
  int buf = 0;
  if (c0 < ncell) issue(c0, 0);
  for (; c0 < ncell; c0 += step, buf ^= 1) {
    if (c0 + step < ncell) issue(c0 + step, buf ^ 1);
    else cp_async_commit();  // an empty group keeps the count uniform
    cp_async_wait<1>();      // this chunk's copies have landed
    __syncthreads();
    V* As = sbase + buf * stage;
    V* Bs = As + CELLS * rsa;
    const V* Gs = Bs + CELLS * rsb;
    for (int w = tid; w < rsb * CELLS; w += kGramThreads) {
      // w / rsb by the multiplier ceil(2^32 / rsb) (exact: w < 2^16).
      const int c = int(__umulhi(unsigned(w), mrsb)), r = w - c * rsb;
      V b;
      if (same) b = r < na ? As[c * rsa + r] : gram_zero(V());
      else b = Bs[c * rsb + r];
      Bs[c * rsb + r] = gram_mul(b, Gs[c]);
    }
    __syncthreads();
    if (active) {
      const int cend = ncell - c0 < CELLS ? int(ncell - c0) : CELLS;
      const float* af = reinterpret_cast<const float*>(As);
      const float* bf = reinterpret_cast<const float*>(Bs);
      for (int c = slice; c < cend; c += S) {
        float a[TI * W], b[TJ * W];
        const float4* va =
            reinterpret_cast<const float4*>(af + (c * rsa + i0) * W);
        const float4* vb =
            reinterpret_cast<const float4*>(bf + (c * rsb + j0) * W);
#pragma unroll
        for (int v = 0; v < TI * W / 4; ++v)
          reinterpret_cast<float4*>(a)[v] = va[v];
#pragma unroll
        for (int v = 0; v < TJ * W / 4; ++v)
          reinterpret_cast<float4*>(b)[v] = vb[v];
#pragma unroll
        for (int i = 0; i < TI; ++i)
#pragma unroll
          for (int j = 0; j < TJ; ++j) {
            if constexpr (CPLX) {
              float& re = p[2 * (i * TJ + j)];
              float& im = p[2 * (i * TJ + j) + 1];
              re = fmaf(a[2 * i], b[2 * j], re);
              re = fmaf(-a[2 * i + 1], b[2 * j + 1], re);
              im = fmaf(a[2 * i], b[2 * j + 1], im);
              im = fmaf(a[2 * i + 1], b[2 * j], im);
            } else {
              p[i * TJ + j] = fmaf(a[i], b[j], p[i * TJ + j]);
            }
          }
        if (++run == kGramRun) {
          run = 0;
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            ff_add(acc[q], p[q]);
            p[q] = 0.f;
          }
        }
      }
    }
    __syncthreads();  // the buffer is refilled two chunks on
  }
  cp_async_wait<0>();
#pragma unroll
  for (int q = 0; q < NP; ++q) ff_add(acc[q], p[q]);
  __syncthreads();  // the staging buffers become the slice table
  double* red = reinterpret_cast<double*>(gsm4);  // [S][T][NP]
  if (active) {
#pragma unroll
    for (int q = 0; q < NP; ++q)
      red[(slice * T + tile) * NP + q] = ff_value(acc[q]);
  }
  __syncthreads();
  for (int w = tid; w < T * NP; w += kGramThreads) {
    const int tl = w / NP, q = w - tl * NP;
    double s = 0.;
    for (int u = 0; u < S; ++u) s += red[(u * T + tl) * NP + q];
    const int2 tt = tiles[g0 + tl];
    const int pr = q / W, comp = q - pr * W;
    const int i = tt.x * TI + pr / TJ, j = tt.y * TJ + pr % TJ;
    if (i < na && j < nb) {
      const int sl = slot[int64_t(i) * nb + j];
      if (sl >= 0) atomicAdd(out + 2 * int64_t(sl) + comp, s);
    }
  }
}

// The same register-tiled Gram form with row-major staging, for fields
// whose rows start on 16-byte boundaries: a chunk of CELLS cells of every
// leg-a row, leg-b row and G is copied with 16-byte cp.async into rows of
// CELLS values (plus 16 bytes of padding), F_b G is formed with vector
// operations, and a thread updates its TI x TJ tile from two cells per
// step (one 8-byte load per real row, one 16-byte load per complex row).
// The copies and the F_b G pass cost a quarter of the per-element
// transposing form's instructions and write shared memory without bank
// conflicts.
template <bool CPLX, int TI, int TJ, int CELLS>
__global__ void __launch_bounds__(kGramThreads, 2)
reduce_pairs_rows_kernel(int64_t ncell, const float* __restrict__ G,
                         const float* __restrict__ Fa, int na, int rsa,
                         const float* __restrict__ Fb, int nb, int rsb,
                         bool same, const int2* __restrict__ tiles,
                         int ntiles, const int* __restrict__ slot,
                         double* out, int64_t ld) {
  constexpr int W = CPLX ? 2 : 1;          // floats per value
  constexpr int NP = TI * TJ * W;          // partial sums per thread
  constexpr int ROW = CELLS * W + 4;       // floats per staged row
  constexpr int VPR = CELLS * W / 4;       // 16-byte vectors per row
  constexpr int STEPS = CELLS / 2;         // two cells per step
  extern __shared__ float4 gsm4[];
  float* const sbase = reinterpret_cast<float*>(gsm4);
  // Staged row R (leg a, then leg b, then G) starts at off(R): every eighth
  // row is moved 16 bytes further, so that rows eight apart (the B rows of
  // neighbouring tiles) fall 16 bytes apart in the banks instead of on the
  // same bank.  The offsets only grow (rows never overlap).
  auto off = [](int R) { return R * ROW + 4 * (R >> 3); };
  const int nrow_all = rsa + rsb + 1;
  const int stage = nrow_all * ROW + 4 * (nrow_all >> 3) + 4;  // floats
  const int g0 = blockIdx.y * kGramThreads;
  const int T = min(kGramThreads, ntiles - g0);
  const int S = kGramThreads / T;
  const int tid = threadIdx.x;
  const bool active = tid < S * T;
  const int tile = tid % T, slice = tid / T;
  int i0 = 0, j0 = 0;
  if (active) {
    const int2 tl = tiles[g0 + tile];
    i0 = tl.x * TI;
    j0 = tl.y * TJ;
  }
  float p[NP];
  FF acc[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    p[q] = 0.f;
    acc[q] = ff_zero();
  }
  int run = 0;
  const int64_t nfl = ncell * W;  // floats per field
  const int64_t rfl = ld * W;     // floats between fields
  // Rows fetched per chunk: leg a, leg b (unless one field set), G.
  const int nfetch = rsa + (same ? 0 : rsb) + 1;
  auto issue = [&](int64_t c0, int buf) {
    float* base = sbase + buf * stage;
    const int64_t f0 = c0 * W;  // first float of the chunk in a row
    for (int w = tid; w < nfetch * VPR; w += kGramThreads) {
      const int row = w / VPR, v = w - row * VPR;
      const float* src;
      float* dst;
      bool valid;
      if (row < rsa) {
        dst = base + off(row);
        valid = row < na;
        src = Fa + int64_t(row) * rfl;
      } else if (row == nfetch - 1) {
        dst = base + off(rsa + rsb);
        valid = true;
        src = G;
      } else {
        const int r = row - rsa;
        dst = base + off(rsa + r);
        valid = r < nb;
        src = Fb + int64_t(r) * rfl;
      }
      dst += 4 * v;
      const int64_t e = f0 + 4 * v;  // first float of the vector
      if (valid && e + 4 <= nfl) {
        const unsigned a =
            static_cast<unsigned>(__cvta_generic_to_shared(dst));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a),
                     "l"(src + e)
                     : "memory");
      } else {
        float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid) {  // the tail of the last chunk
          float t[4] = {0.f, 0.f, 0.f, 0.f};
          for (int k = 0; k < 4; ++k)
            if (e + k < nfl) t[k] = src[e + k];
          z = make_float4(t[0], t[1], t[2], t[3]);
        }
        *reinterpret_cast<float4*>(dst) = z;
      }
    }
    cp_async_commit();
  };
  const int64_t step = int64_t(gridDim.x) * CELLS;
  int64_t c0 = int64_t(blockIdx.x) * CELLS;
  int buf = 0;
  if (c0 < ncell) issue(c0, 0);
  for (; c0 < ncell; c0 += step, buf ^= 1) {
    if (c0 + step < ncell) issue(c0 + step, buf ^ 1);
    else cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    float* const base = sbase + buf * stage;
    const float* Gs = base + off(rsa + rsb);
    // F_b G in place (from the staged F_a when both legs are one set).
    for (int w = tid; w < rsb * VPR; w += kGramThreads) {
      const int r = w / VPR, v = w - r * VPR;
      float* brow = base + off(rsa + r);
      float4 b;
      if (same)
        b = r < na ? reinterpret_cast<const float4*>(base + off(r))[v]
                   : make_float4(0.f, 0.f, 0.f, 0.f);
      else
        b = reinterpret_cast<const float4*>(brow)[v];
      const float4 gg = reinterpret_cast<const float4*>(Gs)[v];
      float4 o;
      if constexpr (CPLX) {
        o = make_float4(b.x * gg.x - b.y * gg.y, b.x * gg.y + b.y * gg.x,
                        b.z * gg.z - b.w * gg.w, b.z * gg.w + b.w * gg.z);
      } else {
        o = make_float4(b.x * gg.x, b.y * gg.y, b.z * gg.z, b.w * gg.w);
      }
      reinterpret_cast<float4*>(brow)[v] = o;
    }
    __syncthreads();
    if (active) {
      const int cend = ncell - c0 < CELLS ? int(ncell - c0) : CELLS;
      const int send = (cend + 1) / 2;  // the padding cell of an odd tail is 0
      for (int st = slice; st < send; st += S) {
        // Two cells: a[i] (and b[j]) hold cell 2 st then cell 2 st + 1.
        float a[TI][2 * W], b[TJ][2 * W];
#pragma unroll
        for (int i = 0; i < TI; ++i) {
          const float* r = base + off(i0 + i) + 2 * W * st;
          if constexpr (CPLX) {
            const float4 v = *reinterpret_cast<const float4*>(r);
            a[i][0] = v.x; a[i][1] = v.y; a[i][2] = v.z; a[i][3] = v.w;
          } else {
            const float2 v = *reinterpret_cast<const float2*>(r);
            a[i][0] = v.x; a[i][1] = v.y;
          }
        }
#pragma unroll
        for (int j = 0; j < TJ; ++j) {
          const float* r = base + off(rsa + j0 + j) + 2 * W * st;
          if constexpr (CPLX) {
            const float4 v = *reinterpret_cast<const float4*>(r);
            b[j][0] = v.x; b[j][1] = v.y; b[j][2] = v.z; b[j][3] = v.w;
          } else {
            const float2 v = *reinterpret_cast<const float2*>(r);
            b[j][0] = v.x; b[j][1] = v.y;
          }
        }
#pragma unroll
        for (int i = 0; i < TI; ++i)
#pragma unroll
          for (int j = 0; j < TJ; ++j) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              if constexpr (CPLX) {
                float& re = p[2 * (i * TJ + j)];
                float& im = p[2 * (i * TJ + j) + 1];
                re = fmaf(a[i][2 * k], b[j][2 * k], re);
                re = fmaf(-a[i][2 * k + 1], b[j][2 * k + 1], re);
                im = fmaf(a[i][2 * k], b[j][2 * k + 1], im);
                im = fmaf(a[i][2 * k + 1], b[j][2 * k], im);
              } else {
                p[i * TJ + j] = fmaf(a[i][k], b[j][k], p[i * TJ + j]);
              }
            }
          }
        run += 2;
        if (run >= kGramRun) {
          run = 0;
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            ff_add(acc[q], p[q]);
            p[q] = 0.f;
          }
        }
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();
#pragma unroll
  for (int q = 0; q < NP; ++q) ff_add(acc[q], p[q]);
  __syncthreads();
  double* red = reinterpret_cast<double*>(gsm4);  // [S][T][NP]
  if (active) {
#pragma unroll
    for (int q = 0; q < NP; ++q)
      red[(slice * T + tile) * NP + q] = ff_value(acc[q]);
  }
  __syncthreads();
  for (int w = tid; w < T * NP; w += kGramThreads) {
    const int tl = w / NP, q = w - tl * NP;
    double sum = 0.;
    for (int u = 0; u < S; ++u) sum += red[(u * T + tl) * NP + q];
    const int2 tt = tiles[g0 + tl];
    const int pr = q / W, comp = q - pr * W;
    const int i = tt.x * TI + pr / TJ, j = tt.y * TJ + pr % TJ;
    if (i < na && j < nb) {
      const int sl = slot[int64_t(i) * nb + j];
      if (sl >= 0) atomicAdd(out + 2 * int64_t(sl) + comp, sum);
    }
  }
}

// Real fields: sum_x F_a F_b G; the imaginary part of the output is left
// at zero.
template <class Real>
__global__ void __launch_bounds__(256)
reduce_pairs_real_kernel(int64_t ncell, const Real* G, const Real* Fa,
                         const Real* Fb, const int* pa, const int* pb,
                         int npairs, double* out) {
  __shared__ double red[kPairChunk * 32];
  const int p0 = blockIdx.y * kPairChunk;
  int ia[kPairChunk], ib[kPairChunk];
  bool ok[kPairChunk];
#pragma unroll
  for (int q = 0; q < kPairChunk; ++q) {
    ok[q] = (p0 + q) < npairs;
    ia[q] = ok[q] ? pa[p0 + q] : 0;
    ib[q] = ok[q] ? pb[p0 + q] : 0;
  }
  Acc<Real> acc[kPairChunk];
  int64_t t0 = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if constexpr (sizeof(Real) == 4) {
    // Four cells per load: more bytes in flight per thread (the scalar loop
    // is bound by load latency); the four products are summed in FP32
    // before the float-float add.
    if (ncell % 4 == 0) {
      const int64_t n4 = ncell / 4;
      for (int64_t t = t0; t < n4; t += int64_t(gridDim.x) * blockDim.x) {
        const float4 g = reinterpret_cast<const float4*>(G)[t];
#pragma unroll
        for (int q = 0; q < kPairChunk; ++q) {
          if (!ok[q]) continue;
          const float4 a =
              reinterpret_cast<const float4*>(Fa + int64_t(ia[q]) * ncell)[t];
          const float4 b =
              (ia[q] == ib[q] && Fa == Fb)
                  ? a
                  : reinterpret_cast<const float4*>(
                        Fb + int64_t(ib[q]) * ncell)[t];
          acc[q].add((a.x * b.x * g.x + a.y * b.y * g.y) +
                     (a.z * b.z * g.z + a.w * b.w * g.w));
        }
      }
      t0 = ncell;  // nothing left for the scalar loop
    }
  }
  for (int64_t t = t0; t < ncell; t += int64_t(gridDim.x) * blockDim.x) {
    const Real g = G[t];
#pragma unroll
    for (int q = 0; q < kPairChunk; ++q) {
      if (!ok[q]) continue;
      const Real a = Fa[int64_t(ia[q]) * ncell + t];
      const Real b = (ia[q] == ib[q] && Fa == Fb)
                         ? a : Fb[int64_t(ib[q]) * ncell + t];
      acc[q].add(a * b * g);
    }
  }
  block_add_acc<kPairChunk, Real>(acc, out + 2 * p0, 2, npairs - p0, red);
}

// (ah + al)(bh + bl)(gh + gl) as an unnormalised float-float pair: the
// leading products by TwoProduct, the cross terms to first order (their
// neglected products are below 2^-46 of the result).
__device__ __forceinline__ FF ff_prod3(float ah, float al, float bh, float bl,
                                       float gh, float gl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const float q = __fmul_rn(p, gh);
  float f = __fmaf_rn(p, gh, -q);
  f = __fmaf_rn(p, gl, f);
  f = __fmaf_rn(e, gh, f);
  return FF{q, f};
}

// sum_x F_a F_b G of float-float fields (hi and lo word arrays, field q at
// q ld): four cells per float4 load, the cells past the last whole quad by
// the first block; a pair whose legs are the same field loads it once.
__device__ __forceinline__ void ff_quad(FF& acc, float4 ah, float4 al,
                                        float4 bh, float4 bl, float4 gh,
                                        float4 gl) {
  ff_merge(acc, ff_prod3(ah.x, al.x, bh.x, bl.x, gh.x, gl.x));
  ff_merge(acc, ff_prod3(ah.y, al.y, bh.y, bl.y, gh.y, gl.y));
  ff_merge(acc, ff_prod3(ah.z, al.z, bh.z, bl.z, gh.z, gl.z));
  ff_merge(acc, ff_prod3(ah.w, al.w, bh.w, bl.w, gh.w, gl.w));
}

template <int CHUNK>
__global__ void __launch_bounds__(256)
reduce_pairs_ff_kernel(int64_t ncell, int64_t ld,
                       const float* __restrict__ Gh,
                       const float* __restrict__ Gl,
                       const float* __restrict__ Fah,
                       const float* __restrict__ Fal,
                       const float* __restrict__ Fbh,
                       const float* __restrict__ Fbl, const int* pa,
                       const int* pb, int npairs, double* out) {
  __shared__ double red[CHUNK * 32];
  const int p0 = blockIdx.y * CHUNK;
  int64_t oa[CHUNK], ob[CHUNK];
  bool ok[CHUNK], same[CHUNK];
#pragma unroll
  for (int q = 0; q < CHUNK; ++q) {
    ok[q] = (p0 + q) < npairs;
    oa[q] = ok[q] ? int64_t(pa[p0 + q]) * ld : 0;
    ob[q] = ok[q] ? int64_t(pb[p0 + q]) * ld : 0;
    same[q] = Fah == Fbh && oa[q] == ob[q];
  }
  Acc<float> acc[CHUNK];
  const int64_t nquad = ncell / 4;
  auto q4 = [](const float* p, int64_t off, int64_t t) {
    return reinterpret_cast<const float4*>(p + off)[t];
  };
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < nquad;
       t += int64_t(gridDim.x) * blockDim.x) {
    const float4 gh = q4(Gh, 0, t), gl = q4(Gl, 0, t);
#pragma unroll
    for (int q = 0; q < CHUNK; ++q) {
      if (!ok[q]) continue;
      const float4 ah = q4(Fah, oa[q], t), al = q4(Fal, oa[q], t);
      if (same[q]) {
        ff_quad(acc[q].v, ah, al, ah, al, gh, gl);
      } else {
        const float4 bh = q4(Fbh, ob[q], t), bl = q4(Fbl, ob[q], t);
        ff_quad(acc[q].v, ah, al, bh, bl, gh, gl);
      }
    }
  }
  if (blockIdx.x == 0) {
    for (int64_t c = nquad * 4 + threadIdx.x; c < ncell; c += blockDim.x) {
#pragma unroll
      for (int q = 0; q < CHUNK; ++q) {
        if (!ok[q]) continue;
        ff_merge(acc[q].v, ff_prod3(Fah[oa[q] + c], Fal[oa[q] + c],
                                    Fbh[ob[q] + c], Fbl[ob[q] + c], Gh[c],
                                    Gl[c]));
      }
    }
  }
  block_add_acc<CHUNK, float>(acc, out + 2 * p0, 2, npairs - p0, red);
}

// Sum of xi * y_a * y_b per integer key s_x^2 + s_y^2 + s_z^2 (cubic cells).
template <class Real>
__global__ void __launch_bounds__(256)
radial_hist_kernel(Geom g, const Real* xi_re, const Real* xi_im, int ell_a,
                   int m_a, int ell_b, int m_b, double* hist) {
  const bool trivial = (ell_a == 0 && m_a == 0 && ell_b == 0 && m_b == 0);
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       t < g.nmesh; t += int64_t(gridDim.x) * blockDim.x) {
    const int k = int(t % g.n[2]);
    const int j = int((t / g.n[2]) % g.n[1]);
    const int i = int(t / (int64_t(g.n[2]) * g.n[1]));
    const int sx = shift_index(i, g.n[0]), sy = shift_index(j, g.n[1]),
              sz = shift_index(k, g.n[2]);
    const int64_t key = int64_t(sx) * sx + int64_t(sy) * sy + int64_t(sz) * sz;
    cd v = {double(xi_re[t]), xi_im != nullptr ? double(xi_im[t]) : 0.};
    if (!trivial) {
      const double rx = dmul(double(sx), g.dr[0]);
      const double ry = dmul(double(sy), g.dr[1]);
      const double rz = dmul(double(sz), g.dr[2]);
      const cd ya = reduced_ylm(ell_a, m_a, rx, ry, rz);
      const cd yb = reduced_ylm(ell_b, m_b, rx, ry, rz);
      v = v * (ya * yb);
    }
    atomicAdd(hist + 2 * key, v.re);
    if (v.im != 0.) atomicAdd(hist + 2 * key + 1, v.im);
  }
}

// The same sums from the flip-averaged xi on the octant (even mesh numbers,
// cubic cells): cell (a, b, c) stands for its 1, 2, 4 or 8 mirror cells
// (one per coordinate not 0 or n/2), xo[(c (hy + 1) + b) (hx + 1) + a].x.
// KIND as for orbit_rows_kernel (0 or 1).
// f * 2^e2 as a double, formed from the bits of f with integer operations
// (exact; GB300 runs float-to-double conversions on its FP64 pipe).  Zero,
// subnormal and non-finite f take the conversion.
__device__ __noinline__ double f2d_pow2_slow(float f, int e2) {
  return double(f) * double(1 << e2);
}

__device__ __forceinline__ double f2d_pow2(float f, int e2) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  if (ex == 0u || ex == 0xffu) return f2d_pow2_slow(f, e2);
  const unsigned long long bits =
      (static_cast<unsigned long long>(u >> 31) << 63) |
      (static_cast<unsigned long long>(ex + 896u + unsigned(e2)) << 52) |
      (static_cast<unsigned long long>(u & 0x7fffffu) << 29);
  return __longlong_as_double(static_cast<long long>(bits));
}

// Legendre polynomial P_l(mu) by the three-term recurrence, in FP32:
// y_l0 of a unit vector with z component mu (reduced_ylm).
__device__ __forceinline__ float legendre_f(int ell, float mu) {
  if (ell == 0) return 1.f;
  float pm = 1.f, p = mu;
  for (int n = 1; n < ell; ++n) {
    const float pn = (float(2 * n + 1) * mu * p - float(n) * pm) / float(n + 1);
    pm = p;
    p = pn;
  }
  return p;
}

template <int KIND>
__global__ void __launch_bounds__(256)
octant_hist_kernel(Geom g, const float2* xo, int ell_a, int ell_b,
                   double* hist) {
  const int hx = g.n[0] / 2, hy = g.n[1] / 2;
  const int c = blockIdx.y, b = blockIdx.x;
  const int64_t row = (int64_t(c) * (hy + 1) + b) * (hx + 1);
  // Mirror cells per coordinate: 1 at 0 and n/2, else 2 (as a power of 2).
  const int ebc = ((b == 0 || b == hy) ? 0 : 1) +
                  ((c == 0 || c == g.n[2] / 2) ? 0 : 1);
  const int64_t key_bc = int64_t(b) * b + int64_t(c) * c;
  for (int a = threadIdx.x; a <= hx; a += blockDim.x) {
    const int e = ebc + ((a == 0 || a == hx) ? 0 : 1);
    const int64_t key = key_bc + int64_t(a) * a;
    float x = xo[row + a].x;
    if constexpr (KIND == 1) {
      // y_la0 y_lb0 at mu = c / |(a, b, c)| (cubic cells; 0 at r = 0);
      // a^2 + b^2 + c^2 < 2^24 is exact in FP32.
      float f = 0.f;
      if (key != 0) {
        const float mu = sqrtf(float(int64_t(c) * c) / float(key));
        f = legendre_f(ell_a, mu) * legendre_f(ell_b, mu);
      }
      x *= f;
    }
    atomicAdd(hist + 2 * key, f2d_pow2(x, e));
  }
}

// The same sums for even mesh numbers, with one atomic per orbit row
// instead of one per cell.  The cells (+-s_x, +-s_y, +-s_z) -- and, when
// n_x = n_y, their x <-> y swaps -- share the key a^2 + b^2 + c^2 with
// (a, b, c) = (|s_x|, |s_y|, |s_z|).  One block per (a, b) (b <= a with the
// swap), threads along c: each thread sums its <= 16 mirror cells and adds
// the sum to the key's FP64 bin.
__device__ __forceinline__ void orbit_ab(int q, bool swap, int hy, int& a,
                                         int& b) {
  if (swap) {
    a = int((sqrtf(8.f * float(q) + 1.f) - 1.f) * 0.5f);
    while ((a + 1) * (a + 2) / 2 <= q) ++a;
    while (a * (a + 1) / 2 > q) --a;
    b = q - a * (a + 1) / 2;
  } else {
    a = q / (hy + 1);
    b = q - a * (hy + 1);
  }
}

// KIND 0: both degrees are (0, 0), so y_a y_b = 1.
// KIND 1: m_a = m_b = 0 and ell_a + ell_b even: y_a y_b is a function of
//   mu^2 = s_z^2 / s^2 alone (y_l0 is a Legendre polynomial in mu of the
//   parity of l), the same on the 16 mirror cells of an orbit row, so it
//   multiplies their sum once.
// KIND 2: any degrees, y_a y_b per cell.
template <class Real, int KIND>
__global__ void __launch_bounds__(256)
orbit_rows_kernel(Geom g, const Real* xi_re, const Real* xi_im, int ell_a,
                  int m_a, int ell_b, int m_b, bool swap, double* hist) {
  const int hy = g.n[1] / 2, hz = g.n[2] / 2;
  int a, b;
  orbit_ab(blockIdx.x, swap, hy, a, b);
  const int xs[2] = {a, (a == 0) ? 0 : g.n[0] - a};
  const int ys[2] = {b, (b == 0) ? 0 : g.n[1] - b};
  const bool x2 = xs[1] != xs[0], y2 = ys[1] != ys[0];
  const bool sw = swap && a != b;
  // Row i * n_y + j of each of the up-to-8 rows of the orbit (-1: absent),
  // held in registers so that every load of a thread is issued at once.
  int rowi[8];
#pragma unroll
  for (int w = 0; w < 2; ++w)
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const bool use = (w == 0 || sw) && (p == 0 || x2) && (q == 0 || y2);
        const int i = (w == 0) ? xs[p] : ys[q];
        const int j = (w == 0) ? ys[q] : xs[p];
        rowi[w * 4 + p * 2 + q] = use ? i * g.n[1] + j : -1;
      }
  const int64_t key_ab = int64_t(a) * a + int64_t(b) * b;
  for (int c = threadIdx.x; c <= hz; c += blockDim.x) {
    const int c2 = (c == 0) ? 0 : g.n[2] - c;
    const bool two = (c2 != c);
    cd acc = {0., 0.};
    if constexpr (KIND != 2) {
      Real sr = Real(0), si = Real(0);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        if (rowi[r] < 0) continue;
        const int64_t base = int64_t(rowi[r]) * g.n[2];
        sr += xi_re[base + c];
        if (two) sr += xi_re[base + c2];
        if (xi_im != nullptr) {
          si += xi_im[base + c];
          if (two) si += xi_im[base + c2];
        }
      }
      acc = cd{double(sr), double(si)};
      if constexpr (KIND == 1) {
        const double rx = dmul(double(a), g.dr[0]);
        const double ry = dmul(double(b), g.dr[1]);
        const double rz = dmul(double(c), g.dr[2]);
        const double f = (reduced_ylm(ell_a, 0, rx, ry, rz) *
                          reduced_ylm(ell_b, 0, rx, ry, rz)).re;
        acc = cd{acc.re * f, acc.im * f};
      }
    } else {
#pragma unroll 1
      for (int r = 0; r < 8; ++r) {
        if (rowi[r] < 0) continue;
        const int i = rowi[r] / g.n[1], j = rowi[r] - i * g.n[1];
        const int64_t base = int64_t(rowi[r]) * g.n[2];
        for (int z = 0; z < (two ? 2 : 1); ++z) {
          const int k = (z == 0) ? c : c2;
          cd v = {double(xi_re[base + k]),
                  xi_im != nullptr ? double(xi_im[base + k]) : 0.};
          const double rx = dmul(double(shift_index(i, g.n[0])), g.dr[0]);
          const double ry = dmul(double(shift_index(j, g.n[1])), g.dr[1]);
          const double rz = dmul(double(shift_index(k, g.n[2])), g.dr[2]);
          v = v * (reduced_ylm(ell_a, m_a, rx, ry, rz) *
                   reduced_ylm(ell_b, m_b, rx, ry, rz));
          acc = acc + v;
        }
      }
    }
    const int64_t key = key_ab + int64_t(c) * c;
    atomicAdd(hist + 2 * key, acc.re);
    if (xi_im != nullptr || KIND == 2) atomicAdd(hist + 2 * key + 1, acc.im);
  }
}

struct PairBesselArgs {
  SplineTable ja, jb;
  const double* ka;
  const double* kb;
};

constexpr int kKeyPairChunk = 8;

// One thread per key: r = dr sqrt(key) once, then the Bessel weights of a
// chunk of pairs (one spline evaluation when both legs coincide).
__global__ void __launch_bounds__(256)
pair_bessel_sums_kernel(int64_t nkeys, double dr, const double* rkey,
                        const double* hist, PairBesselArgs a, int npairs,
                        bool same_leg, double* out) {
  __shared__ double red[2 * kKeyPairChunk * 32];
  const int p0 = blockIdx.y * kKeyPairChunk;
  double ka[kKeyPairChunk], kb[kKeyPairChunk];
#pragma unroll
  for (int q = 0; q < kKeyPairChunk; ++q) {
    const int pi = min(p0 + q, npairs - 1);
    ka[q] = a.ka[pi];
    kb[q] = a.kb[pi];
  }
  double acc[2 * kKeyPairChunk];
#pragma unroll
  for (int q = 0; q < 2 * kKeyPairChunk; ++q) acc[q] = 0.;
  for (int64_t key = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       key < nkeys; key += int64_t(gridDim.x) * blockDim.x) {
    const double hr = hist[2 * key], hi = hist[2 * key + 1];
    if (hr == 0. && hi == 0.) continue;
    const double r = rkey != nullptr ? rkey[key] : dr * sqrt(double(key));
#pragma unroll
    for (int q = 0; q < kKeyPairChunk; ++q) {
      const double ja = spline_eval(a.ja, ka[q] * r);
      const double jb = (same_leg && ka[q] == kb[q])
                            ? ja : spline_eval(a.jb, kb[q] * r);
      const double w = ja * jb;
      acc[2 * q] += w * hr;
      acc[2 * q + 1] += w * hi;
    }
  }
  block_add<2 * kKeyPairChunk>(acc, out + 2 * p0, red, 2 * (npairs - p0));
}

// j_ell(x) at x = x.hi + x.lo >= 0 from the FP32 copy of the spline: the
// knot value in float-float, the cubic terms (dx < 0.05) in FP32, which
// keeps about 1e-8 absolute error; the same interval rule as spline_eval.
__device__ __forceinline__ FF spline_eval_ff(const SplineTable& t, FF x) {
  if (x.hi >= float(t.split)) {
    const double v = sph_bessel_upward(t.ell, double(x.hi) + double(x.lo));
    return FF{float(v), float(v - double(float(v)))};
  }
  const float hh = 0x1.99999ap-5f, hl = -0x1.99999ap-31f;  // 0.05
  auto offset = [&](int i) {  // x - 0.05 i in FP32 (float-float knot)
    const float fi = float(i);
    const float p = __fmul_rn(hh, fi);
    const float e = __fmaf_rn(hl, fi, __fmaf_rn(hh, fi, -p));
    return __fadd_rn(__fsub_rn(x.hi, p), __fsub_rn(x.lo, e));
  };
  int i = int(__fmul_rn(x.hi, 20.f));
  i = max(0, min(i, t.n - 2));
  float dx = offset(i);
  if (dx < 0.f && i > 0) {
    --i;
    dx = offset(i);
  } else if (dx >= hh && i < t.n - 2) {
    ++i;
    dx = offset(i);
  }
  const float4 q = t.q[i];
  const float poly =
      __fmul_rn(dx, __fmaf_rn(dx, __fmaf_rn(dx, t.dq[i], q.w), q.z));
  return ffadd(FF{q.x, q.y}, FF{poly, 0.f});
}

// pair_bessel_sums_kernel on the FP32 pipe: r = dr sqrt(key) and k r in
// float-float, Bessel weights from spline_eval_ff, products and sums in
// float-float; FP64 only per key (the histogram words) and at the end.
__global__ void __launch_bounds__(256)
pair_bessel_sums_ff_kernel(int64_t nkeys, double dr, const double* rkey,
                           const double* hist, PairBesselArgs a, int npairs,
                           bool same_leg, double* out) {
  __shared__ double red[2 * kKeyPairChunk * 32];
  const int p0 = blockIdx.y * kKeyPairChunk;
  FF ka[kKeyPairChunk], kb[kKeyPairChunk];
  bool same[kKeyPairChunk];
#pragma unroll
  for (int q = 0; q < kKeyPairChunk; ++q) {
    const int pi = min(p0 + q, npairs - 1);
    ka[q] = ff_from_double(a.ka[pi]);
    kb[q] = ff_from_double(a.kb[pi]);
    same[q] = same_leg && a.ka[pi] == a.kb[pi];
  }
  const FF drf = ff_from_double(dr);
  FF acc[2 * kKeyPairChunk];
#pragma unroll
  for (int q = 0; q < 2 * kKeyPairChunk; ++q) acc[q] = FF{0.f, 0.f};
  for (int64_t key = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       key < nkeys; key += int64_t(gridDim.x) * blockDim.x) {
    const double2 h = reinterpret_cast<const double2*>(hist)[key];
    if (h.x == 0. && h.y == 0.) continue;
    const FF hr = ff_from_double(h.x), hi = ff_from_double(h.y);
    FF r;
    if (rkey != nullptr) {
      r = ff_from_double(rkey[key]);
    } else {
      // sqrt(key) in float-float (key < 2^24 is exact in FP32).
      const float kf = float(key);
      const float sh = __fsqrt_rn(kf);
      const float sl =
          sh > 0.f ? __fdiv_rn(__fmaf_rn(-sh, sh, kf), __fmul_rn(2.f, sh))
                   : 0.f;
      r = ffmul(drf, FF{sh, sl});
    }
#pragma unroll
    for (int q = 0; q < kKeyPairChunk; ++q) {
      const FF ja = spline_eval_ff(a.ja, ffmul(ka[q], r));
      const FF jb = same[q] ? ja : spline_eval_ff(a.jb, ffmul(kb[q], r));
      const FF w = ffmul(ja, jb);
      ff_merge(acc[2 * q], ffnorm(ffmul(w, hr)));
      ff_merge(acc[2 * q + 1], ffnorm(ffmul(w, hi)));
    }
  }
  double v[2 * kKeyPairChunk];
#pragma unroll
  for (int q = 0; q < 2 * kKeyPairChunk; ++q) v[q] = ff_value(acc[q]);
  block_add<2 * kKeyPairChunk>(v, out + 2 * p0, red, 2 * (npairs - p0));
}

// pair_bessel_sums_ff_kernel as a Gram product: the weight of pair p at a
// key is J_a(key) J_b(key) with J_a = j_la(k_a r) of bin a, so a block
// evaluates J for every distinct bin over a chunk of keys into shared
// memory (per key 2 x bins spline evaluations instead of 2 x pairs) and
// accumulates sum_key H J_a J_b for its pairs from there, in float-float.
// ka_d[nka], kb_d[nkb]: the distinct k of the two legs; pa, pb: each pair's
// indices into them.
constexpr int kGramKeys = 128;
// J rows one element longer than a chunk: lanes reading different rows at
// one key fall in different banks.
constexpr int kGramRow = kGramKeys + 1;
constexpr int kGramPairsPerThread = 2;

struct GramArgs {
  SplineTable ja, jb;
  const double* ka_d;
  const double* kb_d;
  int nka, nkb;
  bool same;  // one leg: J_b = J_a
  const int* pa;
  const int* pb;
};

__global__ void __launch_bounds__(256)
pair_bessel_gram_ff_kernel(int64_t nkeys, double dr, const double* rkey,
                           const double* hist, GramArgs g, int npairs,
                           double* out) {
  // Shared memory: the histogram words of the chunk, then the J rows of
  // leg a and of leg b (absent when one leg), kGramRow apart.
  extern __shared__ float4 gsm[];
  const int nrows = g.nka + (g.same ? 0 : g.nkb);
  float4* H = gsm;
  float2* J = reinterpret_cast<float2*>(gsm + kGramKeys);
  const int boff = g.same ? 0 : g.nka;
  const int pbase = blockIdx.y * blockDim.x * kGramPairsPerThread;
  int ia[kGramPairsPerThread], ib[kGramPairsPerThread];
  bool on[kGramPairsPerThread];
  FF acc[2 * kGramPairsPerThread];
#pragma unroll
  for (int u = 0; u < kGramPairsPerThread; ++u) {
    const int pp = pbase + u * blockDim.x + threadIdx.x;
    on[u] = pp < npairs;
    ia[u] = on[u] ? g.pa[pp] : 0;
    ib[u] = on[u] ? boff + g.pb[pp] : 0;
    acc[2 * u] = acc[2 * u + 1] = FF{0.f, 0.f};
  }
  const FF drf = ff_from_double(dr);
  for (int64_t k0 = int64_t(blockIdx.x) * kGramKeys; k0 < nkeys;
       k0 += int64_t(gridDim.x) * kGramKeys) {
    __syncthreads();  // the previous chunk is consumed
    for (int k = threadIdx.x; k < kGramKeys; k += blockDim.x) {
      const int64_t key = k0 + k;
      double2 h = make_double2(0., 0.);
      if (key < nkeys) h = reinterpret_cast<const double2*>(hist)[key];
      const FF hr = ff_from_double(h.x), hi = ff_from_double(h.y);
      H[k] = make_float4(hr.hi, hr.lo, hi.hi, hi.lo);
    }
    __syncthreads();
    for (int w = threadIdx.x; w < nrows * kGramKeys; w += blockDim.x) {
      const int row = w / kGramKeys, k = w - row * kGramKeys;
      const float4 h = H[k];
      FF v{0.f, 0.f};
      if (h.x != 0.f || h.z != 0.f) {
        const int64_t key = k0 + k;
        FF r;
        if (rkey != nullptr) {
          r = ff_from_double(rkey[key]);
        } else {
          // sqrt(key) in float-float (key < 2^24 is exact in FP32).
          const float kf = float(key);
          const float sh = __fsqrt_rn(kf);
          const float sl =
              sh > 0.f ? __fdiv_rn(__fmaf_rn(-sh, sh, kf), __fmul_rn(2.f, sh))
                       : 0.f;
          r = ffmul(drf, FF{sh, sl});
        }
        const bool leg_a = row < g.nka;
        const FF kk =
            ff_from_double(leg_a ? g.ka_d[row] : g.kb_d[row - g.nka]);
        v = spline_eval_ff(leg_a ? g.ja : g.jb, ffmul(kk, r));
      }
      J[row * kGramRow + k] = make_float2(v.hi, v.lo);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kGramPairsPerThread; ++u) {
      if (!on[u]) continue;
      const float2* ja = J + ia[u] * kGramRow;
      const float2* jb = J + ib[u] * kGramRow;
      // Unnormalised float-float sums over the chunk (the next operation
      // splits the leading words again), normalised once per chunk.
      FF sr = acc[2 * u], si = acc[2 * u + 1];
      for (int k = 0; k < kGramKeys; ++k) {
        const float4 h = H[k];
        if (h.x == 0.f && h.z == 0.f) continue;
        const float2 a = ja[k], b = jb[k];
        const FF w = ffmul(FF{a.x, a.y}, FF{b.x, b.y});
        sr = ffadd(sr, ffmul(w, FF{h.x, h.y}));
        si = ffadd(si, ffmul(w, FF{h.z, h.w}));
      }
      acc[2 * u] = ffnorm(sr);
      acc[2 * u + 1] = ffnorm(si);
    }
  }
#pragma unroll
  for (int u = 0; u < kGramPairsPerThread; ++u) {
    if (!on[u]) continue;
    const int pp = pbase + u * blockDim.x + threadIdx.x;
    atomicAdd(out + 2 * pp, ff_value(acc[2 * u]));
    atomicAdd(out + 2 * pp + 1, ff_value(acc[2 * u + 1]));
  }
}


// Cells of any shape grouped by (|s_x|, |s_y|, |s_z|), which fixes |r|:
// hist[key] = sum of xi y_a y_b over the key's cells, key = (|s_x| D_y +
// |s_y|) D_z + |s_z| with D = n - n/2 + 1 per axis (|s| reaches n/2 + 1 on
// an odd axis, where index n/2 has frequency -(n/2 + 1)), and rkey[key] =
// |r| (the sign of s does not change a product s dr).  One thread per key:
// its (up to eight) cells are summed in the thread and the bin is written
// once, without atomics.  Along an axis, key a holds cell a when a < n/2
// (shift a) and cell n - a when 1 <= a <= n - n/2 (shift -a).  FP32 fields
// take y_a y_b in FP32.
template <class Real>
__global__ void octant_key_hist_kernel(Geom g, const Real* xi_re,
                                       const Real* xi_im, int ell_a, int m_a,
                                       int ell_b, int m_b, double cna,
                                       double cnb, double* hist,
                                       double* rkey) {
  const bool trivial = (ell_a == 0 && m_a == 0 && ell_b == 0 && m_b == 0);
  const int dx = g.n[0] - g.n[0] / 2 + 1, dy = g.n[1] - g.n[1] / 2 + 1,
            dz = g.n[2] - g.n[2] / 2 + 1;
  const int64_t nk = int64_t(dx) * dy * dz;
  // Cell of key index a along an axis of n cells: side 0 is cell a, side 1
  // cell n - a; -1 where the side holds none.
  auto cell_of = [](int a, int n, int side) {
    if (side == 0) return a < n / 2 ? a : -1;
    return (a >= 1 && a <= n - n / 2) ? n - a : -1;
  };
  for (int64_t key = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       key < nk; key += int64_t(gridDim.x) * blockDim.x) {
    const int c = int(key % dz);
    const int b = int((key / dz) % dy);
    const int a = int(key / (int64_t(dz) * dy));
    double sre = 0., sim = 0.;
    for (int fx = 0; fx < 2; ++fx) {
      const int i = cell_of(a, g.n[0], fx);
      if (i < 0) continue;
      const int sx = shift_index(i, g.n[0]);
      for (int fy = 0; fy < 2; ++fy) {
        const int j = cell_of(b, g.n[1], fy);
        if (j < 0) continue;
        const int sy = shift_index(j, g.n[1]);
        for (int fz = 0; fz < 2; ++fz) {
          const int k = cell_of(c, g.n[2], fz);
          if (k < 0) continue;
          const int sz = shift_index(k, g.n[2]);
          const int64_t t = (int64_t(i) * g.n[1] + j) * g.n[2] + k;
          const double vr = double(xi_re[t]);
          const double vi = xi_im != nullptr ? double(xi_im[t]) : 0.;
          if (trivial) {
            sre += vr;
            sim += vi;
            continue;
          }
          if constexpr (sizeof(Real) == 4) {
            const float rx = float(sx) * float(g.dr[0]);
            const float ry = float(sy) * float(g.dr[1]);
            const float rz = float(sz) * float(g.dr[2]);
            const float r = sqrtf(rx * rx + ry * ry + rz * rz);
            if (r < 1.e-9f) continue;
            const float inv = 1.f / r;
            const float2 u = make_float2(rx * inv, -ry * inv);
            const float2 ya = ylm_lean_f(ell_a, m_a, float(cna), rz * inv, u);
            const float2 yb = ylm_lean_f(ell_b, m_b, float(cnb), rz * inv, u);
            const float2 y = make_float2(ya.x * yb.x - ya.y * yb.y,
                                         ya.x * yb.y + ya.y * yb.x);
            const float fr = float(vr), fi = float(vi);
            sre += double(fr * y.x - fi * y.y);
            sim += double(fr * y.y + fi * y.x);
          } else {
            const double rx = dmul(double(sx), g.dr[0]);
            const double ry = dmul(double(sy), g.dr[1]);
            const double rz = dmul(double(sz), g.dr[2]);
            const double r = dsqrt(dadd(dadd(dmul(rx, rx), dmul(ry, ry)),
                                        dmul(rz, rz)));
            if (fabs(r) < 1.e-9) continue;
            const double inv = 1.0 / r;
            const cd u = cmk(rx * inv, -ry * inv);
            const cd y = ylm_lean(ell_a, m_a, cna, rz * inv, u) *
                         ylm_lean(ell_b, m_b, cnb, rz * inv, u);
            sre += vr * y.re - vi * y.im;
            sim += vr * y.im + vi * y.re;
          }
        }
      }
    }
    hist[2 * key] = sre;
    hist[2 * key + 1] = sim;
    rkey[key] = vec3_mag(dmul(double(a), g.dr[0]), dmul(double(b), g.dr[1]),
                         dmul(double(c), g.dr[2]));
  }
}

template <class Real>
__global__ void __launch_bounds__(256)
shotnoise_3pcf_kernel(Geom g, const Real* xi_re, const Real* xi_im, int ell_a,
                      int m_a, int ell_b, int m_b, BinsDev bins,
                      long long* npairs, double* rsum, double* xi) {
  extern __shared__ unsigned char smem_raw[];
  double* s_r = reinterpret_cast<double*>(smem_raw);
  double* s_xi = s_r + bins.nbins;
  long long* s_n = reinterpret_cast<long long*>(s_xi + 2 * bins.nbins);
  for (int q = threadIdx.x; q < bins.nbins; q += blockDim.x) {
    s_r[q] = 0.;
    s_xi[2 * q] = s_xi[2 * q + 1] = 0.;
    s_n[q] = 0;
  }
  __syncthreads();
  const int n_sample = 100000;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       t < g.nmesh; t += int64_t(gridDim.x) * blockDim.x) {
    const int k = int(t % g.n[2]);
    const int j = int((t / g.n[2]) % g.n[1]);
    const int i = int(t / (int64_t(g.n[2]) * g.n[1]));
    const int sx = shift_index(i, g.n[0]), sy = shift_index(j, g.n[1]),
              sz = shift_index(k, g.n[2]);
    // Beyond every bin by an integer test (no FP64 for most cells).
    if (bins.key_max >= 0 &&
        int64_t(sx) * sx + int64_t(sy) * sy + int64_t(sz) * sz > bins.key_max)
      continue;
    const double rx = dmul(double(sx), g.dr[0]);
    const double ry = dmul(double(sy), g.dr[1]);
    const double rz = dmul(double(sz), g.dr[2]);
    const double r = vec3_mag(rx, ry, rz);
    const int idx_r = int(ddiv(r, 1.));
    if (idx_r < 0 || idx_r >= n_sample) continue;
    bool any = false;
    for (int q = 0; q < bins.nbins; ++q)
      any |= (bins.smin[q] <= idx_r && idx_r < bins.smax[q]);
    if (!any) continue;
    cd v = {double(xi_re[t]), xi_im != nullptr ? double(xi_im[t]) : 0.};
    v = v * (reduced_ylm(ell_a, m_a, rx, ry, rz) *
             reduced_ylm(ell_b, m_b, rx, ry, rz));
    for (int q = 0; q < bins.nbins; ++q) {
      if (bins.smin[q] <= idx_r && idx_r < bins.smax[q]) {
        atomicAdd(reinterpret_cast<unsigned long long*>(s_n + q), 1ull);
        atomicAdd(s_r + q, r);
        atomicAdd(s_xi + 2 * q, v.re);
        atomicAdd(s_xi + 2 * q + 1, v.im);
      }
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < bins.nbins; q += blockDim.x) {
    if (s_n[q] == 0) continue;
    atomicAdd(reinterpret_cast<unsigned long long*>(npairs + q),
              (unsigned long long)s_n[q]);
    atomicAdd(rsum + q, s_r[q]);
    atomicAdd(xi + 2 * q, s_xi[2 * q]);
    atomicAdd(xi + 2 * q + 1, s_xi[2 * q + 1]);
  }
}

}  // namespace

template <class Real>
void launch_reduce_pairs(Context& ctx, int64_t ncell,
                         const typename CplxOf<Real>::type* G,
                         const typename CplxOf<Real>::type* Fa,
                         const typename CplxOf<Real>::type* Fb,
                         const int* pa, const int* pb, int npairs,
                         double* out, int na, int nb, bool conj_b) {
  if (npairs <= 0) return;
  if constexpr (sizeof(Real) == 4) {
    const size_t smem = size_t(na + nb) * kRedRow * sizeof(float2);
    if (!conj_b && na > 0 && nb > 0 && smem <= 200 * 1024) {
      static bool configured[64] = {};
      if (ctx.device < 0 || ctx.device >= 64 || !configured[ctx.device]) {
        TRVG_CUDA(cudaFuncSetAttribute(
            reduce_pairs_gram_kernel,
            cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        if (ctx.device >= 0 && ctx.device < 64) configured[ctx.device] = true;
      }
      const int per_block = 256 * kRedPairsPerThread;
      const int64_t tiles = (ncell + kRedTile - 1) / kRedTile;
      dim3 grid(unsigned(std::min<int64_t>(tiles, 152 * 8)),
                unsigned((npairs + per_block - 1) / per_block));
      TRVG_KBEGIN(ctx, "reduce_pairs_kernel");
      reduce_pairs_gram_kernel<<<grid, 256, smem, ctx.stream>>>(
          ncell, G, Fa, na, Fb, nb, pa, pb, npairs, out);
      TRVG_LAUNCHED(ctx);
      return;
    }
  }
  const int chunks = (npairs + kPairChunk - 1) / kPairChunk;
  dim3 grid(grid_for(ncell, 256, 152 * 8), chunks);
  TRVG_KBEGIN(ctx, "reduce_pairs_kernel");
  reduce_pairs_kernel<Real><<<grid, 256, 0, ctx.stream>>>(
      ncell, G, Fa, Fb, pa, pb, npairs, out, conj_b);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_reduce_pairs_real(Context& ctx, int64_t ncell, const Real* G,
                              const Real* Fa, const Real* Fb, const int* pa,
                              const int* pb, int npairs, double* out, int na,
                              int nb) {
  if (npairs <= 0) return;
  if constexpr (sizeof(Real) == 4) {
    const size_t smem = size_t(na + nb) * kRedRow * sizeof(float);
    if (na > 0 && nb > 0 && smem <= 200 * 1024) {
      static bool configured[64] = {};
      if (ctx.device < 0 || ctx.device >= 64 || !configured[ctx.device]) {
        TRVG_CUDA(cudaFuncSetAttribute(
            reduce_pairs_gram_real_kernel,
            cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        if (ctx.device >= 0 && ctx.device < 64) configured[ctx.device] = true;
      }
      const int per_block = 256 * kRedPairsPerThread;
      const int64_t tiles = (ncell + kRedTile - 1) / kRedTile;
      dim3 grid(unsigned(std::min<int64_t>(tiles, 152 * 8)),
                unsigned((npairs + per_block - 1) / per_block));
      TRVG_KBEGIN(ctx, "reduce_pairs_kernel");
      reduce_pairs_gram_real_kernel<<<grid, 256, smem, ctx.stream>>>(
          ncell, G, Fa, na, Fb, nb, pa, pb, npairs, out);
      TRVG_LAUNCHED(ctx);
      return;
    }
  }
  const int chunks = (npairs + kPairChunk - 1) / kPairChunk;
  dim3 grid(grid_for(ncell, 256, 152 * 8), chunks);
  TRVG_KBEGIN(ctx, "reduce_pairs_kernel");
  reduce_pairs_real_kernel<Real><<<grid, 256, 0, ctx.stream>>>(
      ncell, G, Fa, Fb, pa, pb, npairs, out);
  TRVG_LAUNCHED(ctx);
}

namespace {

// Cells per staged chunk, values per staged row and shared memory of the
// tiled Gram form.
int gram_cells(bool cplx) { return cplx ? 64 : 128; }

void gram_rows(bool cplx, int na, int nb, int& rsa, int& rsb) {
  const GramTile t = gram_tile(cplx);
  // Rows padded to whole tiles and 16-byte vectors.
  const int va = cplx ? 2 : 4;
  rsa = (na + t.ti - 1) / t.ti * t.ti;
  rsa = (rsa + va - 1) / va * va;
  rsb = (nb + t.tj - 1) / t.tj * t.tj;
  rsb = (rsb + va - 1) / va * va;
}

size_t gram_smem(bool cplx, int na, int nb) {
  int rsa, rsb;
  gram_rows(cplx, na, nb, rsa, rsb);
  const GramTile t = gram_tile(cplx);
  const int w = cplx ? 2 : 1;
  // Two staging buffers of leg a, leg b and G.
  const size_t stage =
      2 * size_t(gram_cells(cplx)) * (rsa + rsb + 1) * w * 4;
  const size_t red = size_t(kGramThreads) * t.ti * t.tj * w * 8;
  return std::max(stage, red);
}

constexpr size_t kGramSmemMax = 112 * 1024;  // two blocks per SM

}  // namespace

bool gram_tiled_fits(bool cplx, int na, int nb) {
  return na > 0 && nb > 0 && gram_smem(cplx, na, nb) <= kGramSmemMax;
}

void launch_reduce_pairs_tiled(Context& ctx, int64_t ncell, bool cplx,
                               const float* G, const float* Fa, int na,
                               const float* Fb, int nb, const int2* tiles,
                               int ntiles, const int* slot, double* out,
                               int64_t ld) {
  if (ntiles <= 0 || ncell <= 0) return;
  if (ld == 0) ld = ncell;
  if (ld < ncell)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Tiled pair sums: field stride %lld below %lld cells.",
                (long long)ld, (long long)ncell);
  if (!gram_tiled_fits(cplx, na, nb))
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Tiled pair sums: %d x %d fields exceed the staged chunk.",
                na, nb);
  int rsa, rsb;
  gram_rows(cplx, na, nb, rsa, rsb);
  const size_t smem = gram_smem(cplx, na, nb);
  // One field set for both legs: stage it once.
  const bool same = Fa == Fb && na == nb;
  // Multiplier of the division by rsb in the F_b G pass (rsb < 2^8, the
  // dividend below rsb * cells < 2^16).
  const unsigned mrsb = unsigned((uint64_t(1) << 32) / unsigned(rsb) + 1);
  const int cells = gram_cells(cplx);
  const int64_t chunks = (ncell + cells - 1) / cells;
  dim3 grid(unsigned(std::min<int64_t>(chunks, 152 * 2)),
            unsigned((ntiles + kGramThreads - 1) / kGramThreads));
  // Both kernels have one function-pointer type, so the opt-in flags are
  // kept per form (real, complex) and device.
  static bool configured[2][64] = {};
  auto go = [&](auto kernel) {
    bool* done = (ctx.device >= 0 && ctx.device < 64)
                     ? &configured[cplx ? 1 : 0][ctx.device]
                     : nullptr;
    if (done == nullptr || !*done) {
      TRVG_CUDA(cudaFuncSetAttribute(
          kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
          int(kGramSmemMax)));
      if (done != nullptr) *done = true;
    }
    TRVG_KBEGIN(ctx, "reduce_pairs_tiled_kernel");
    kernel<<<grid, kGramThreads, smem, ctx.stream>>>(
        ncell, G, Fa, na, rsa, Fb, nb, rsb, mrsb, same, tiles, ntiles, slot,
        out, ld);
    TRVG_LAUNCHED(ctx);
  };
  // Row-major staging with 16-byte copies when every row starts on a
  // 16-byte boundary (field stride a multiple of 4 / floats per value).
  const int w = cplx ? 2 : 1;
  const int nrow_all = rsa + rsb + 1;
  const size_t smem_rows =
      std::max(2 * (size_t(nrow_all) * (cells * w + 4) +
                    4 * size_t(nrow_all >> 3) + 4) * 4,
               size_t(kGramThreads) * gram_tile(cplx).ti *
                   gram_tile(cplx).tj * w * 8);
  if (!ctx.gram_per_pair && (ld * w) % 4 == 0 &&
      smem_rows <= kGramSmemMax) {
    static bool rows_configured[2][64] = {};
    bool* done = (ctx.device >= 0 && ctx.device < 64)
                     ? &rows_configured[cplx ? 1 : 0][ctx.device]
                     : nullptr;
    auto rows = [&](auto kernel) {
      if (done == nullptr || !*done) {
        TRVG_CUDA(cudaFuncSetAttribute(
            kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
            int(kGramSmemMax)));
        if (done != nullptr) *done = true;
      }
      TRVG_KBEGIN(ctx, "reduce_pairs_tiled_kernel");
      kernel<<<grid, kGramThreads, smem_rows, ctx.stream>>>(
          ncell, G, Fa, na, rsa, Fb, nb, rsb, same, tiles, ntiles, slot, out,
          ld);
      TRVG_LAUNCHED(ctx);
    };
    if (cplx)
      rows(reduce_pairs_rows_kernel<true, 2, 4, 64>);
    else
      rows(reduce_pairs_rows_kernel<false, 4, 8, 128>);
    return;
  }
  if (cplx)
    go(reduce_pairs_tiled_kernel<true, 2, 4, 64>);
  else
    go(reduce_pairs_tiled_kernel<false, 4, 8, 128>);
}

void launch_reduce_pairs_ff(Context& ctx, int64_t ncell, int64_t ld,
                            const float* Gh, const float* Gl,
                            const float* Fah, const float* Fal,
                            const float* Fbh, const float* Fbl, const int* pa,
                            const int* pb, int npairs, double* out,
                            int pairs_per_block) {
  if (npairs <= 0) return;
  if (ld % 4 != 0 || ld < ncell)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Field stride %lld is not a multiple of 4 cells >= %lld.",
                (long long)ld, (long long)ncell);
  auto go = [&](auto kernel, int chunk) {
    dim3 grid(grid_for((ncell + 3) / 4, 256, 152 * 4),
              (npairs + chunk - 1) / chunk);
    TRVG_KBEGIN(ctx, "reduce_pairs_kernel");
    kernel<<<grid, 256, 0, ctx.stream>>>(ncell, ld, Gh, Gl, Fah, Fal, Fbh,
                                         Fbl, pa, pb, npairs, out);
  };
  switch (pairs_per_block) {
    case 4: go(reduce_pairs_ff_kernel<4>, 4); break;
    case 16: go(reduce_pairs_ff_kernel<16>, 16); break;
    default: go(reduce_pairs_ff_kernel<8>, 8); break;
  }
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_radial_hist(Context& ctx, const Geom& g, const Real* xi_re,
                        const Real* xi_im, int ell_a, int m_a, int ell_b,
                        int m_b, double* hist) {
  const bool even = (g.n[0] % 2 == 0) && (g.n[1] % 2 == 0) &&
                    (g.n[2] % 2 == 0);
  if (even) {
    const bool swap = g.n[0] == g.n[1];
    const int hx = g.n[0] / 2, hy = g.n[1] / 2, hz = g.n[2] / 2;
    const int nblocks =
        swap ? (hx + 1) * (hx + 2) / 2 : (hx + 1) * (hy + 1);
    const int threads = std::min(256, ((hz + 1 + 31) / 32) * 32);
    const bool trivial = ell_a == 0 && m_a == 0 && ell_b == 0 && m_b == 0;
    const bool axial = m_a == 0 && m_b == 0 && (ell_a + ell_b) % 2 == 0;
    TRVG_KBEGIN(ctx, "orbit_rows_kernel");
    if (trivial)
      orbit_rows_kernel<Real, 0><<<nblocks, threads, 0, ctx.stream>>>(
          g, xi_re, xi_im, ell_a, m_a, ell_b, m_b, swap, hist);
    else if (axial)
      orbit_rows_kernel<Real, 1><<<nblocks, threads, 0, ctx.stream>>>(
          g, xi_re, xi_im, ell_a, m_a, ell_b, m_b, swap, hist);
    else
      orbit_rows_kernel<Real, 2><<<nblocks, threads, 0, ctx.stream>>>(
          g, xi_re, xi_im, ell_a, m_a, ell_b, m_b, swap, hist);
    TRVG_LAUNCHED(ctx);
    return;
  }
  TRVG_KBEGIN(ctx, "radial_hist_kernel");
  radial_hist_kernel<Real><<<grid_for(g.nmesh, 256), 256, 0, ctx.stream>>>(
      g, xi_re, xi_im, ell_a, m_a, ell_b, m_b, hist);
  TRVG_LAUNCHED(ctx);
}

void launch_octant_hist(Context& ctx, const Geom& g, const float2* xo,
                        int ell_a, int ell_b, double* hist) {
  dim3 grid(g.n[1] / 2 + 1, g.n[2] / 2 + 1);
  const int threads = std::min(256, ((g.n[0] / 2 + 1 + 31) / 32) * 32);
  TRVG_KBEGIN(ctx, "orbit_rows_kernel");
  if (ell_a == 0 && ell_b == 0)
    octant_hist_kernel<0><<<grid, threads, 0, ctx.stream>>>(g, xo, ell_a,
                                                            ell_b, hist);
  else
    octant_hist_kernel<1><<<grid, threads, 0, ctx.stream>>>(g, xo, ell_a,
                                                            ell_b, hist);
  TRVG_LAUNCHED(ctx);
}

void launch_pair_bessel_sums(Context& ctx, const Geom& g, int64_t nkeys,
                             const double* hist, const SplineTable& sja,
                             const SplineTable& sjb, const double* ka,
                             const double* kb, int npairs, bool ff,
                             double* out, const double* rkey) {
  if (npairs <= 0) return;
  PairBesselArgs a{sja, sjb, ka, kb};
  const bool same_leg = sja.ell == sjb.ell;
  const int chunks = (npairs + kKeyPairChunk - 1) / kKeyPairChunk;
  dim3 grid(grid_for(nkeys, 256, 152 * 2), chunks);
  TRVG_KBEGIN(ctx, "pair_bessel_sums_kernel");
  if (ff && sja.q != nullptr && sjb.q != nullptr)
    pair_bessel_sums_ff_kernel<<<grid, 256, 0, ctx.stream>>>(
        nkeys, g.dr[0], rkey, hist, a, npairs, same_leg, out);
  else
    pair_bessel_sums_kernel<<<grid, 256, 0, ctx.stream>>>(
        nkeys, g.dr[0], rkey, hist, a, npairs, same_leg, out);
  TRVG_LAUNCHED(ctx);
}

// The Gram form of pair_bessel_sums_ff_kernel; false when its shared
// memory would not fit (the caller then uses launch_pair_bessel_sums).
bool launch_pair_bessel_gram(Context& ctx, const Geom& g, int64_t nkeys,
                             const double* hist, const SplineTable& sja,
                             const SplineTable& sjb, const double* ka_d,
                             int nka, const double* kb_d, int nkb, bool same,
                             const int* pa, const int* pb, int npairs,
                             double* out, const double* rkey) {
  if (npairs <= 0) return true;
  if (sja.q == nullptr || sjb.q == nullptr) return false;
  const int nrows = nka + (same ? 0 : nkb);
  const size_t smem = size_t(nrows) * kGramRow * sizeof(float2) +
                      kGramKeys * sizeof(float4);
  if (smem > 200 * 1024) return false;
  static bool configured[64] = {};
  if (ctx.device < 0 || ctx.device >= 64 || !configured[ctx.device]) {
    TRVG_CUDA(cudaFuncSetAttribute(pair_bessel_gram_ff_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   200 * 1024));
    if (ctx.device >= 0 && ctx.device < 64) configured[ctx.device] = true;
  }
  GramArgs a{sja, sjb, ka_d, kb_d, nka, nkb, same, pa, pb};
  const int per_block = 256 * kGramPairsPerThread;
  const int64_t chunks = (nkeys + kGramKeys - 1) / kGramKeys;
  dim3 grid(unsigned(std::min<int64_t>(chunks, 152 * 4)),
            unsigned((npairs + per_block - 1) / per_block));
  TRVG_KBEGIN(ctx, "pair_bessel_sums_kernel");
  pair_bessel_gram_ff_kernel<<<grid, 256, smem, ctx.stream>>>(
      nkeys, g.dr[0], rkey, hist, a, npairs, out);
  TRVG_LAUNCHED(ctx);
  return true;
}

template <class Real>
void launch_octant_cell_hist(Context& ctx, const Geom& g, const Real* xi_re,
                             const Real* xi_im, int ell_a, int m_a, int ell_b,
                             int m_b, double* hist, double* rkey) {
  const int64_t nk = int64_t(g.n[0] - g.n[0] / 2 + 1) *
                     (g.n[1] - g.n[1] / 2 + 1) * (g.n[2] - g.n[2] / 2 + 1);
  double na[kMaxYlmDegree + 1], nb[kMaxYlmDegree + 1];
  if (ell_a > kMaxYlmDegree || ell_b > kMaxYlmDegree)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Degree above %d.",
                kMaxYlmDegree);
  ylm_all_norms(ell_a, na);
  ylm_all_norms(ell_b, nb);
  TRVG_KBEGIN(ctx, "orbit_rows_kernel");
  octant_key_hist_kernel<Real><<<grid_for(nk, 256), 256, 0, ctx.stream>>>(
      g, xi_re, xi_im, ell_a, m_a, ell_b, m_b, na[std::abs(m_a)],
      nb[std::abs(m_b)], hist, rkey);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_shotnoise_3pcf_bins(Context& ctx, const Geom& g, const Real* xi_re,
                                const Real* xi_im, int ell_a, int m_a,
                                int ell_b, int m_b, const BinsDev& bins,
                                long long* npairs, double* rsum, double* xi) {
  const size_t smem = bins.nbins * (3 * sizeof(double) + sizeof(long long));
  TRVG_KBEGIN(ctx, "shotnoise_3pcf_kernel");
  shotnoise_3pcf_kernel<Real><<<grid_for(g.nmesh, 256), 256, smem,
                                ctx.stream>>>(g, xi_re, xi_im, ell_a, m_a,
                                              ell_b, m_b, bins, npairs, rsum,
                                              xi);
  TRVG_LAUNCHED(ctx);
}

#define TRVG_INST(R)                                                          \
  template void launch_reduce_pairs<R>(Context&, int64_t,                     \
                                       const CplxOf<R>::type*,                \
                                       const CplxOf<R>::type*,                \
                                       const CplxOf<R>::type*, const int*,    \
                                       const int*, int, double*, int, int,    \
                                       bool);                                 \
  template void launch_reduce_pairs_real<R>(Context&, int64_t, const R*,     \
                                            const R*, const R*, const int*,   \
                                            const int*, int, double*, int,    \
                                            int);                             \
  template void launch_radial_hist<R>(Context&, const Geom&, const R*,        \
                                      const R*, int, int, int, int, double*); \
  template void launch_octant_cell_hist<R>(Context&, const Geom&, const R*,   \
                                           const R*, int, int, int, int,      \
                                           double*, double*);                 \
  template void launch_shotnoise_3pcf_bins<R>(                                \
      Context&, const Geom&, const R*, const R*, int, int, int, int,          \
      const BinsDev&, long long*, double*, double*);
TRVG_INST(float)
TRVG_INST(double)
#undef TRVG_INST

}  // namespace trvg
