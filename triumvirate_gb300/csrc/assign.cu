// K1: particle -> mesh assignment (NGP / CIC / TSC / PCS, with the
// interlacing shadow in the same pass).
//
// Follows MeshField::assign_weighted_field_to_mesh_{ngp,cic,tsc,pcs}
// (field.cpp:618-1112): per axis the covered cell indices and window values
// are derived from loc = ngrid * x / L exactly as there (FP64, same
// comparisons and periodic wrap), and the product window * weight is
// accumulated with atomics.  The mesh stores the deposited weight per cell
// (the reference's n(x) * dV), which is what its forward FFT consumes after
// the vol_cell scaling (field.cpp:1503-1510).
#include <type_traits>

#include "ff.cuh"
#include "kernels.h"
#include "stencil.cuh"

namespace trvg {

namespace {

__device__ __forceinline__ void atomic_add_real(float* p, float v) {
  atomicAdd(p, v);
}
__device__ __forceinline__ void atomic_add_real(double* p, double v) {
  atomicAdd(p, v);
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

struct AssignArgs {
  int n[3];
  double L[3];
  double ratio[3];  // n / L
  int64_t nmesh;
  DevCatalogue cat;
  WeightSpec ws;
  bool vec4;        // z rows 16-byte aligned in every target mesh
  // Compensated FP32 deposit: each target mesh has a second FP32 mesh
  // lo_off elements after it that collects the rounding errors of the
  // products and of the atomic sums (0: none).
  int64_t lo_off;
};

// Rounding error of s = fl(a + b): a + b = s + err exactly (Knuth's
// TwoSum; the _rn intrinsics keep the compiler from contracting it).
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
  const float bb = __fsub_rn(s, a);
  return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Compensated atomic add of the float-float value (vh, vl) to cell p: the
// add to p returns the cell's previous value, from which the exact
// rounding error of the add follows (a float atomic add rounds to
// nearest); the error and vl go to the compensation cell.
__device__ __forceinline__ void atomic_add_comp(float* p, int64_t lo_off,
                                                float vh, float vl) {
  const float old = atomicAdd(p, vh);
  const float e = __fadd_rn(two_sum_err(old, vh, __fadd_rn(old, vh)), vl);
  if (e != 0.f) atomicAdd(p + lo_off, e);
}

// ---- FP32-mesh fast stencil ------------------------------------------------
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so for FP32 meshes
// FP64 enters only in loc = x * (n / L) and its split into cell index and
// offset; windows and products are FP32.  The multiply by the ratio differs
// from the library's (n x) / L by a few ulps of loc (< 1e-12 here), which
// can change a cell choice only when the offset lies that close to 0, 1/2
// or 1 (the cell edge, the TSC / NGP split and the interlacing shadow's
// half-cell shift).  Particles whose offset lies within kTieMargin of those
// values, or outside [0, L), take the exact FP64 stencil instead.

constexpr float kTieMargin = 1e-6f;

template <int ORDER>
struct StencilF {
  int idx[ORDER];
  float win[ORDER];
};

// Cell indices (the same branches as axis_stencil) and FP32 windows for the
// offset s of cell idx.
template <int ORDER>
__device__ __forceinline__ void fill_stencil_f(int idx, float s, int n,
                                               bool shadow,
                                               StencilF<ORDER>& st) {
  if (ORDER == 1) {
    int i0 = idx;
    if (s >= 0.5f) i0 = (idx == n - 1) ? 0 : idx + 1;
    st.idx[0] = i0;
    st.win[0] = 1.f;
  } else if (ORDER == 2) {
    st.idx[0] = idx;
    st.idx[1] = (idx == n - 1) ? 0 : idx + 1;
    st.win[0] = 1.f - s;
    st.win[1] = s;
  } else if (ORDER == 3) {
    if (s < 0.5f) {
      st.idx[0] = (idx == 0) ? n - 1 : idx - 1;
      st.idx[1] = idx;
      st.idx[2] = (idx == n - 1) ? 0 : idx + 1;
      st.win[0] = 0.5f * (0.5f - s) * (0.5f - s);
      st.win[1] = 0.75f - s * s;
      st.win[2] = 0.5f * (0.5f + s) * (0.5f + s);
    } else {
      st.idx[0] = idx;
      st.idx[1] = (idx == n - 1) ? 0 : idx + 1;
      if (shadow) {
        st.idx[2] = (idx == n - 1) ? 0 : st.idx[1] + 1;
      } else {
        st.idx[2] = (st.idx[1] == n - 1) ? 0 : st.idx[1] + 1;
      }
      const float t = 1.f - s;
      st.win[0] = 0.5f * (0.5f + t) * (0.5f + t);
      st.win[1] = 0.75f - t * t;
      st.win[2] = 0.5f * (0.5f - t) * (0.5f - t);
    }
  } else {
    st.idx[0] = (idx == 0) ? n - 1 : idx - 1;
    st.idx[1] = idx;
    st.idx[2] = (idx == n - 1) ? 0 : idx + 1;
    st.idx[3] = (st.idx[2] == n - 1) ? 0 : st.idx[2] + 1;
    const float t = 1.f - s;
    const float c = 1.f / 6.f;
    st.win[0] = c * t * t * t;
    st.win[1] = c * (4.f - 6.f * s * s + 3.f * s * s * s);
    st.win[2] = c * (4.f - 6.f * t * t + 3.f * t * t * t);
    st.win[3] = c * s * s * s;
  }
}

// The same stencil with float-float windows (about 2^-44 relative), for
// the compensated deposit: the offset s = s.hi + s.lo carries the 48
// leading fraction bits of loc, and every window is formed from it with
// error-free float operations (1 - s, 1/2 +- s and 3/2 - s are exact in
// s.hi because s.hi holds 24 fraction bits).
template <int ORDER>
struct StencilFF {
  int idx[ORDER];
  FF win[ORDER];
};

__device__ __forceinline__ FF ff_const(float v) { return FF{v, 0.f}; }

template <int ORDER>
__device__ __forceinline__ void fill_stencil_ff(int idx, FF s, int n,
                                                bool shadow,
                                                StencilFF<ORDER>& st) {
  if (ORDER == 1) {
    int i0 = idx;
    if (s.hi >= 0.5f) i0 = (idx == n - 1) ? 0 : idx + 1;
    st.idx[0] = i0;
    st.win[0] = ff_const(1.f);
  } else if (ORDER == 2) {
    st.idx[0] = idx;
    st.idx[1] = (idx == n - 1) ? 0 : idx + 1;
    st.win[0] = FF{1.f - s.hi, -s.lo};
    st.win[1] = s;
  } else if (ORDER == 3) {
    if (s.hi < 0.5f) {
      st.idx[0] = (idx == 0) ? n - 1 : idx - 1;
      st.idx[1] = idx;
      st.idx[2] = (idx == n - 1) ? 0 : idx + 1;
      const FF u = FF{0.5f - s.hi, -s.lo}, v = FF{0.5f + s.hi, s.lo};
      st.win[0] = ffscale2(ffmul(u, u), 0.5f);
      st.win[1] = ffsub(ff_const(0.75f), ffmul(s, s));
      st.win[2] = ffscale2(ffmul(v, v), 0.5f);
    } else {
      st.idx[0] = idx;
      st.idx[1] = (idx == n - 1) ? 0 : idx + 1;
      if (shadow) {
        st.idx[2] = (idx == n - 1) ? 0 : st.idx[1] + 1;
      } else {
        st.idx[2] = (st.idx[1] == n - 1) ? 0 : st.idx[1] + 1;
      }
      const FF t = FF{1.f - s.hi, -s.lo};
      const FF u = FF{1.5f - s.hi, -s.lo}, v = FF{s.hi - 0.5f, s.lo};
      st.win[0] = ffscale2(ffmul(u, u), 0.5f);
      st.win[1] = ffsub(ff_const(0.75f), ffmul(t, t));
      st.win[2] = ffscale2(ffmul(v, v), 0.5f);
    }
  } else {
    st.idx[0] = (idx == 0) ? n - 1 : idx - 1;
    st.idx[1] = idx;
    st.idx[2] = (idx == n - 1) ? 0 : idx + 1;
    st.idx[3] = (st.idx[2] == n - 1) ? 0 : st.idx[2] + 1;
    const FF t = FF{1.f - s.hi, -s.lo};
    const FF c = FF{0x1.555556p-3f, -0x1.555556p-28f};  // 1/6
    const FF s2 = ffmul(s, s), s3 = ffmul(s2, s);
    const FF t2 = ffmul(t, t), t3 = ffmul(t2, t);
    st.win[0] = ffmul(c, t3);
    st.win[1] = ffmul(c, ffadd(ffadd(ff_const(4.f), ffmul(ff_const(-6.f), s2)),
                               ffmul(ff_const(3.f), s3)));
    st.win[2] = ffmul(c, ffadd(ffadd(ff_const(4.f), ffmul(ff_const(-6.f), t2)),
                               ffmul(ff_const(3.f), t3)));
    st.win[3] = ffmul(c, s3);
  }
}

// Main (and, if `shadow` is given, shadow) stencil of one axis; false when
// the particle must take the exact path.  The shadow cell follows from the
// main one: loc + 1/2 stays in cell idx when s < 1/2 and moves to the next
// cell (wrapping to 0 past the last, as the library's loc -= n does)
// otherwise.
// Cell index (the truncation of loc) and the leading 24 bits of the
// fraction of loc >= 0, read from the bits of the double with integer
// operations (GB300 converts FP64 on its slow FP64 pipe).  idx is -1 for
// negative offsets and INT_MAX at or above 2^30; both fail the range test.
__device__ __forceinline__ void split_offset(double loc, int& idx, float& s) {
  const long long bits = __double_as_longlong(loc);
  const int e = int((bits >> 52) & 0x7ff) - 1023;
  if (bits < 0) {
    idx = -1;
    s = 0.f;
  } else if (e < 0) {  // 0 <= loc < 1 (zero and subnormals included)
    idx = 0;
    s = float(loc);
  } else if (e >= 30) {
    idx = 0x7fffffff;
    s = 0.f;
  } else {
    const unsigned long long m =
        (static_cast<unsigned long long>(bits) & ((1ull << 52) - 1)) |
        (1ull << 52);
    const int sh = 52 - e;  // fraction bits, 23..52
    idx = int(m >> sh);
    const unsigned long long f = m & ((1ull << sh) - 1);
    s = sh > 24 ? float(unsigned(f >> (sh - 24))) * 0x1p-24f
                : ldexpf(float(unsigned(f)), -sh);
  }
}

// split_offset with the fraction as float-float: s.hi the leading 24 bits
// (as split_offset gives them), s.lo the next ones.
__device__ __forceinline__ void split_offset_ff(double loc, int& idx, FF& s) {
  const long long bits = __double_as_longlong(loc);
  const int e = int((bits >> 52) & 0x7ff) - 1023;
  if (bits < 0) {
    idx = -1;
    s = FF{0.f, 0.f};
  } else if (e < 0) {  // 0 <= loc < 1: the rare cell 0 takes FP64 once
    idx = 0;
    const float h = float(loc);
    s = FF{h, float(loc - double(h))};
  } else if (e >= 30) {
    idx = 0x7fffffff;
    s = FF{0.f, 0.f};
  } else {
    const unsigned long long m =
        (static_cast<unsigned long long>(bits) & ((1ull << 52) - 1)) |
        (1ull << 52);
    const int sh = 52 - e;  // fraction bits, 23..52
    idx = int(m >> sh);
    const unsigned long long f = m & ((1ull << sh) - 1);
    if (sh > 24) {
      s.hi = float(unsigned(f >> (sh - 24))) * 0x1p-24f;
      const unsigned long long r = f & ((1ull << (sh - 24)) - 1);
      s.lo = ldexpf(float(r), -sh);
    } else {
      s = FF{ldexpf(float(unsigned(f)), -sh), 0.f};
    }
  }
}

template <int ORDER>
__device__ __forceinline__ bool axis_stencil_f(double pos, int n, double ratio,
                                               StencilF<ORDER>& main,
                                               StencilF<ORDER>* shadow) {
  const double loc = pos * ratio;
  int idx;
  float s;
  split_offset(loc, idx, s);
  if (idx < 0 || idx >= n || !(s >= kTieMargin) || s > 1.f - kTieMargin ||
      fabsf(s - 0.5f) < kTieMargin)
    return false;
  fill_stencil_f<ORDER>(idx, s, n, false, main);
  if (shadow != nullptr) {
    if (s < 0.5f)
      fill_stencil_f<ORDER>(idx, s + 0.5f, n, true, *shadow);
    else
      fill_stencil_f<ORDER>((idx == n - 1) ? 0 : idx + 1, s - 0.5f, n, true,
                            *shadow);
  }
  return true;
}

// axis_stencil_f with float-float windows (same cells and tie test).
template <int ORDER>
__device__ __forceinline__ bool axis_stencil_ff(double pos, int n,
                                                double ratio,
                                                StencilFF<ORDER>& main,
                                                StencilFF<ORDER>* shadow) {
  const double loc = pos * ratio;
  int idx;
  FF s;
  split_offset_ff(loc, idx, s);
  if (idx < 0 || idx >= n || !(s.hi >= kTieMargin) ||
      s.hi > 1.f - kTieMargin || fabsf(s.hi - 0.5f) < kTieMargin)
    return false;
  fill_stencil_ff<ORDER>(idx, s, n, false, main);
  if (shadow != nullptr) {
    if (s.hi < 0.5f)
      fill_stencil_ff<ORDER>(idx, FF{s.hi + 0.5f, s.lo}, n, true, *shadow);
    else
      fill_stencil_ff<ORDER>((idx == n - 1) ? 0 : idx + 1,
                             FF{s.hi - 0.5f, s.lo}, n, true, *shadow);
  }
  return true;
}

// Adds v[0..ORDER) to the z run starting at cell `z0` of a row beginning at
// `row` (16-byte aligned): one or two float4 atomics, zeros in the lanes
// outside the run (adding 0 leaves a cell unchanged).
template <int ORDER>
__device__ __forceinline__ void red_run4(float* row, int z0, const float* v) {
  const int off = z0 & 3;
  float q[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    float x = 0.f;
#pragma unroll
    for (int k = 0; k < ORDER; ++k) x = (l == off + k) ? v[k] : x;
    q[l] = x;
  }
  float4* p = reinterpret_cast<float4*>(row + (z0 - off));
  atomicAdd(p, make_float4(q[0], q[1], q[2], q[3]));
  if (off + ORDER > 4) atomicAdd(p + 1, make_float4(q[4], q[5], q[6], q[7]));
}

// FP32 window k of a stencil (a float-float window rounded once).
template <int ORDER>
__device__ __forceinline__ float win_f(const StencilF<ORDER>& s, int k) {
  return s.win[k];
}
template <int ORDER>
__device__ __forceinline__ float win_f(const StencilFF<ORDER>& s, int k) {
  return __fadd_rn(s.win[k].hi, s.win[k].lo);
}

template <int ORDER, class St>
__device__ __forceinline__ void deposit_f(const AssignArgs& a, const St& sx,
                                          const St& sy, const St& sz,
                                          float wgt, float* mesh) {
  bool run = a.vec4;
#pragma unroll
  for (int k = 1; k < ORDER; ++k) run = run && (sz.idx[k] == sz.idx[0] + k);
#pragma unroll
  for (int i = 0; i < ORDER; ++i) {
    const float wi = win_f(sx, i) * wgt;
#pragma unroll
    for (int j = 0; j < ORDER; ++j) {
      float* row =
          mesh + (int64_t(sx.idx[i]) * a.n[1] + sy.idx[j]) * a.n[2];
      const float wij = wi * win_f(sy, j);
      float v[ORDER];
#pragma unroll
      for (int k = 0; k < ORDER; ++k) v[k] = wij * win_f(sz, k);
      if (run) {
        red_run4<ORDER>(row, sz.idx[0], v);
      } else {
#pragma unroll
        for (int k = 0; k < ORDER; ++k) atomicAdd(row + sz.idx[k], v[k]);
      }
    }
  }
}

// deposit_f with float-float windows and products, deposited with
// compensated atomics.
template <int ORDER>
__device__ __forceinline__ void deposit_ff(const AssignArgs& a,
                                           const StencilFF<ORDER>& sx,
                                           const StencilFF<ORDER>& sy,
                                           const StencilFF<ORDER>& sz, FF wgt,
                                           bool unit, float* mesh) {
  bool run = a.vec4;
#pragma unroll
  for (int k = 1; k < ORDER; ++k) run = run && (sz.idx[k] == sz.idx[0] + k);
  if (!run) {
#pragma unroll
    for (int i = 0; i < ORDER; ++i) {
      const FF wi = unit ? sx.win[i] : ffmul(sx.win[i], wgt);
#pragma unroll
      for (int j = 0; j < ORDER; ++j) {
        float* row =
            mesh + (int64_t(sx.idx[i]) * a.n[1] + sy.idx[j]) * a.n[2];
        const FF wij = ffmul(wi, sy.win[j]);
#pragma unroll
        for (int k = 0; k < ORDER; ++k) {
          const FF v = ffmul(wij, sz.win[k]);
          atomic_add_comp(row + sz.idx[k], a.lo_off, v.hi, v.lo);
        }
      }
    }
    return;
  }
  // Float4 runs along z.  Per x cell, the value atomics of all its y rows
  // are issued first and their returned values awaited together, so that
  // several round trips to L2 overlap; the compensation atomics follow.
  const int z0 = sz.idx[0], off = z0 & 3;
  const bool two = off + ORDER > 4;
  auto lanes = [&](const FF* v, float* q, float* ql) {
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      float x = 0.f, y = 0.f;
#pragma unroll
      for (int k = 0; k < ORDER; ++k) {
        x = (l == off + k) ? v[k].hi : x;
        y = (l == off + k) ? v[k].lo : y;
      }
      q[l] = x;
      ql[l] = y;
    }
  };
  auto err = [](float o, float h, float l) {
    return __fadd_rn(two_sum_err(o, h, __fadd_rn(o, h)), l);
  };
#pragma unroll
  for (int i = 0; i < ORDER; ++i) {
    const FF wi = unit ? sx.win[i] : ffmul(sx.win[i], wgt);
    float4 o1[ORDER], o2[ORDER];
    FF v[ORDER][ORDER];
#pragma unroll
    for (int j = 0; j < ORDER; ++j) {
      float4* p = reinterpret_cast<float4*>(
          mesh + (int64_t(sx.idx[i]) * a.n[1] + sy.idx[j]) * a.n[2] +
          (z0 - off));
      const FF wij = ffmul(wi, sy.win[j]);
#pragma unroll
      for (int k = 0; k < ORDER; ++k) v[j][k] = ffmul(wij, sz.win[k]);
      float q[8], ql[8];
      lanes(v[j], q, ql);
      o1[j] = atomicAdd(p, make_float4(q[0], q[1], q[2], q[3]));
      if (two) o2[j] = atomicAdd(p + 1, make_float4(q[4], q[5], q[6], q[7]));
    }
#pragma unroll
    for (int j = 0; j < ORDER; ++j) {
      float4* pl = reinterpret_cast<float4*>(
          mesh + a.lo_off +
          (int64_t(sx.idx[i]) * a.n[1] + sy.idx[j]) * a.n[2] + (z0 - off));
      float q[8], ql[8];
      lanes(v[j], q, ql);
      atomicAdd(pl, make_float4(err(o1[j].x, q[0], ql[0]),
                                err(o1[j].y, q[1], ql[1]),
                                err(o1[j].z, q[2], ql[2]),
                                err(o1[j].w, q[3], ql[3])));
      if (two)
        atomicAdd(pl + 1, make_float4(err(o2[j].x, q[4], ql[4]),
                                      err(o2[j].y, q[5], ql[5]),
                                      err(o2[j].z, q[6], ql[6]),
                                      err(o2[j].w, q[7], ql[7])));
    }
  }
}

// Deposit one stencil; returns the weight that landed inside the mesh.
// Stencil indices and window values are FP64 (they decide the cells); the
// products deposited into an FP32 mesh are formed in FP32.  The landed
// weight is w * (sum_i wx_i)(sum_j wy_j)(sum_k wz_k) in FP64 when every
// cell is inside the mesh, and accumulated cell by cell otherwise.
template <int ORDER, class Real>
__device__ __forceinline__ cd deposit(const AssignArgs& a, const double pos[3],
                                      bool shadow, cd wgt, Real* re,
                                      Real* im) {
  Stencil<ORDER> sx = axis_stencil<ORDER>(pos[0], a.n[0], a.L[0], shadow);
  Stencil<ORDER> sy = axis_stencil<ORDER>(pos[1], a.n[1], a.L[1], shadow);
  Stencil<ORDER> sz = axis_stencil<ORDER>(pos[2], a.n[2], a.L[2], shadow);
  Real wx[ORDER], wy[ORDER], wz[ORDER];
  double tx = 0., ty = 0., tz = 0.;
#pragma unroll
  for (int i = 0; i < ORDER; ++i) {
    tx += sx.win[i];
    ty += sy.win[i];
    tz += sz.win[i];
  }
  const Real wre = Real(wgt.re), wim = Real(wgt.im);
#pragma unroll
  for (int i = 0; i < ORDER; ++i) {
    wx[i] = Real(sx.win[i]) * wre;
    wy[i] = Real(sy.win[i]);
    wz[i] = Real(sz.win[i]);
  }
  bool all_in = true;
  cd landed = {0., 0.};
#pragma unroll
  for (int i = 0; i < ORDER; ++i) {
#pragma unroll
    for (int j = 0; j < ORDER; ++j) {
      const int64_t row = (int64_t(sx.idx[i]) * a.n[1] + sy.idx[j]) * a.n[2];
      const Real wij = wx[i] * wy[j];
#pragma unroll
      for (int k = 0; k < ORDER; ++k) {
        const int64_t gid = row + sz.idx[k];
        if (gid < 0 || gid >= a.nmesh) {
          all_in = false;
          continue;
        }
        if constexpr (sizeof(Real) == 4) {
          if (a.lo_off != 0) {
            const double v = sx.win[i] * wgt.re * sy.win[j] * sz.win[k];
            const float vh = float(v);
            atomic_add_comp(re + gid, a.lo_off, vh, float(v - double(vh)));
            continue;
          }
        }
        atomic_add_real(re + gid, wij * wz[k]);
      }
    }
  }
  if (im != nullptr) {
#pragma unroll
    for (int i = 0; i < ORDER; ++i) {
#pragma unroll
      for (int j = 0; j < ORDER; ++j) {
        const int64_t row =
            (int64_t(sx.idx[i]) * a.n[1] + sy.idx[j]) * a.n[2];
        const Real wij = Real(sx.win[i]) * wim * wy[j];
#pragma unroll
        for (int k = 0; k < ORDER; ++k) {
          const int64_t gid = row + sz.idx[k];
          if (gid < 0 || gid >= a.nmesh) continue;
          if constexpr (sizeof(Real) == 4) {
            if (a.lo_off != 0) {
              const double v = sx.win[i] * wgt.im * sy.win[j] * sz.win[k];
              const float vh = float(v);
              atomic_add_comp(im + gid, a.lo_off, vh, float(v - double(vh)));
              continue;
            }
          }
          atomic_add_real(im + gid, wij * wz[k]);
        }
      }
    }
  }
  if (all_in) {
    const double t = tx * ty * tz;
    landed = cd{wgt.re * t, wgt.im * t};
  } else {
#pragma unroll
    for (int i = 0; i < ORDER; ++i)
#pragma unroll
      for (int j = 0; j < ORDER; ++j)
#pragma unroll
        for (int k = 0; k < ORDER; ++k) {
          const int64_t gid =
              (int64_t(sx.idx[i]) * a.n[1] + sy.idx[j]) * a.n[2] + sz.idx[k];
          if (gid < 0 || gid >= a.nmesh) continue;
          const double wv = sx.win[i] * sy.win[j] * sz.win[k];
          landed.re += wgt.re * wv;
          landed.im += wgt.im * wv;
        }
  }
  return landed;
}

// Exact deposit of one particle (main and shadow); out of line in the FP32
// kernel, where only the rare particles near a tie take it.
template <int ORDER, class Real>
__device__ __noinline__ void exact_particle(const AssignArgs& a,
                                            const double* pos, cd wgt,
                                            Real* re, Real* im, Real* sre,
                                            Real* sim, cd* landed) {
  landed[0] = deposit<ORDER, Real>(a, pos, false, wgt, re, im);
  if (sre != nullptr)
    landed[1] = deposit<ORDER, Real>(a, pos, true, wgt, sre, sim);
}

// Fast-path deposit of one particle (main and shadow) into FP32 meshes,
// plain or compensated (COMP, float-float windows); false if the particle
// must take the exact path.
template <int ORDER, bool SH, bool COMP>
__device__ __forceinline__ bool fast_particle(const AssignArgs& a,
                                              const double* pos, cd wgt,
                                              float* re, float* im,
                                              float* sre, float* sim) {
  if constexpr (COMP) {
    StencilFF<ORDER> sx, sy, sz, hx, hy, hz;
    if (!(axis_stencil_ff<ORDER>(pos[0], a.n[0], a.ratio[0], sx,
                                 SH ? &hx : nullptr) &&
          axis_stencil_ff<ORDER>(pos[1], a.n[1], a.ratio[1], sy,
                                 SH ? &hy : nullptr) &&
          axis_stencil_ff<ORDER>(pos[2], a.n[2], a.ratio[2], sz,
                                 SH ? &hz : nullptr)))
      return false;
    const bool unit_re = wgt.re == 1.;
    const FF wr = ff_from_double(wgt.re), wi = ff_from_double(wgt.im);
    deposit_ff<ORDER>(a, sx, sy, sz, wr, unit_re, re);
    if (im != nullptr) deposit_ff<ORDER>(a, sx, sy, sz, wi, false, im);
    if constexpr (SH) {
      deposit_ff<ORDER>(a, hx, hy, hz, wr, unit_re, sre);
      if (sim != nullptr) deposit_ff<ORDER>(a, hx, hy, hz, wi, false, sim);
    }
  } else {
    StencilF<ORDER> sx, sy, sz, hx, hy, hz;
    if (!(axis_stencil_f<ORDER>(pos[0], a.n[0], a.ratio[0], sx,
                                SH ? &hx : nullptr) &&
          axis_stencil_f<ORDER>(pos[1], a.n[1], a.ratio[1], sy,
                                SH ? &hy : nullptr) &&
          axis_stencil_f<ORDER>(pos[2], a.n[2], a.ratio[2], sz,
                                SH ? &hz : nullptr)))
      return false;
    deposit_f<ORDER>(a, sx, sy, sz, float(wgt.re), re);
    if (im != nullptr) deposit_f<ORDER>(a, sx, sy, sz, float(wgt.im), im);
    if constexpr (SH) {
      deposit_f<ORDER>(a, hx, hy, hz, float(wgt.re), sre);
      if (sim != nullptr)
        deposit_f<ORDER>(a, hx, hy, hz, float(wgt.im), sim);
    }
  }
  return true;
}

// SH: the interlacing shadow is deposited too (sre != nullptr).  COMP: FP32
// meshes with compensation meshes (a.lo_off).
// Blocks per SM by the registers each form needs without spills: TSC and
// PCS at two (at three, 85 registers, the TSC kernel spilled 104 bytes and
// measured 6 % slower), their compensated forms at one (at two they
// spilled 0.3-2 KB: 7 % slower for the survey's PCS deposit), NGP and CIC
// at three (two when compensated).
template <int ORDER, class Real, bool SH, bool COMP>
__global__ void __launch_bounds__(256, ORDER >= 3 ? (COMP ? 1 : 2)
                                                  : (COMP ? 2 : 3))
assign_kernel(AssignArgs a, Real* re, Real* im, Real* sre, Real* sim,
              double* sums) {
  cd acc = {0., 0.}, acc_s = {0., 0.};
  // Equal weights: fully landed particles are counted, not summed in FP64.
  const bool uniform = a.cat.w == nullptr && !a.ws.use_ylm;
  long long nland = 0;
  const int64_t np = a.cat.count(), p0 = a.cat.first();
  for (int64_t p = p0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       p < p0 + np; p += int64_t(gridDim.x) * blockDim.x) {
    const double pos[3] = {a.cat.x[p], a.cat.y[p], a.cat.z[p]};
    double w = (a.cat.w != nullptr) ? a.cat.w[p] : 1.0;
    double wp = w;
    for (int i = 1; i < a.ws.power; ++i) wp *= w;
    cd wgt = {a.ws.scale * wp, 0.};
    if (a.ws.use_ylm) {
      cd y = reduced_ylm(a.ws.ell, a.ws.m, a.cat.lx[p], a.cat.ly[p],
                         a.cat.lz[p]);
      if (a.ws.conj_ylm) y = conjg(y);
      wgt = (a.ws.scale * wp) * y;
    }
    if constexpr (sizeof(Real) == 4) {
      if (fast_particle<ORDER, SH, COMP>(a, pos, wgt, re, im, sre, sim)) {
        // Every cell is inside the mesh and the windows sum to one: the
        // landed weight is the weight itself.
        if (uniform) {
          ++nland;
        } else {
          acc = acc + wgt;
          if constexpr (SH) acc_s = acc_s + wgt;
        }
        continue;
      }
      cd landed[2] = {{0., 0.}, {0., 0.}};
      exact_particle<ORDER, Real>(a, pos, wgt, re, im, sre, sim, landed);
      acc = acc + landed[0];
      acc_s = acc_s + landed[1];
    } else {
      cd l = deposit<ORDER, Real>(a, pos, false, wgt, re, im);
      acc = acc + l;
      if constexpr (SH) {
        cd ls = deposit<ORDER, Real>(a, pos, true, wgt, sre, sim);
        acc_s = acc_s + ls;
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (uniform) {
    // Landed count: integer block sum, one FP64 product per block (the FP64
    // warp sums below would cost more than the particles themselves when a
    // thread handles few particles).
    __shared__ long long cnt[8];
    for (int o = 16; o > 0; o >>= 1)
      nland += __shfl_down_sync(0xffffffffu, nland, o);
    if (lane == 0) cnt[wid] = nland;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long t = 0;
      for (int q = 0; q < int(blockDim.x >> 5); ++q) t += cnt[q];
      const double land = double(t) * a.ws.scale;
      if (t != 0) {
        atomicAdd(sums + 0, land);
        if constexpr (SH) atomicAdd(sums + 2, land);
      }
    }
    // Particles of the exact path landed their weights in acc / acc_s.
    if (__syncthreads_or(acc.re != 0. || acc_s.re != 0.) == 0) return;
  }
  // Block-wide FP64 sums of the deposited weight (k = 0 modes).
  __shared__ double red[4][8];
  double v[4] = {warp_sum(acc.re), warp_sum(acc.im), warp_sum(acc_s.re),
                 warp_sum(acc_s.im)};
  if (lane == 0)
    for (int q = 0; q < 4; ++q) red[q][wid] = v[q];
  __syncthreads();
  if (threadIdx.x < 4) {
    double s = 0.;
    for (int q = 0; q < int(blockDim.x >> 5); ++q) s += red[threadIdx.x][q];
    atomicAdd(sums + threadIdx.x, s);
  }
}

// ---- Tiled FP32 deposit ------------------------------------------------------
//
// For a catalogue sorted by 32^3-cell mesh tiles, one block owns one tile at
// a time and deposits the tile's particles into a shared-memory window of
// the tile plus the cells its stencils reach (one below, two above per
// axis: (32 + 3)^3 floats), with shared-memory atomics.  The window then
// goes to the mesh once: cells that no other tile's particles reach (tile
// offsets 2 .. extent - 2 on every axis) are stored, the others take one
// global atomic per nonzero cell.  Particles off the fast FP32 stencil
// (near a tie, or outside the box) are appended to a list with
// warp-aggregated atomics and deposited exactly by assign_deferred_kernel.

constexpr int kTileShift = 5;
constexpr int kTile = 1 << kTileShift;
constexpr int kHaloLo = 1, kHaloHi = 2;
constexpr int kWin = kTile + kHaloLo + kHaloHi;  // x and y extent
// z: the window starts 4 cells below the tile so that its rows are
// 16-byte aligned in the mesh (float4 flush); 40 = 4 + 32 + 2, rounded up.
constexpr int kZLo = 4;
constexpr int kWinZ = 40;
constexpr int kGroupsZ = kWinZ / 4;
constexpr int kWinCells = kWin * kWin * kWinZ;
constexpr int kTiledBlock = 1024;

struct TiledArgs {
  AssignArgs a;
  int tiles[3];
  int* deferred;   // particle positions (from the first) taking the exact path
  int* ndeferred;
  const double* fill_dsum;  // the mesh holds the fill value (first deposit)
  double fill_hsum;
  bool store_exclusive;
};

// Window coordinate of cell `c` for a tile starting at `lo` (periodic):
// `below` cells of the window lie under the tile, `extent` in all.
template <int below, int extent>
__device__ __forceinline__ int win_coord(int c, int lo, int n) {
  int l = c - lo + below;
  if (l < 0) l += n;
  else if (l >= extent) l -= n;
  return l;
}

template <int ORDER>
__global__ void __launch_bounds__(kTiledBlock, 1)
assign_tiled_kernel(TiledArgs t, float* mesh, double* sums) {
  extern __shared__ __align__(16) float win[];
  const AssignArgs& a = t.a;
  const int ntiles = t.tiles[0] * t.tiles[1] * t.tiles[2];
  const int64_t np = a.cat.count(), p0 = a.cat.first();
  const bool uniform = a.cat.w == nullptr;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  float fill = 0.f;
  if (t.store_exclusive)
    fill = float(-((t.fill_dsum != nullptr) ? *t.fill_dsum : t.fill_hsum) /
                 double(a.nmesh));
  long long nland = 0;
  double acc = 0.;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int b = a.cat.tile_start[tile];
    const int e = (tile + 1 < ntiles) ? a.cat.tile_start[tile + 1] : int(np);
    if (b >= e) continue;
    const int tz = tile % t.tiles[2];
    const int ty = (tile / t.tiles[2]) % t.tiles[1];
    const int tx = tile / (t.tiles[2] * t.tiles[1]);
    const int lo[3] = {tx << kTileShift, ty << kTileShift, tz << kTileShift};
    int ext[3], wn[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      ext[i] = min(kTile, a.n[i] - lo[i]);
      wn[i] = ext[i] + kHaloLo + kHaloHi;
    }
    for (int i = threadIdx.x; i < kWinCells / 4; i += blockDim.x)
      reinterpret_cast<float4*>(win)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = (kWinCells / 4) * 4 + threadIdx.x; i < kWinCells;
         i += blockDim.x)
      win[i] = 0.f;
    __syncthreads();
    for (int base = b; base < e; base += blockDim.x) {
      const int q = base + threadIdx.x;
      const bool valid = q < e;
      bool fast = false;
      StencilF<ORDER> sx, sy, sz;
      float wgt = 0.f;
      if (valid) {
        const int64_t p = p0 + q;
        double wd = a.ws.scale;
        if (!uniform) {
          const double w = a.cat.w[p];
          double wp = w;
          for (int i = 1; i < a.ws.power; ++i) wp *= w;
          wd *= wp;
        }
        wgt = float(wd);
        fast = axis_stencil_f<ORDER>(a.cat.x[p], a.n[0], a.ratio[0], sx,
                                     nullptr) &&
               axis_stencil_f<ORDER>(a.cat.y[p], a.n[1], a.ratio[1], sy,
                                     nullptr) &&
               axis_stencil_f<ORDER>(a.cat.z[p], a.n[2], a.ratio[2], sz,
                                     nullptr);
        if (fast) {
          if (uniform) ++nland;
          else acc += wd;
        }
      }
      // Warp-aggregated append of the particles that take the exact path.
      const unsigned slow = __ballot_sync(0xffffffffu, valid && !fast);
      if (slow != 0u) {
        const int leader = __ffs(slow) - 1;
        int at = 0;
        if (lane == leader) at = atomicAdd(t.ndeferred, __popc(slow));
        at = __shfl_sync(0xffffffffu, at, leader);
        if (valid && !fast)
          t.deferred[at + __popc(slow & ((1u << lane) - 1u))] = q;
      }
      if (!fast) continue;
      int lx[ORDER], ly[ORDER], lz[ORDER];
#pragma unroll
      for (int k = 0; k < ORDER; ++k) {
        lx[k] = win_coord<kHaloLo, kWin>(sx.idx[k], lo[0], a.n[0]);
        ly[k] = win_coord<kHaloLo, kWin>(sy.idx[k], lo[1], a.n[1]);
        lz[k] = win_coord<kZLo, kWinZ>(sz.idx[k], lo[2], a.n[2]);
      }
#pragma unroll
      for (int i = 0; i < ORDER; ++i) {
        const float wi = sx.win[i] * wgt;
#pragma unroll
        for (int j = 0; j < ORDER; ++j) {
          const float wij = wi * sy.win[j];
          float* row = win + (lx[i] * kWin + ly[j]) * kWinZ;
#pragma unroll
          for (int k = 0; k < ORDER; ++k) atomicAdd(row + lz[k], wij * sz.win[k]);
        }
      }
    }
    __syncthreads();
    // Flush in float4 groups along z: groups whose four cells only this
    // tile reaches are stored over the fill value, the other nonzero
    // groups take one vector atomic.
    const int rows = wn[0] * wn[1];
    const int zlo = lo[2] - kZLo;
    for (int i = threadIdx.x; i < rows * kGroupsZ; i += blockDim.x) {
      const int r = i / kGroupsZ, q = i - r * kGroupsZ;
      const int wx = r / wn[1], wy = r - wx * wn[1];
      const float4 v =
          reinterpret_cast<const float4*>(win + (wx * kWin + wy) * kWinZ)[q];
      if (v.x == 0.f && v.y == 0.f && v.z == 0.f && v.w == 0.f) continue;
      int gx = lo[0] - kHaloLo + wx, gy = lo[1] - kHaloLo + wy;
      gx += (gx < 0) ? a.n[0] : ((gx >= a.n[0]) ? -a.n[0] : 0);
      gy += (gy < 0) ? a.n[1] : ((gy >= a.n[1]) ? -a.n[1] : 0);
      int gz = zlo + 4 * q;
      gz += (gz < 0) ? a.n[2] : ((gz >= a.n[2]) ? -a.n[2] : 0);
      float4* g = reinterpret_cast<float4*>(
          mesh + (int64_t(gx) * a.n[1] + gy) * a.n[2] + gz);
      // Tile offsets of the group's cells: 4q - kZLo .. 4q - kZLo + 3.
      const int c0 = 4 * q - kZLo;
      const bool excl = t.store_exclusive && wx >= kHaloLo + 2 &&
                        wx < kHaloLo + ext[0] - 1 && wy >= kHaloLo + 2 &&
                        wy < kHaloLo + ext[1] - 1 && c0 >= 2 &&
                        c0 + 3 < ext[2] - 1;
      if (excl)
        *g = make_float4(fill + v.x, fill + v.y, fill + v.z, fill + v.w);
      else
        atomicAdd(g, v);
    }
    __syncthreads();
  }
  // Landed weight of the fast-path particles (the k = 0 mode).
  __shared__ long long cnt[kTiledBlock / 32];
  __shared__ double red[kTiledBlock / 32];
  for (int o = 16; o > 0; o >>= 1) {
    nland += __shfl_down_sync(0xffffffffu, nland, o);
    acc += __shfl_down_sync(0xffffffffu, acc, o);
  }
  if (lane == 0) {
    cnt[wid] = nland;
    red[wid] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long c = 0;
    double s = 0.;
    for (int q = 0; q < nwarps; ++q) {
      c += cnt[q];
      s += red[q];
    }
    const double land = uniform ? double(c) * a.ws.scale : s;
    if (land != 0.) atomicAdd(sums, land);
  }
}

// The particles the tiled deposit left to the exact FP64 stencil.
template <int ORDER>
__global__ void __launch_bounds__(256)
assign_deferred_kernel(AssignArgs a, const int* deferred,
                       const int* ndeferred, float* mesh, double* sums) {
  const int nd = *ndeferred;
  const int64_t p0 = a.cat.first();
  double acc = 0.;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd;
       i += gridDim.x * blockDim.x) {
    const int64_t p = p0 + deferred[i];
    const double pos[3] = {a.cat.x[p], a.cat.y[p], a.cat.z[p]};
    double w = (a.cat.w != nullptr) ? a.cat.w[p] : 1.0;
    double wp = w;
    for (int k = 1; k < a.ws.power; ++k) wp *= w;
    cd landed[2] = {{0., 0.}, {0., 0.}};
    exact_particle<ORDER, float>(a, pos, cd{a.ws.scale * wp, 0.}, mesh,
                                 nullptr, nullptr, nullptr, landed);
    acc += landed[0].re;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0 && acc != 0.) atomicAdd(sums, acc);
}

// ---- Y_lm-weighted fields of every order in one pass -----------------------
//
// Per particle: the weight powers, the reduced harmonics of every order
// (FP64 Legendre recurrences, reduced_ylm_all) and the FP32 stencil are
// formed once; each target then deposits its complex weight.

__device__ __forceinline__ cd target_weight(const YlmTarget& t,
                                            const double* wpow,
                                            const cd* ypos, int ell) {
  const cd y = (ell == 0) ? cd{1., 0.} : ylm_of(ypos, t.m);
  const cd v = t.conj ? conjg(y) : y;
  if (ell == 0) return cd{t.scale * wpow[t.power], 0.};
  return (t.scale * wpow[t.power]) * v;
}

__device__ __forceinline__ void particle_terms(const DevCatalogue& cat,
                                               int64_t p, int ell,
                                               const double* cnorm,
                                               double* wpow, cd* ypos) {
  const double w = (cat.w != nullptr) ? cat.w[p] : 1.0;
  wpow[0] = 1.;
  wpow[1] = w;
  wpow[2] = w * w;
  wpow[3] = wpow[2] * w;
  if (ell > 0)
    reduced_ylm_all(ell, cnorm, cat.lx[p], cat.ly[p], cat.lz[p], ypos);
}

__global__ void __launch_bounds__(256)
ylm_weight_sums_kernel(DevCatalogue cat, YlmTargets ts, double* out) {
  cd acc[kMaxYlmTargets];
#pragma unroll
  for (int t = 0; t < kMaxYlmTargets; ++t) acc[t] = cd{0., 0.};
  const int64_t np = cat.count(), p0 = cat.first();
  for (int64_t p = p0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       p < p0 + np; p += int64_t(gridDim.x) * blockDim.x) {
    double wpow[4];
    cd ypos[kMaxYlmDegree + 1];
    particle_terms(cat, p, ts.ell, ts.cnorm, wpow, ypos);
#pragma unroll
    for (int t = 0; t < kMaxYlmTargets; ++t) {
      if (t >= ts.count) break;
      // scale applied after the sum, as in weight_sum_kernel
      YlmTarget u = ts.t[t];
      u.scale = 1.;
      acc[t] = acc[t] + target_weight(u, wpow, ypos, ts.ell);
    }
  }
  __shared__ double red[2][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int t = 0; t < ts.count; ++t) {
    const double v0 = warp_sum(acc[t].re), v1 = warp_sum(acc[t].im);
    if (lane == 0) {
      red[0][wid] = v0;
      red[1][wid] = v1;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
      double s = 0.;
      for (int q = 0; q < int(blockDim.x >> 5); ++q) s += red[threadIdx.x][q];
      atomicAdd(out + 2 * t + threadIdx.x, ts.t[t].scale * s);
    }
    __syncthreads();
  }
}

// Compensated TSC / PCS forms at one block per SM: at two they spilled
// 64-2080 bytes (3 % slower for the survey's B_202 deposit).
template <int ORDER, bool SH, bool COMP>
__global__ void __launch_bounds__(256, (COMP && ORDER <= 2) ? 2 : 1)
assign_ylm_kernel(AssignArgs a, YlmTargets ts) {
  const int64_t np = a.cat.count(), p0 = a.cat.first();
  for (int64_t p = p0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       p < p0 + np; p += int64_t(gridDim.x) * blockDim.x) {
    double wpow[4];
    cd ypos[kMaxYlmDegree + 1];
    particle_terms(a.cat, p, ts.ell, ts.cnorm, wpow, ypos);
    const double pos[3] = {a.cat.x[p], a.cat.y[p], a.cat.z[p]};
    using St = typename std::conditional<COMP, StencilFF<ORDER>,
                                         StencilF<ORDER>>::type;
    St sx, sy, sz, hx, hy, hz;
    bool fast;
    if constexpr (COMP)
      fast = axis_stencil_ff<ORDER>(pos[0], a.n[0], a.ratio[0], sx,
                                    SH ? &hx : nullptr) &&
             axis_stencil_ff<ORDER>(pos[1], a.n[1], a.ratio[1], sy,
                                    SH ? &hy : nullptr) &&
             axis_stencil_ff<ORDER>(pos[2], a.n[2], a.ratio[2], sz,
                                    SH ? &hz : nullptr);
    else
      fast = axis_stencil_f<ORDER>(pos[0], a.n[0], a.ratio[0], sx,
                                   SH ? &hx : nullptr) &&
             axis_stencil_f<ORDER>(pos[1], a.n[1], a.ratio[1], sy,
                                   SH ? &hy : nullptr) &&
             axis_stencil_f<ORDER>(pos[2], a.n[2], a.ratio[2], sz,
                                   SH ? &hz : nullptr);
    for (int t = 0; t < ts.count; ++t) {
      const YlmTarget& u = ts.t[t];
      if (u.re == nullptr) continue;
      const cd wgt = target_weight(u, wpow, ypos, ts.ell);
      if constexpr (COMP) {
        // Targets whose sums do not cancel: plain FP32 atomics with the
        // float-float windows rounded once.
        if (fast && !u.comp) {
          deposit_f<ORDER>(a, sx, sy, sz, float(wgt.re), u.re);
          if (u.im != nullptr)
            deposit_f<ORDER>(a, sx, sy, sz, float(wgt.im), u.im);
          if constexpr (SH) {
            deposit_f<ORDER>(a, hx, hy, hz, float(wgt.re), u.sre);
            if (u.sim != nullptr)
              deposit_f<ORDER>(a, hx, hy, hz, float(wgt.im), u.sim);
          }
          continue;
        }
      }
      if (fast) {
        if constexpr (COMP) {
          const FF wr = ff_from_double(wgt.re), wi = ff_from_double(wgt.im);
          deposit_ff<ORDER>(a, sx, sy, sz, wr, false, u.re);
          if (u.im != nullptr)
            deposit_ff<ORDER>(a, sx, sy, sz, wi, false, u.im);
          if constexpr (SH) {
            deposit_ff<ORDER>(a, hx, hy, hz, wr, false, u.sre);
            if (u.sim != nullptr)
              deposit_ff<ORDER>(a, hx, hy, hz, wi, false, u.sim);
          }
        } else {
          deposit_f<ORDER>(a, sx, sy, sz, float(wgt.re), u.re);
          if (u.im != nullptr)
            deposit_f<ORDER>(a, sx, sy, sz, float(wgt.im), u.im);
          if constexpr (SH) {
            deposit_f<ORDER>(a, hx, hy, hz, float(wgt.re), u.sre);
            if (u.sim != nullptr)
              deposit_f<ORDER>(a, hx, hy, hz, float(wgt.im), u.sim);
          }
        }
      } else {
        // The target's sums hold the full weight: add what did not land.
        cd landed[2] = {{0., 0.}, {0., 0.}};
        exact_particle<ORDER, float>(a, pos, wgt, u.re, u.im,
                                     SH ? u.sre : nullptr,
                                     SH ? u.sim : nullptr, landed);
        const cd d0 = landed[0] - wgt;
        if (d0.re != 0.) atomicAdd(u.sums + 0, d0.re);
        if (d0.im != 0.) atomicAdd(u.sums + 1, d0.im);
        if constexpr (SH) {
          const cd d1 = landed[1] - wgt;
          if (d1.re != 0.) atomicAdd(u.sums + 2, d1.re);
          if (d1.im != 0.) atomicAdd(u.sums + 3, d1.im);
        }
      }
    }
  }
}

template <class Real>
__global__ void sum_pow_kernel(const Real* mesh, int64_t n, int order,
                               double* out) {
  double acc = 0.;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const double v = double(mesh[i]);
    double p = 1.;
    for (int q = 0; q < order; ++q) p *= v;
    acc += p;
  }
  __shared__ double red[32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.;
    for (int q = 0; q < int(blockDim.x >> 5); ++q) s += red[q];
    atomicAdd(out, s);
  }
}

template <class Real>
__global__ void to_double_kernel(const Real* mesh, int64_t n, double scale,
                                 double* out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = double(mesh[i]) * scale;
}

// Every cell set to -(sum / n): the mesh starts at minus the mean of the
// deposit to come.  `sum` is read from device memory when `dsum` is given.
template <class Real>
__global__ void fill_offset_kernel(Real* mesh, int64_t n, const double* dsum,
                                   double hsum, int64_t lo_off) {
  const double f = -((dsum != nullptr) ? *dsum : hsum) / double(n);
  const Real v = Real(f);
  // A compensation mesh starts at the rounding error of the fill value.
  const Real vl = Real(f - double(v));
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    mesh[i] = v;
    if (lo_off != 0) mesh[i + lo_off] = vl;
  }
}

template <class Real>
__global__ void mesh_copy_kernel(const float* src, int64_t n, Real* dst) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = Real(src[i]);
}

// hi + lo -> (fl(hi + lo), exact remainder): the FP32 mesh becomes the
// correctly rounded value of the compensated sum.
__global__ void mesh_renorm_kernel(float* mesh, int64_t n, int64_t lo_off) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const float h = mesh[i], l = mesh[i + lo_off];
    const float s = __fadd_rn(h, l);
    mesh[i] = s;
    mesh[i + lo_off] = two_sum_err(h, l, s);
  }
}

// sum_p scale * w_p^power * [conj] y_lm(los_p) in FP64
// (calc_ylm_wgtd_shotnoise_amp_for_bispec, threept.cpp:156-208, and its
// power-spectrum twin, twopt.cpp:298-350).
__global__ void weight_sum_kernel(DevCatalogue cat, WeightSpec ws,
                                  double* out) {
  cd acc = {0., 0.};
  const int64_t np = cat.count(), p0 = cat.first();
  for (int64_t p = p0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       p < p0 + np; p += int64_t(gridDim.x) * blockDim.x) {
    const double w = (cat.w != nullptr) ? cat.w[p] : 1.0;
    double wp = 1.;
    for (int i = 0; i < ws.power; ++i) wp *= w;
    cd y = {1., 0.};
    if (ws.use_ylm) {
      y = reduced_ylm(ws.ell, ws.m, cat.lx[p], cat.ly[p], cat.lz[p]);
      if (ws.conj_ylm) y = conjg(y);
    }
    acc = acc + wp * y;
  }
  __shared__ double red[2][8];
  const double v0 = warp_sum(acc.re), v1 = warp_sum(acc.im);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = v0;
    red[1][wid] = v1;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0.;
    for (int q = 0; q < int(blockDim.x >> 5); ++q) s += red[threadIdx.x][q];
    atomicAdd(out + threadIdx.x, ws.scale * s);
  }
}

int grid_for(int64_t work, int block) {
  int64_t g = (work + block - 1) / block;
  const int64_t cap = 152 * 16;  // a few waves of resident blocks
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return int(g);
}

}  // namespace

// Tiled deposit of a real FP32 mesh without interlacing, for a catalogue
// sorted by 32^3 tiles on a mesh of at least 64 cells per axis (the window
// of one tile then never wraps onto itself).
template <int ORDER>
void launch_tiled(Context& ctx, const AssignArgs& a, float* mesh,
                  double* sums, const MeshFill* fill) {
  TiledArgs t;
  t.a = a;
  for (int i = 0; i < 3; ++i) t.tiles[i] = (a.n[i] + kTile - 1) >> kTileShift;
  t.deferred = ctx.buf<int>("assign.deferred", size_t(a.cat.n));
  t.ndeferred = ctx.buf<int>("assign.ndeferred", 1);
  t.fill_dsum = fill ? fill->dsum : nullptr;
  t.fill_hsum = fill ? fill->hsum : 0.;
  t.store_exclusive = fill != nullptr;
  TRVG_CUDA(cudaMemsetAsync(t.ndeferred, 0, sizeof(int), ctx.stream));
  const size_t smem = size_t(kWinCells) * sizeof(float);
  static bool configured[64] = {};
  if (ctx.device < 0 || ctx.device >= 64 || !configured[ctx.device]) {
    TRVG_CUDA(cudaFuncSetAttribute(assign_tiled_kernel<ORDER>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   int(smem)));
    if (ctx.device >= 0 && ctx.device < 64) configured[ctx.device] = true;
  }
  const int ntiles = t.tiles[0] * t.tiles[1] * t.tiles[2];
  TRVG_KBEGIN(ctx, "assign_tiled_kernel");
  assign_tiled_kernel<ORDER><<<std::min(ntiles, 152), kTiledBlock, smem,
                               ctx.stream>>>(t, mesh, sums);
  TRVG_LAUNCHED(ctx);
  TRVG_KBEGIN(ctx, "assign_deferred_kernel");
  assign_deferred_kernel<ORDER><<<152, 256, 0, ctx.stream>>>(
      a, t.deferred, t.ndeferred, mesh, sums);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_assign(Context& ctx, const Geom& g, int order, bool interlace,
                   const DevCatalogue& cat, const WeightSpec& ws,
                   Real* mesh_re, Real* mesh_im, Real* shadow_re,
                   Real* shadow_im, double* sums, const MeshFill* fill,
                   int64_t lo_off) {
  if (cat.n == 0) return;
  if (sizeof(Real) != 4) lo_off = 0;
  AssignArgs a;
  a.lo_off = lo_off;
  for (int i = 0; i < 3; ++i) {
    a.n[i] = g.n[i];
    a.L[i] = g.L[i];
    a.ratio[i] = double(g.n[i]) / g.L[i];
  }
  a.nmesh = g.nmesh;
  a.cat = cat;
  a.ws = ws;
  Real* sre = interlace ? shadow_re : nullptr;
  Real* sim = interlace ? shadow_im : nullptr;
  auto aligned16 = [](const Real* p) {
    return p == nullptr || reinterpret_cast<uintptr_t>(p) % 16 == 0;
  };
  a.vec4 = g.n[2] % 4 == 0 && aligned16(mesh_re) && aligned16(mesh_im) &&
           aligned16(sre) && aligned16(sim);
  if constexpr (sizeof(Real) == 4) {
    const bool tiled = lo_off == 0 && cat.tile_start != nullptr &&
                       cat.tile_shift == kTileShift && !interlace &&
                       mesh_im == nullptr && !ws.use_ylm && a.vec4 &&
                       g.n[0] >= 64 &&
                       g.n[1] >= 64 && g.n[2] >= 64 &&
                       cat.n <= int64_t(2147483647);
    if (tiled) {
      switch (order) {
        case 1: return launch_tiled<1>(ctx, a, mesh_re, sums, fill);
        case 2: return launch_tiled<2>(ctx, a, mesh_re, sums, fill);
        case 3: return launch_tiled<3>(ctx, a, mesh_re, sums, fill);
        case 4: return launch_tiled<4>(ctx, a, mesh_re, sums, fill);
        default: break;
      }
    }
  }
  const int block = 256;
  // Several particles per thread: the per-block k = 0 sums are amortised.
  const int grid = std::min(grid_for(cat.n, block), 152 * 8);
  auto go = [&](auto kernel) {
    TRVG_KBEGIN(ctx, "assign_kernel");
    kernel<<<grid, block, 0, ctx.stream>>>(a, mesh_re, mesh_im, sre, sim,
                                           sums);
  };
  const bool sh = sre != nullptr;
  auto by_order = [&](auto sh_c, auto comp_c) {
    constexpr bool S = decltype(sh_c)::value, P = decltype(comp_c)::value;
    switch (order) {
      case 1: go(assign_kernel<1, Real, S, P>); break;
      case 2: go(assign_kernel<2, Real, S, P>); break;
      case 3: go(assign_kernel<3, Real, S, P>); break;
      case 4: go(assign_kernel<4, Real, S, P>); break;
      default:
        throw_error(TRVG_ERR_INVALID_PARAMETER,
                    "Unsupported mesh assignment order: %d.", order);
    }
  };
  using T = std::true_type;
  using F = std::false_type;
  if (sizeof(Real) == 4 && lo_off != 0) {
    sh ? by_order(T(), T()) : by_order(F(), T());
  } else {
    sh ? by_order(T(), F()) : by_order(F(), F());
  }
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_mesh_sum_pow(Context& ctx, const Real* mesh, int64_t n, int order,
                         double* out) {
  TRVG_KBEGIN(ctx, "sum_pow_kernel");
  sum_pow_kernel<Real><<<grid_for(n, 256), 256, 0, ctx.stream>>>(mesh, n,
                                                                 order, out);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_mesh_to_double(Context& ctx, const Real* mesh, int64_t n,
                           double scale, double* out) {
  TRVG_KBEGIN(ctx, "to_double_kernel");
  to_double_kernel<Real><<<grid_for(n, 256), 256, 0, ctx.stream>>>(
      mesh, n, scale, out);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_fill_offset(Context& ctx, Real* mesh, int64_t n,
                        const double* dsum, double hsum, int64_t lo_off) {
  TRVG_KBEGIN(ctx, "fill_offset_kernel");
  fill_offset_kernel<Real><<<grid_for(n, 256), 256, 0, ctx.stream>>>(
      mesh, n, dsum, hsum, lo_off);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_mesh_copy(Context& ctx, const float* src, int64_t n, Real* dst) {
  TRVG_KBEGIN(ctx, "mesh_copy_kernel");
  mesh_copy_kernel<Real><<<grid_for(n, 256), 256, 0, ctx.stream>>>(src, n,
                                                                   dst);
  TRVG_LAUNCHED(ctx);
}

void launch_mesh_renorm(Context& ctx, float* mesh, int64_t n,
                        int64_t lo_off) {
  if (mesh == nullptr || lo_off == 0) return;
  TRVG_KBEGIN(ctx, "mesh_renorm_kernel");
  mesh_renorm_kernel<<<grid_for(n, 256), 256, 0, ctx.stream>>>(mesh, n,
                                                               lo_off);
  TRVG_LAUNCHED(ctx);
}

void launch_ylm_weight_sums(Context& ctx, const DevCatalogue& cat,
                            const YlmTargets& ts, double* out) {
  if (cat.n == 0 || ts.count == 0) return;
  if (ts.count > kMaxYlmTargets || ts.ell > kMaxYlmDegree || ts.ell < 0)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Too many Y_lm targets.");
  YlmTargets tn = ts;
  ylm_all_norms(tn.ell, tn.cnorm);
  TRVG_KBEGIN(ctx, "weight_sum_kernel");
  ylm_weight_sums_kernel<<<grid_for(cat.n, 256), 256, 0, ctx.stream>>>(
      cat, tn, out);
  TRVG_LAUNCHED(ctx);
}

void launch_assign_ylm(Context& ctx, const Geom& g, int order, bool interlace,
                       const DevCatalogue& cat, const YlmTargets& ts,
                       int64_t lo_off) {
  if (cat.n == 0 || ts.count == 0) return;
  if (ts.count > kMaxYlmTargets || ts.ell > kMaxYlmDegree || ts.ell < 0)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Too many Y_lm targets.");
  AssignArgs a;
  for (int i = 0; i < 3; ++i) {
    a.n[i] = g.n[i];
    a.L[i] = g.L[i];
    a.ratio[i] = double(g.n[i]) / g.L[i];
  }
  a.nmesh = g.nmesh;
  a.cat = cat;
  a.ws = WeightSpec();
  a.lo_off = lo_off;
  a.vec4 = g.n[2] % 4 == 0;
  for (int t = 0; t < ts.count; ++t)
    for (const float* q : {ts.t[t].re, ts.t[t].im, ts.t[t].sre, ts.t[t].sim})
      if (q != nullptr && reinterpret_cast<uintptr_t>(q) % 16 != 0)
        a.vec4 = false;
  YlmTargets tn = ts;
  ylm_all_norms(tn.ell, tn.cnorm);
  const int grid = std::min(grid_for(cat.n, 256), 152 * 8);
  auto go = [&](auto kernel) {
    TRVG_KBEGIN(ctx, "assign_kernel");
    kernel<<<grid, 256, 0, ctx.stream>>>(a, tn);
    TRVG_LAUNCHED(ctx);
  };
  auto by_order = [&](auto sh_c, auto comp_c) {
    constexpr bool S = decltype(sh_c)::value, P = decltype(comp_c)::value;
    switch (order) {
      case 1: go(assign_ylm_kernel<1, S, P>); break;
      case 2: go(assign_ylm_kernel<2, S, P>); break;
      case 3: go(assign_ylm_kernel<3, S, P>); break;
      case 4: go(assign_ylm_kernel<4, S, P>); break;
      default:
        throw_error(TRVG_ERR_INVALID_PARAMETER,
                    "Unsupported mesh assignment order: %d.", order);
    }
  };
  using T = std::true_type;
  using F = std::false_type;
  if (lo_off != 0) {
    interlace ? by_order(T(), T()) : by_order(F(), T());
  } else {
    interlace ? by_order(T(), F()) : by_order(F(), F());
  }
}

void launch_weight_sum(Context& ctx, const DevCatalogue& cat,
                       const WeightSpec& ws, double* out) {
  if (cat.n == 0) return;
  TRVG_KBEGIN(ctx, "weight_sum_kernel");
  weight_sum_kernel<<<grid_for(cat.n, 256), 256, 0, ctx.stream>>>(cat, ws,
                                                                  out);
  TRVG_LAUNCHED(ctx);
}

#define TRVG_INST(R)                                                        \
  template void launch_assign<R>(Context&, const Geom&, int, bool,          \
                                 const DevCatalogue&, const WeightSpec&, R*, \
                                 R*, R*, R*, double*, const MeshFill*,      \
                                 int64_t);                                  \
  template void launch_mesh_sum_pow<R>(Context&, const R*, int64_t, int,    \
                                       double*);                            \
  template void launch_mesh_to_double<R>(Context&, const R*, int64_t,       \
                                         double, double*);                  \
  template void launch_fill_offset<R>(Context&, R*, int64_t, const double*, \
                                      double, int64_t);                     \
  template void launch_mesh_copy<R>(Context&, const float*, int64_t, R*);
TRVG_INST(float)
TRVG_INST(double)
#undef TRVG_INST

}  // namespace trvg
