// Float-float ("double-single") arithmetic for the accurate transforms.
//
// A value is the unevaluated sum hi + lo of two floats, about 48
// significant bits, computed on the FP32 pipe only.  Sums use Knuth's
// TwoSum on the leading words, products the FMA form of Dekker's
// TwoProduct.  The results are left unnormalised (lo may exceed half an ulp
// of hi by a few ulps): the next operation splits the leading words exactly
// again, so skipping the renormalisation costs no accuracy, and ffnorm
// restores the canonical form where a value leaves the transforms.  Every
// operation goes through the _rn intrinsics, which the compiler never
// contracts into FMAs: a contracted product or sum would lose the exactly
// recovered rounding errors these formulas depend on.
#pragma once

#include "common.cuh"

namespace trvg {

__device__ __forceinline__ FF ffadd(FF a, FF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float v = __fsub_rn(s, a.hi);
  const float e =
      __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  return FF{s, __fadd_rn(e, __fadd_rn(a.lo, b.lo))};
}

// Canonical form (|lo| <= ulp(hi) / 2) by TwoSum of the two words.
__device__ __forceinline__ FF ffnorm(FF a) {
  const float s = __fadd_rn(a.hi, a.lo);
  const float v = __fsub_rn(s, a.hi);
  return FF{s, __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)),
                         __fsub_rn(a.lo, v))};
}

__device__ __forceinline__ FF ffneg(FF a) { return FF{-a.hi, -a.lo}; }

__device__ __forceinline__ FF ffsub(FF a, FF b) { return ffadd(a, ffneg(b)); }

__device__ __forceinline__ FF ffmul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return FF{p, e};
}

// Multiplication by a power of two (exact).
__device__ __forceinline__ FF ffscale2(FF a, float p2) {
  return FF{__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)};
}

__device__ __forceinline__ FF ff_from_double(double x) {
  const float h = float(x);
  return FF{h, float(x - double(h))};
}

// Complex float-float.
struct FFC {
  FF re, im;
};

__device__ __forceinline__ FFC ffc_add(FFC a, FFC b) {
  return FFC{ffadd(a.re, b.re), ffadd(a.im, b.im)};
}
__device__ __forceinline__ FFC ffc_sub(FFC a, FFC b) {
  return FFC{ffsub(a.re, b.re), ffsub(a.im, b.im)};
}
// a b + c d: both leading products and their sum are split exactly
// (TwoProduct, TwoSum); the cross terms go into the error word by FMA, and
// only lo * lo is dropped (about 2^-48 relative).
__device__ __forceinline__ FF ffdot2(FF a, FF b, FF c, FF d) {
  const float p1 = __fmul_rn(a.hi, b.hi);
  const float e1 = __fmaf_rn(a.hi, b.hi, -p1);
  const float p2 = __fmul_rn(c.hi, d.hi);
  const float e2 = __fmaf_rn(c.hi, d.hi, -p2);
  const float s = __fadd_rn(p1, p2);
  const float v = __fsub_rn(s, p1);
  const float es =
      __fadd_rn(__fsub_rn(p1, __fsub_rn(s, v)), __fsub_rn(p2, v));
  float e = __fadd_rn(__fadd_rn(e1, e2), es);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(c.hi, d.lo, e);
  e = __fmaf_rn(c.lo, d.hi, e);
  return FF{s, e};
}

__device__ __forceinline__ FFC ffc_mul(FFC a, FFC b) {
  return FFC{ffdot2(a.re, b.re, ffneg(a.im), b.im),
             ffdot2(a.re, b.im, a.im, b.re)};
}
// a * s for a real float-float s.
__device__ __forceinline__ FFC ffc_mulr(FFC a, FF s) {
  return FFC{ffmul(a.re, s), ffmul(a.im, s)};
}
// a * (d i), d = +-1 (exact).
__device__ __forceinline__ FFC ffc_muli(FFC a, int d) {
  return d > 0 ? FFC{ffneg(a.im), a.re} : FFC{a.im, ffneg(a.re)};
}
__device__ __forceinline__ FFC ffc_conj(FFC a) { return FFC{a.re, ffneg(a.im)}; }
__device__ __forceinline__ FFC ffc_scale2(FFC a, float p2) {
  return FFC{ffscale2(a.re, p2), ffscale2(a.im, p2)};
}
__device__ __forceinline__ FFC ffc_zero() {
  return FFC{FF{0.f, 0.f}, FF{0.f, 0.f}};
}

__device__ __forceinline__ FFC ffc_norm(FFC a) {
  return FFC{ffnorm(a.re), ffnorm(a.im)};
}

// Storage: float4 (re.hi, re.lo, im.hi, im.lo).
__device__ __forceinline__ FFC ffc_load(const float4* p) {
  const float4 v = *p;
  return FFC{FF{v.x, v.y}, FF{v.z, v.w}};
}
__device__ __forceinline__ void ffc_store(float4* p, FFC a) {
  *p = make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo);
}

}  // namespace trvg
