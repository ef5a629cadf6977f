// Exact assignment stencils (FP64), shared by the mesh assignment and the
// gradient gather of the adjoint.
#pragma once

#include "common.cuh"

namespace trvg {

template <int ORDER>
struct Stencil {
  int idx[ORDER];
  double win[ORDER];
};

// One axis of the assignment stencil.  `shadow` selects the half-cell-shifted
// pass (field.cpp:673-726 etc.), including the reference's own index
// arithmetic of the TSC shadow pass (field.cpp:940-945).
template <int ORDER>
__device__ __forceinline__ Stencil<ORDER> axis_stencil(double pos, int n,
                                                       double L, bool shadow) {
  Stencil<ORDER> st;
  double loc = ddiv(dmul(double(n), pos), L);
  if (shadow) {
    loc = dadd(loc, 0.5);
    if (loc > double(n)) loc = loc - double(n);
  }
  const int idx = int(loc);
  double s = loc - double(idx);
  if (ORDER == 1) {
    int i0 = idx;
    if (s >= 0.5) i0 = (idx == n - 1) ? 0 : idx + 1;
    st.idx[0] = i0;
    st.win[0] = 1.;
  } else if (ORDER == 2) {
    st.idx[0] = idx;
    st.idx[1] = (idx == n - 1) ? 0 : idx + 1;
    st.win[0] = 1. - s;
    st.win[1] = s;
  } else if (ORDER == 3) {
    if (s < 0.5) {
      st.idx[0] = (idx == 0) ? n - 1 : idx - 1;
      st.idx[1] = idx;
      st.idx[2] = (idx == n - 1) ? 0 : idx + 1;
      st.win[0] = 0.5 * (0.5 - s) * (0.5 - s);
      st.win[1] = 0.75 - s * s;
      st.win[2] = 0.5 * (0.5 + s) * (0.5 + s);
    } else {
      st.idx[0] = idx;
      st.idx[1] = (idx == n - 1) ? 0 : idx + 1;
      if (shadow) {
        st.idx[2] = (idx == n - 1) ? 0 : st.idx[1] + 1;
      } else {
        st.idx[2] = (st.idx[1] == n - 1) ? 0 : st.idx[1] + 1;
      }
      const double t = 1. - s;
      st.win[0] = 0.5 * (0.5 + t) * (0.5 + t);
      st.win[1] = 0.75 - t * t;
      st.win[2] = 0.5 * (0.5 - t) * (0.5 - t);
    }
  } else {
    st.idx[0] = (idx == 0) ? n - 1 : idx - 1;
    st.idx[1] = idx;
    st.idx[2] = (idx == n - 1) ? 0 : idx + 1;
    st.idx[3] = (st.idx[2] == n - 1) ? 0 : st.idx[2] + 1;
    const double t = 1. - s;
    st.win[0] = 1. / 6 * t * t * t;
    st.win[1] = 1. / 6 * (4. - 6. * s * s + 3. * s * s * s);
    st.win[2] = 1. / 6 * (4. - 6. * t * t + 3. * t * t * t);
    st.win[3] = 1. / 6 * s * s * s;
  }
  return st;
}

// Derivatives d win_i / d s of the windows of axis_stencil, s being the
// offset loc - idx of the same stencil (d loc / d x = n / L).
template <int ORDER>
__device__ __forceinline__ void axis_window_deriv(double pos, int n, double L,
                                                  double dwin[ORDER]) {
  const double loc = ddiv(dmul(double(n), pos), L);
  const int idx = int(loc);
  const double s = loc - double(idx);
  if (ORDER == 1) {
    dwin[0] = 0.;
  } else if (ORDER == 2) {
    dwin[0] = -1.;
    dwin[1] = 1.;
  } else if (ORDER == 3) {
    if (s < 0.5) {
      dwin[0] = -(0.5 - s);
      dwin[1] = -2. * s;
      dwin[2] = 0.5 + s;
    } else {
      const double t = 1. - s;  // d t / d s = -1
      dwin[0] = -(0.5 + t);
      dwin[1] = 2. * t;
      dwin[2] = 0.5 - t;
    }
  } else {
    const double t = 1. - s;
    dwin[0] = -0.5 * t * t;
    dwin[1] = 1. / 6 * (-12. * s + 9. * s * s);
    dwin[2] = -1. / 6 * (-12. * t + 9. * t * t);
    dwin[3] = 0.5 * s * s;
  }
}

}  // namespace trvg
