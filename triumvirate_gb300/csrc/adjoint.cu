// Adjoint of the raw periodic-box bispectrum on the evaluation grid.
//
// The raw estimate of pair p = (a, b) is
//   B_p = C_p sum_y F_a(y) F_b(y) G(y),
// with F_a = E (mask_a / W) D m and G = E (mask_G / (W V)) D m linear in
// the count mesh m (D: forward DFT of the mesh, E: inverse DFT onto the
// evaluation grid, masks: the shell of bin a and the cube of G).  For a
// cotangent lambda_p = dL/dB_p the mesh gradient is
//   dL/dm = sum_p lambda_p C_p [A_a^T (F_b G) + A_b^T (F_a G)
//                               + A_G^T (F_a F_b)],
// and for a real field v on the evaluation grid
//   A^T v (x) = sum_k mask(k) / W(k) FFT_M[v](k) e^{i k x}
// (unnormalised), i.e. a forward FFT on the evaluation grid, the masks and
// window, then one band-limited C2R onto the full mesh.  The gradients of
// the particle weights and positions gather dL/dm with the assignment
// window and its derivative.
#include "kernels.h"
#include "stencil.cuh"

namespace trvg {

namespace {

int grid_for(int64_t work, int block, int64_t cap = 152 * 16) {
  int64_t g = (work + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return int(g);
}

__device__ __forceinline__ int wrap(int s, int n) { return s < 0 ? s + n : s; }

// H_a = G * sum_{(partner, lambda) of a} lambda F_partner for every bin a,
// and Q = sum_p lambda_p F_row(p) F_col(p).
template <class FR>
__global__ void __launch_bounds__(256)
adjoint_fields_kernel(int64_t ncell, const FR* G, const FR* F, int nb,
                      AdjointLists l, FR* H, FR* Q) {
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < ncell;
       t += int64_t(gridDim.x) * blockDim.x) {
    const double gv = double(G[t]);
    for (int a = 0; a < nb; ++a) {
      double acc = 0.;
      for (int e = l.off[a]; e < l.off[a + 1]; ++e)
        acc += l.lam[e] * double(F[int64_t(l.partner[e]) * ncell + t]);
      H[int64_t(a) * ncell + t] = FR(acc * gv);
    }
    double q = 0.;
    for (int p = 0; p < l.npairs; ++p)
      q += l.plam[p] * double(F[int64_t(l.prow[p]) * ncell + t]) *
           double(F[int64_t(l.pcol[p]) * ncell + t]);
    Q[t] = FR(q);
  }
}

// The full-mesh half spectrum of the gradient, written at the modes of the
// evaluation cube (the rest of `U` is zero):
//   U(k) = [sum_a [k in shell a] H^_a(k) + [k in G's cube] Q^(k) / V] / W(k).
// Membership uses the same exact |k| and cube tests as the forward field
// builders.
template <class FR, class UR>
__global__ void __launch_bounds__(256)
adjoint_spectrum_kernel(Geom g, int M0, int M1, int M2, int K0, int K1,
                        int K2, int Kg0, int Kg1, int Kg2,
                        const typename CplxOf<FR>::type* Hh,
                        const typename CplxOf<FR>::type* Qh, const double* lo,
                        const double* hi, int nb, AxisTablesDev ax,
                        typename CplxOf<UR>::type* U) {
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
    const bool in_g = (M0 == g.n[0] || abs(sx) <= Kg0) &&
                      (M1 == g.n[1] || abs(sy) <= Kg1) &&
                      (M2 == g.n[2] || abs(sz) <= Kg2);
    if (!in_g) continue;
    const bool in_f = (M0 == g.n[0] || abs(sx) <= K0) &&
                      (M1 == g.n[1] || abs(sy) <= K1) &&
                      (M2 == g.n[2] || abs(sz) <= K2);
    const int i = wrap(sx, g.n[0]), j = wrap(sy, g.n[1]),
              k = wrap(sz, g.n[2]);
    cd u = {double(Qh[t].x) / g.vol, double(Qh[t].y) / g.vol};
    if (in_f) {
      const double kx = dmul(double(sx), g.dk[0]);
      const double ky = dmul(double(sy), g.dk[1]);
      const double kz = dmul(double(sz), g.dk[2]);
      const double km = vec3_mag(kx, ky, kz);
      for (int q = 0; q < nb; ++q) {
        if (lo[q] <= km && km < hi[q]) {
          const auto h = Hh[int64_t(q) * count + t];
          u.re += double(h.x);
          u.im += double(h.y);
        }
      }
    }
    const double w = window_pow(ax, i, j, k);
    typename CplxOf<UR>::type o;
    o.x = UR(u.re / w);
    o.y = UR(u.im / w);
    U[(int64_t(i) * g.n[1] + j) * g.nzh + k] = o;
  }
}

// Per particle: dL/dw = sum_c grad(c) W(c) and
// dL/dx = w (n / L) sum_c grad(c) dW/ds(c), with the exact stencil of the
// assignment (unit weights when the catalogue has none).
template <int ORDER, class Real>
__global__ void __launch_bounds__(256)
gather_grad_kernel(Geom g, DevCatalogue cat, const Real* grad, double* gw,
                   double* gx, double* gy, double* gz) {
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < cat.n;
       p += int64_t(gridDim.x) * blockDim.x) {
    const double pos[3] = {cat.x[p], cat.y[p], cat.z[p]};
    Stencil<ORDER> st[3];
    double dw[3][ORDER];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      st[a] = axis_stencil<ORDER>(pos[a], g.n[a], g.L[a], false);
      axis_window_deriv<ORDER>(pos[a], g.n[a], g.L[a], dw[a]);
    }
    double sw = 0., sdx = 0., sdy = 0., sdz = 0.;
#pragma unroll
    for (int i = 0; i < ORDER; ++i)
#pragma unroll
      for (int j = 0; j < ORDER; ++j)
#pragma unroll
        for (int k = 0; k < ORDER; ++k) {
          const int64_t c =
              (int64_t(st[0].idx[i]) * g.n[1] + st[1].idx[j]) * g.n[2] +
              st[2].idx[k];
          if (c < 0 || c >= g.nmesh) continue;
          const double v = double(grad[c]);
          const double wx = st[0].win[i], wy = st[1].win[j],
                       wz = st[2].win[k];
          sw += v * wx * wy * wz;
          sdx += v * dw[0][i] * wy * wz;
          sdy += v * wx * dw[1][j] * wz;
          sdz += v * wx * wy * dw[2][k];
        }
    const double w = (cat.w != nullptr) ? cat.w[p] : 1.;
    if (gw != nullptr) gw[p] = sw;
    if (gx != nullptr) {
      gx[p] = w * sdx * (double(g.n[0]) / g.L[0]);
      gy[p] = w * sdy * (double(g.n[1]) / g.L[1]);
      gz[p] = w * sdz * (double(g.n[2]) / g.L[2]);
    }
  }
}

// The weight field of the uncoupled shot-noise terms S_ab = vol_cell
// sum_x xi(x) j_0(k_a |x|) j_0(k_b |x|) of every pair:
// W(x) = sum_p mu_p j_0(k_a |x|) j_0(k_b |x|), from a table over the
// integer keys sx^2 + sy^2 + sz^2 (cubic cells) or evaluated per cell.
__global__ void shot_weight_table_kernel(int nkeys, double dr,
                                         SplineTable sj, int np,
                                         const double* ka, const double* kb,
                                         const double* mu, double* table) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nkeys;
       t += gridDim.x * blockDim.x) {
    const double r = sqrt(double(t)) * dr;
    double acc = 0.;
    for (int p = 0; p < np; ++p)
      acc += mu[p] * spline_eval(sj, ka[p] * r) * spline_eval(sj, kb[p] * r);
    table[t] = acc;
  }
}

template <class Real>
__global__ void shot_weight_field_kernel(Geom g, const double* table,
                                         SplineTable sj, int np,
                                         const double* ka, const double* kb,
                                         const double* mu, Real* W) {
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
       t < g.nmesh; t += int64_t(gridDim.x) * blockDim.x) {
    const int k = int(t % g.n[2]);
    const int j = int((t / g.n[2]) % g.n[1]);
    const int i = int(t / (int64_t(g.n[2]) * g.n[1]));
    const int sx = shift_index(i, g.n[0]), sy = shift_index(j, g.n[1]),
              sz = shift_index(k, g.n[2]);
    if (table != nullptr) {
      W[t] = Real(table[sx * sx + sy * sy + sz * sz]);
      continue;
    }
    const double rx = double(sx) * g.dr[0], ry = double(sy) * g.dr[1],
                 rz = double(sz) * g.dr[2];
    const double r = sqrt(rx * rx + ry * ry + rz * rz);
    double acc = 0.;
    for (int p = 0; p < np; ++p)
      acc += mu[p] * spline_eval(sj, ka[p] * r) * spline_eval(sj, kb[p] * r);
    W[t] = Real(acc);
  }
}

}  // namespace

template <class Real>
void launch_shot_weight_field(Context& ctx, const Geom& g,
                              const SplineTable& sj, int np,
                              const double* ka, const double* kb,
                              const double* mu, double* table, Real* W) {
  const bool cubic = g.dr[0] == g.dr[1] && g.dr[1] == g.dr[2];
  const int nkeys = (g.n[0] / 2) * (g.n[0] / 2) + (g.n[1] / 2) * (g.n[1] / 2) +
                    (g.n[2] / 2) * (g.n[2] / 2) + 1;
  if (cubic) {
    TRVG_KBEGIN(ctx, "shot_weight_table_kernel");
    shot_weight_table_kernel<<<grid_for(nkeys, 128), 128, 0, ctx.stream>>>(
        nkeys, g.dr[0], sj, np, ka, kb, mu, table);
    TRVG_LAUNCHED(ctx);
  }
  TRVG_KBEGIN(ctx, "shot_weight_field_kernel");
  shot_weight_field_kernel<Real><<<grid_for(g.nmesh, 256), 256, 0,
                                   ctx.stream>>>(g, cubic ? table : nullptr,
                                                 sj, np, ka, kb, mu, W);
  TRVG_LAUNCHED(ctx);
}

template void launch_shot_weight_field<float>(Context&, const Geom&,
                                              const SplineTable&, int,
                                              const double*, const double*,
                                              const double*, double*, float*);
template void launch_shot_weight_field<double>(Context&, const Geom&,
                                               const SplineTable&, int,
                                               const double*, const double*,
                                               const double*, double*,
                                               double*);

template <class FR>
void launch_adjoint_fields(Context& ctx, int64_t ncell, const FR* G,
                           const FR* F, int nb, const AdjointLists& l, FR* H,
                           FR* Q) {
  TRVG_KBEGIN(ctx, "adjoint_fields_kernel");
  adjoint_fields_kernel<FR><<<grid_for(ncell, 256), 256, 0, ctx.stream>>>(
      ncell, G, F, nb, l, H, Q);
  TRVG_LAUNCHED(ctx);
}

template <class FR, class UR>
void launch_adjoint_spectrum(Context& ctx, const Geom& g, const int M[3],
                             const int K[3], const int Kg[3],
                             const typename CplxOf<FR>::type* Hh,
                             const typename CplxOf<FR>::type* Qh,
                             const double* lo, const double* hi, int nb,
                             const AxisTablesDev& ax,
                             typename CplxOf<UR>::type* U) {
  const int64_t count = int64_t(M[0]) * M[1] * (M[2] / 2 + 1);
  if (count >= (int64_t(1) << 32))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Evaluation grid too large.");
  TRVG_KBEGIN(ctx, "adjoint_spectrum_kernel");
  adjoint_spectrum_kernel<FR, UR><<<grid_for(count, 256), 256, 0,
                                    ctx.stream>>>(
      g, M[0], M[1], M[2], K[0], K[1], K[2], Kg[0], Kg[1], Kg[2], Hh, Qh, lo,
      hi, nb, ax, U);
  TRVG_LAUNCHED(ctx);
}

template <class Real>
void launch_gather_grad(Context& ctx, const Geom& g, int order,
                        const DevCatalogue& cat, const Real* grad, double* gw,
                        double* gx, double* gy, double* gz) {
  if (cat.n == 0) return;
  const int grid = grid_for(cat.n, 256);
  TRVG_KBEGIN(ctx, "gather_grad_kernel");
  switch (order) {
    case 1:
      gather_grad_kernel<1, Real><<<grid, 256, 0, ctx.stream>>>(
          g, cat, grad, gw, gx, gy, gz);
      break;
    case 2:
      gather_grad_kernel<2, Real><<<grid, 256, 0, ctx.stream>>>(
          g, cat, grad, gw, gx, gy, gz);
      break;
    case 3:
      gather_grad_kernel<3, Real><<<grid, 256, 0, ctx.stream>>>(
          g, cat, grad, gw, gx, gy, gz);
      break;
    case 4:
      gather_grad_kernel<4, Real><<<grid, 256, 0, ctx.stream>>>(
          g, cat, grad, gw, gx, gy, gz);
      break;
    default:
      throw_error(TRVG_ERR_INVALID_PARAMETER,
                  "Unsupported mesh assignment order: %d.", order);
  }
  TRVG_LAUNCHED(ctx);
}

template void launch_adjoint_fields<float>(Context&, int64_t, const float*,
                                           const float*, int,
                                           const AdjointLists&, float*,
                                           float*);
template void launch_adjoint_fields<double>(Context&, int64_t, const double*,
                                            const double*, int,
                                            const AdjointLists&, double*,
                                            double*);
template void launch_adjoint_spectrum<float, float>(
    Context&, const Geom&, const int*, const int*, const int*, const float2*,
    const float2*, const double*, const double*, int, const AxisTablesDev&,
    float2*);
template void launch_adjoint_spectrum<double, double>(
    Context&, const Geom&, const int*, const int*, const int*,
    const double2*, const double2*, const double*, const double*, int,
    const AxisTablesDev&, double2*);
template void launch_adjoint_spectrum<float, double>(
    Context&, const Geom&, const int*, const int*, const int*, const float2*,
    const float2*, const double*, const double*, int, const AxisTablesDev&,
    double2*);
template void launch_gather_grad<float>(Context&, const Geom&, int,
                                        const DevCatalogue&, const float*,
                                        double*, double*, double*, double*);
template void launch_gather_grad<double>(Context&, const Geom&, int,
                                         const DevCatalogue&, const double*,
                                         double*, double*, double*, double*);

}  // namespace trvg
