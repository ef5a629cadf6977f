// Host launchers of the CUDA kernels.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace trvg {

template <class Real> struct CplxOf;
template <> struct CplxOf<float> { using type = float2; };
template <> struct CplxOf<double> { using type = double2; };

// Mesh geometry of one estimate.
struct Geom {
  int n[3];
  double L[3];
  double dk[3];        // 2 pi / L (field.cpp:358-360)
  double dr[3];        // L / n   (field.cpp:353-355)
  double vol, vol_cell;
  int64_t nmesh;
  int nzh;             // n[2] / 2 + 1 (half-spectrum extent)
  int64_t nhalf;       // n[0] * n[1] * nzh
};

// Particle arrays in device memory.
struct DevCatalogue {
  int64_t n = 0;  // particle count (the largest count in a replayed batch)
  const double* x = nullptr;
  const double* y = nullptr;
  const double* z = nullptr;
  const double* w = nullptr;
  const double* lx = nullptr;
  const double* ly = nullptr;
  const double* lz = nullptr;
  // Replayed batches: the current mock's count and first particle are read
  // on the device (the columns then start at x + *dev_first).
  const int64_t* dev_n = nullptr;
  const int64_t* dev_first = nullptr;
  // Set by sort_catalogue: particles of mesh tile k (cubes of 2^tile_shift
  // cells, x-major) are [tile_start[k], tile_start[k + 1]), the last tile
  // ending at count().
  const int* tile_start = nullptr;
  int tile_shift = 0;
  __device__ __forceinline__ int64_t count() const {
    return dev_n != nullptr ? *dev_n : n;
  }
  __device__ __forceinline__ int64_t first() const {
    return dev_first != nullptr ? *dev_first : 0;
  }
};

// Several Y_lm-weighted fields of one degree built in one pass over a
// catalogue (compute_ylm_wgtd_field / compute_ylm_wgtd_quad_field,
// field.cpp:1246-1500, for every order
// at once): target t deposits scale_t * w^power_t * [conj] y_l,m_t(los)
// into its own meshes (re; im for complex fields; shadows when
// interlacing).  A target without meshes only sums the weights.
constexpr int kMaxYlmTargets = 16;
constexpr int kMaxYlmDegree = 8;

struct YlmTarget {
  int m = 0;
  int power = 1;
  bool conj = false;
  double scale = 1.;
  float* re = nullptr;
  float* im = nullptr;
  float* sre = nullptr;
  float* sim = nullptr;
  double* sums = nullptr;  // [4]: landed weight (re, im, shadow re, im)
  // Compensated deposit (launches with compensation meshes): the target's
  // catalogues enter with opposite signs, so its sums cancel.  Other
  // targets deposit plain FP32 sums into the same meshes.
  bool comp = true;
};

struct YlmTargets {
  int ell = 0;
  int count = 0;
  double cnorm[kMaxYlmDegree + 1] = {};  // ylm_all_norms(ell), by the launchers
  YlmTarget t[kMaxYlmTargets];
};

// The value every cell of a mesh holds before its first deposit
// (fill_offset_kernel: -sum / ncells, sum read from dsum when given).  With
// it the tiled assignment stores the cells that only its own tile reaches
// instead of adding to them.
struct MeshFill {
  const double* dsum = nullptr;
  double hsum = 0.;
};

// Per-particle weight scale * w^power * [conj] y_lm(los).
struct WeightSpec {
  double scale = 1.0;
  int power = 1;
  bool use_ylm = false;
  int ell = 0, m = 0;
  bool conj_ylm = false;
};

// Spectrum of a (possibly complex) mesh field stored as the half spectra
// of its real and imaginary part meshes, with an optional interlacing
// shadow and an exact override of the k = 0 mode.
template <class Real>
struct FieldSpec {
  using C = typename CplxOf<Real>::type;
  const C* re = nullptr;
  const C* im = nullptr;
  const C* re_s = nullptr;
  const C* im_s = nullptr;
  cd k0 = {0., 0.};
  bool k0_set = false;
  // Replayed batches: the k = 0 mode (re, im) in device memory instead.
  const double* k0_dev = nullptr;
  // The real FP32 mesh the spectrum came from (real fields without
  // interlacing), valid while mesh_gen equals the context's counter.
  const Real* mesh = nullptr;
  // Its compensation mesh (compensated FP32 deposit), or nullptr.
  const Real* mesh_lo = nullptr;
  int64_t mesh_gen = -1;
  // The field is sign * (FFT[re] + i im_sign FFT[im]) away from k = 0: a
  // conjugated view (im_sign = -1) gives the order -M of a Y_lm-weighted
  // field from the meshes of order M.
  double sign = 1.;
  double im_sign = 1.;
};

// Device copies of the per-axis Fourier factor tables.
struct AxisTablesDev {
  AxisTables t;
  int order;           // assignment order
  bool interlace;
};

// W(k)^order (field.cpp:1114-1146) at full-mesh index (i, j, k).
__device__ __forceinline__ double window_pow(const AxisTablesDev& ax, int i,
                                             int j, int k) {
  const double wk = ax.t.sinc[0][i] * ax.t.sinc[1][j] * ax.t.sinc[2][k];
  double r = 1.;
  for (int q = 0; q < ax.order; ++q) r *= wk;
  return r;
}

// Bin edges and the fine-sample index ranges of each bin.
struct BinsDev {
  int nbins = 0;
  const double* lo = nullptr;
  const double* hi = nullptr;
  const int* smin = nullptr;   // first fine sample index in the bin
  const int* smax = nullptr;   // one past the last
  // Cells with s_x^2 + s_y^2 + s_z^2 above key_max lie beyond every bin
  // (-1: no such bound).
  int64_t key_max = -1;
};

// ---- shot-noise field on one octant (spectral.cu, reduce.cu) --------------
// Flip-averaged FP32 spectrum of a real two-point field as the even
// extensions of its z lines ((n_x/2 + 1)(n_y/2 + 1) lines of n_z floats).
void launch_xi_octant_spectrum(Context& ctx, const Geom& g, const float2* fa,
                               const float2* fb, const float* const inv_alias[3],
                               float shot, float2 p0, const double* k0a,
                               const double* k0b, const double* shotp,
                               float* ext);
// The same from one field's FP32 planes planes[kz][x][y] (both legs that
// field).
void launch_xi_octant_planes(Context& ctx, const Geom& g, const float2* planes,
                             const float* const inv_alias[3], float shot,
                             float2 p0, const double* k0a, const double* k0b,
                             const double* shotp, float* ext);
// dst[s dS + k dK + r] = dst[s dS + k dK + len - r] = src[s sS + r sR + k].x.
void launch_octant_transpose(Context& ctx, const float2* src, int64_t sS,
                             int64_t sR, float* dst, int64_t dS, int64_t dK,
                             int nslab, int nrow, int ncol, int len);
// Radial sums of the octant xi (weights y_l0 y_l'0 for degrees > 0).
void launch_octant_hist(Context& ctx, const Geom& g, const float2* xo,
                        int ell_a, int ell_b, double* hist);

// ---- assign.cu -----------------------------------------------------------
template <class Real>
void launch_assign(Context& ctx, const Geom& g, int order, bool interlace,
                   const DevCatalogue& cat, const WeightSpec& ws,
                   Real* mesh_re, Real* mesh_im, Real* shadow_re,
                   Real* shadow_im, double* sums /* [4]: re, im, s_re, s_im */,
                   const MeshFill* fill = nullptr, int64_t lo_off = 0);
// lo_off != 0 (FP32 meshes): every target mesh m has a compensation mesh
// at m + lo_off; windows and products are float-float and the atomic sums
// compensated, so that m + (m + lo_off) holds the deposit to about 2^-44.
// sum_p scale_t * w^power_t * [conj] y_lm_t for every target, added to
// out[2 t], out[2 t + 1].
void launch_ylm_weight_sums(Context& ctx, const DevCatalogue& cat,
                            const YlmTargets& ts, double* out);
// Deposit of every target's weights into its meshes (FP32), the stencil
// of each particle formed once; targets' sums must hold their weight sums
// (launch_ylm_weight_sums): particles off the fast stencil add the
// difference between their landed and their full weight.
void launch_assign_ylm(Context& ctx, const Geom& g, int order, bool interlace,
                       const DevCatalogue& cat, const YlmTargets& ts,
                       int64_t lo_off = 0);
void launch_weight_sum(Context& ctx, const DevCatalogue& cat,
                       const WeightSpec& ws, double* out /* [2] */);
template <class Real>
void launch_mesh_sum_pow(Context& ctx, const Real* mesh, int64_t n, int order,
                         double* out);
template <class Real>
void launch_mesh_to_double(Context& ctx, const Real* mesh, int64_t n,
                           double scale, double* out);
// Fill a mesh with -(sum / n), sum from device memory (`dsum`) or `hsum`
// (and its compensation mesh, lo_off != 0, with the fill's rounding error).
template <class Real>
void launch_fill_offset(Context& ctx, Real* mesh, int64_t n,
                        const double* dsum, double hsum, int64_t lo_off = 0);
// dst = src (an FP32 mesh of the caller) in precision Real.
template <class Real>
void launch_mesh_copy(Context& ctx, const float* src, int64_t n, Real* dst);
// Compensated FP32 mesh -> (correctly rounded sum, remainder).
void launch_mesh_renorm(Context& ctx, float* mesh, int64_t n, int64_t lo_off);

// ---- sort.cu -------------------------------------------------------------
// Copy of `in` ordered by mesh tiles of 2^shift cells a side (device
// buffers named by tag).
DevCatalogue sort_catalogue(Context& ctx, const Geom& g, const DevCatalogue& in,
                            const std::string& tag, int shift = 3);

// ---- spectral.cu ---------------------------------------------------------
// Mode cube: frequencies s in [-K, K] per axis, or the whole axis when
// dense[ax].
struct Cube {
  int K[3];
  bool dense[3];
  int ext[3];
  int64_t count;
};

void launch_count_modes(Context& ctx, const Geom& g, const Cube& cube,
                        const BinsDev& bins, long long* nmodes,
                        double* ksum);

// Field builders read spectra of precision Real and write evaluation-grid
// fields of precision FR.
template <class Real, class FR>
void launch_build_G(Context& ctx, const Geom& g, const int M[3],
                    const int Kg[3], const FieldSpec<Real>& f,
                    const AxisTablesDev& ax,
                    typename CplxOf<FR>::type* out);

template <class Real, class FR>
void launch_build_F(Context& ctx, const Geom& g, const int M[3],
                    const int K[3], const FieldSpec<Real>& f,
                    const AxisTablesDev& ax, int ell, int m,
                    const double* lo, const double* hi, int nb,
                    double hi_max, typename CplxOf<FR>::type* out,
                    bool disjoint_bins = false);

template <class Real, class FR>
// iw: per-axis FP32 1 / W factors (FP32 mode values on meshes with one
// fundamental frequency), or entries nullptr.
void launch_build_F_sjl(Context& ctx, const Geom& g, const FieldSpec<Real>& f,
                        const AxisTablesDev& ax, int ell, int m,
                        const SplineTable& sj, const double* radii, int nb,
                        typename CplxOf<FR>::type* out,
                        const float* const iw[3]);

// Half-spectrum builders for real fields (C2R on the evaluation grid).
template <class Real, class FR>
void launch_build_G_half(Context& ctx, const Geom& g, const int M[3],
                         const int Kg[3], const FieldSpec<Real>& f,
                         const AxisTablesDev& ax,
                         typename CplxOf<FR>::type* out);
template <class Real, class FR>
void launch_build_F_half(Context& ctx, const Geom& g, const int M[3],
                         const int K[3], const FieldSpec<Real>& f,
                         const AxisTablesDev& ax, int ell, int m,
                         const double* lo, const double* hi, int nb,
                         double hi_max, typename CplxOf<FR>::type* out);
template <class Real, class FR>
void launch_build_F_sjl_half(Context& ctx, const Geom& g,
                             const FieldSpec<Real>& f, const AxisTablesDev& ax,
                             int ell, int m, const SplineTable& sj,
                             const double* radii, int nb,
                             typename CplxOf<FR>::type* out,
                             const float* const iw[3]);

// FP32-mixed builders of real fields without interlacing (values FP32,
// shell membership from a table of the exact FP64 test).
void launch_shell_table(Context& ctx, const Geom& g, const int M[3],
                        const int K[3], const double* lo, const double* hi,
                        int nb, double hi_max, int16_t* tab);
void launch_build_G_half_f32(Context& ctx, const Geom& g, const int M[3],
                             const int Kg[3], const float2* f, cd k0,
                             const float* const iw[3], float2* out);
// The shot-noise field spectrum (|f_a f_b^*| / C_1 - S) / V of FP32 spectra
// without interlacing, in FP32; out_im: the imaginary part's spectrum when
// the field is complex (nullptr: real).
void launch_twopt_field_f32(Context& ctx, const Geom& g,
                            const FieldSpec<float>& fa,
                            const FieldSpec<float>& fb, float2 shot,
                            const float* const inv_alias[3], float2* out_re,
                            float2* out_im);
// G on the full evaluation grid for FP32 spectra without interlacing, in
// FP32.
void launch_build_G_f32(Context& ctx, const Geom& g, const int M[3],
                        const int Kg[3], const FieldSpec<float>& f,
                        const float* const iw[3], float2* out);
// Complex FP32 shell spectra on the full evaluation grid from the half-grid
// shell table of disjoint bins (FP32 fields without interlacing).
void launch_build_F_tab_f32(Context& ctx, const Geom& g, const int M[3],
                            const int16_t* tab, const FieldSpec<float>& f,
                            const float* const iw[3], int ell, int m, int nb,
                            float2* out);
void launch_build_F_half_f32(Context& ctx, const Geom& g, const int M[3],
                             const int16_t* tab, const float2* f, cd k0,
                             const float* const iw[3], int ell, int nb,
                             float2* out);

// Cached mode lists of the fine-binned two-point statistics.
// Per cube mode: bin (or -1), coefficient y / W_pk, |k| and the shot-noise
// weight C1 y / W_sn (the per-bin sums are formed on the host, in mode
// order, so that near-cancelling sums do not depend on atomic order).
void launch_stats_plan(Context& ctx, const Geom& g, const Cube& cube,
                       int ell, int m, const AxisTablesDev& ax,
                       const BinsDev& bins, int16_t* qtab, double2* coef,
                       double* kmode, double2* snmode);
void launch_stats_fill(Context& ctx, int64_t nmode, const int16_t* qtab,
                       const int* off, int* cursor, uint32_t* list);
template <class Real>
void launch_stats_pk(Context& ctx, const Geom& g, const Cube& cube,
                     const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                     int nbins, int max_count, const int* off,
                     const uint32_t* list, const double2* coef, double* pk);
// f(x) *= r^-p on the full mesh (r < 1e-6 unchanged): the 3PCF window's
// wide-angle kernel; T is float, double, float2 or double2.
template <class T>
void launch_wide_angle(Context& ctx, const Geom& g, T* f, double p);

// The same sums for one real source mesh (both legs) from its float-float
// spectrum cube |s| <= Kc (launch_ff_forward_cube), k = 0 from k0a / k0b.
void launch_stats_pk_cube(Context& ctx, const Geom& g, const Cube& cube,
                          const float4* ffcube, int Kc, cd k0a, cd k0b,
                          int nbins, int max_count, const int* off,
                          const uint32_t* list, const double2* coef,
                          double* pk, const double* k0a_dev = nullptr,
                          const double* k0b_dev = nullptr);

template <class Real>
void launch_twopt_stats(Context& ctx, const Geom& g, const Cube& cube,
                        const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                        cd shot, int ell, int m, const AxisTablesDev& ax,
                        const BinsDev& bins, long long* nmodes, double* ksum,
                        double* pk, double* sn);

// The shot-noise field spectrum, written in precision XR for its C2R.
template <class Real, class XR>
void launch_twopt_field(Context& ctx, const Geom& g, const FieldSpec<Real>& fa,
                        const FieldSpec<Real>& fb, cd shot,
                        const AxisTablesDev& ax,
                        typename CplxOf<XR>::type* out_re,
                        typename CplxOf<XR>::type* out_im);

// FP32 fast path of the shot-noise field spectrum for two real-mesh spectra
// without interlacing; `p0` is the exact k = 0 mode (already / V).
void launch_twopt_field_real_f32(Context& ctx, const Geom& g,
                                 const float2* fa, const float2* fb,
                                 const float* const inv_alias[3], float shot,
                                 float2 p0, float2* out,
                                 const double* k0a = nullptr,
                                 const double* k0b = nullptr,
                                 const double* shotp = nullptr);

// ---- reduce.cu -----------------------------------------------------------
template <class Real>
void launch_reduce_pairs(Context& ctx, int64_t ncell,
                         const typename CplxOf<Real>::type* G,
                         const typename CplxOf<Real>::type* Fa,
                         const typename CplxOf<Real>::type* Fb,
                         const int* pa, const int* pb, int npairs,
                         double* out /* 2 * npairs */, int na = 0,
                         int nb = 0 /* fields per leg: FP32 tiled form */,
                         bool conj_b = false /* leg b read conjugated
                                                (streaming form only) */);

template <class Real>
void launch_reduce_pairs_real(Context& ctx, int64_t ncell, const Real* G,
                              const Real* Fa, const Real* Fb, const int* pa,
                              const int* pb, int npairs,
                              double* out /* 2 * npairs, imaginary 0 */, int na = 0,
                              int nb = 0);

// Register-tiled Gram form for FP32 fields (real: float, complex: float2
// stored as float pairs).  One thread accumulates a tile of ti leg-a by tj
// leg-b fields; `tiles` lists the (a / ti, b / tj) tiles that hold at least
// one data-vector entry and slot[a * nb + b] is the entry of field pair
// (a, b), -1 when it has none.  Field r of a leg starts ld values after
// field r - 1 (ld = 0: ncell).
struct GramTile {
  int ti, tj;
};
inline GramTile gram_tile(bool cplx) {
  return cplx ? GramTile{2, 4} : GramTile{4, 8};
}
bool gram_tiled_fits(bool cplx, int na, int nb);
void launch_reduce_pairs_tiled(Context& ctx, int64_t ncell, bool cplx,
                               const float* G, const float* Fa, int na,
                               const float* Fb, int nb, const int2* tiles,
                               int ntiles, const int* slot,
                               double* out /* 2 per entry */,
                               int64_t ld = 0);

// ---- ffft.cu -------------------------------------------------------------
// Float-float transforms of the shell fields: a plan is the radix list of
// the length and its twiddle table (cos, sin of 2 pi k / n, float-float).
struct FFPlan {
  int n;
  int nstage;
  int radix[16];
  // Per stage: butterflies per line (n / radix), span of the finished
  // sub-transforms (Ns), twiddle stride n / (Ns radix), and the multipliers
  // floor(2^32 / d) + 1 that divide by n / radix and Ns exactly through a
  // multiply-high (valid for dividends below 2^32 / d).
  int nb[16], ns[16], tstep[16];
  unsigned mnb[16], mns[16];
  // Every stage fits one warp per line (WarpItems butterflies per lane).
  bool warp_lines;
  // Twiddles stage by stage: stage s holds exp(2 pi i r k tstep / n) (the
  // forward direction takes the conjugate) at twoff[s] + (r - 1) ns + k for
  // 1 <= r < radix, 0 <= k < ns, so that the butterflies of a warp
  // (consecutive k) read consecutive entries.
  int twoff[16];
  const float4* tw;
};
bool ff_length_ok(int n);
// The cube's modes (|sx|, |sy| <= Kg, 0 <= sz <= Kg) rounded to FP32 into
// the half spectrum h of the mesh (other entries untouched).
void launch_ff_cube_to_half(Context& ctx, const Geom& g, const float4* cube,
                            int Kg, float2* h);
FFPlan ff_plan(Context& ctx, int n);
// Spectrum of the FP32 mesh on the cube |sx|, |sy| <= Kg, 0 <= sz <= Kg:
// cube[sx + Kg][sy + Kg][sz] (T1, T2: scratch of n0 (Kg+1) n1 and
// (2Kg+1)(Kg+1) n0 float4).  With `full` set the z pass also writes every
// row's transform along z in FP32, plane by plane (full[kz][x][y], kz <=
// n2/2), and `after_z` is recorded on the stream after that pass.
void launch_ff_forward_cube(Context& ctx, const Geom& g, const float* mesh,
                            const float* mesh_lo, int Kg, float4* T1,
                            float4* T2, float4* cube, float2* full = nullptr,
                            cudaEvent_t after_z = nullptr);
// spec[x][y][kz] (the R2C layout, kz <= n2/2) from planes[kz][x][y].
void launch_planes_to_half(Context& ctx, const Geom& g, const float2* planes,
                           float2* spec);
// Evaluation-grid half spectra E[c][b][a] of G (planes c <= Kg) and
// E[q][c][b][a] of nq shell fields (planes c <= K) from the cube.
// k0_dev (re, im in device memory), when given, replaces the host k0.
void launch_ff_build_G(Context& ctx, const Geom& g, const int M[3],
                       const float4* cube, int Kg, const float2* const iw[3],
                       cd k0, float4* E, const double* k0_dev = nullptr);
void launch_ff_build_F(Context& ctx, const Geom& g, const int M[3],
                       const float4* cube, int Kg, int K, const int16_t* tab,
                       int nq, int ell, const float2* const iw[3], cd k0,
                       float4* E, const double* k0_dev = nullptr);
// Lines of the inverse passes that can hold modes when each field of a
// group is a shell (null pointers: every line of the band box).  x lines
// are listed by code (f (Kcf + 1) + c) (2 Kf + 1) + sy + Kf; bm[f (Kcf + 1)
// + c] is the largest |sy| of plane c of field f (-1: none), kz[f] the
// largest plane of field f, and field f owns the y lines [yoff[f],
// yoff[f + 1]), M0 (kz[f] + 1) of them.
struct FFBand {
  const int* xl = nullptr;
  int64_t nxl = 0;
  const int* bm = nullptr;
  const int* kz = nullptr;
  const int64_t* yoff = nullptr;
  int64_t nyl = 0;
};

// Real fields on the M grid of nf half spectra E with planes c <= Kcf and
// band |sx|, |sy| <= Kf, as float-float words: field f at out + f ld (hi)
// and out_lo + f ld (not written when out_lo is null), cells [a][b][z]
// (Y1, Y2: scratch of
// nf (Kcf+1) M0 M1 float4 each).
void launch_ff_inverse(Context& ctx, const int M[3], int nf, int Kf, int Kcf,
                       const float4* E, float4* Y1, float4* Y2, float* out,
                       float* out_lo, int64_t ld,
                       const FFBand& band = FFBand());
// Field stride of the reductions: cells rounded up to whole float4 quads.
inline int64_t ff_field_stride(int64_t ncell) { return (ncell + 3) / 4 * 4; }
// sum_x F_a F_b G of float-float fields (hi, lo words; field q of a leg at
// q ld, ld a multiple of 4, 16-byte aligned bases) for every pair (real
// parts at out[2 p]).
// pairs_per_block: the bin batch of one block (4, 8 or 16; autotuned).
void launch_reduce_pairs_ff(Context& ctx, int64_t ncell, int64_t ld,
                            const float* Gh, const float* Gl,
                            const float* Fah, const float* Fal,
                            const float* Fbh, const float* Fbl, const int* pa,
                            const int* pb, int npairs, double* out,
                            int pairs_per_block = 8);

// ---- batch.cu ------------------------------------------------------------
// Scalars of the current mock of a replayed batch (device memory).
struct MockState {
  int64_t index;      // position in the replay order
  int64_t mock;       // mock number order[index]
  int64_t first;      // first particle of the mock
  int64_t count;      // particle count
  double count_d[2];  // (count, 0): unit-weight deposit and S-bar
  double k0_dn[2];    // k = 0 mode of delta n: deposit - count
  double k0_nf[2];    // k = 0 mode of N: the deposit
  double norm;        // normalisation
};

// Per-term inputs of the host's B and shot-noise combinations: pair sums
// `comp`, statistics sums of the row / column legs (null when unused) with
// their plans' mode counts and shot weights, and shot-noise pair sums.
struct MockTermArgs {
  int ndv;
  const int* prow;
  const int* pcol;
  const double* nmodes;  // shell mode counts per bin
  const double* comp;    // 2 ndv
  double fac, coupling, vol_cell, mirror, mirror_w3j, phase_re, phase_im;
  bool sn_const;         // ell1 = ell2 = 0: + coupling S-bar
  const double* pk_row;
  const double* nst_row;
  const double* snsum_row;
  const double* pk_col;
  const double* nst_col;
  const double* snsum_col;
  const double* sij;     // 2 ndv, before the cell volume
};

// acc: 4 ndv doubles (B re, im; shot re, im), zeroed by mock_begin.
void launch_mock_begin(Context& ctx, MockState* st, const int64_t* order,
                       const int64_t* offsets, const double* norms,
                       double* acc, int nacc);
void launch_mock_k0(Context& ctx, MockState* st, const double* sums);
void launch_mock_term(Context& ctx, const MockState* st,
                      const MockTermArgs& a, double* acc);
// raw, shot: [mock][ndv] complex, times the mock's norm; advances index.
void launch_mock_store(Context& ctx, MockState* st, const double* acc,
                       int ndv, double* raw, double* shot);

// ---- adjoint.cu ----------------------------------------------------------
// Cotangent bookkeeping of the bispectrum adjoint: the partners of bin a in
// the pairs, with their weights, are entries [off[a], off[a + 1]) of
// partner / lam; the pairs themselves are (prow, pcol) with weights plam.
struct AdjointLists {
  const int* off;
  const int* partner;
  const double* lam;
  const int* prow;
  const int* pcol;
  const double* plam;
  int npairs;
};

template <class FR>
void launch_adjoint_fields(Context& ctx, int64_t ncell, const FR* G,
                           const FR* F, int nb, const AdjointLists& l, FR* H,
                           FR* Q);
template <class FR, class UR>
void launch_adjoint_spectrum(Context& ctx, const Geom& g, const int M[3],
                             const int K[3], const int Kg[3],
                             const typename CplxOf<FR>::type* Hh,
                             const typename CplxOf<FR>::type* Qh,
                             const double* lo, const double* hi, int nb,
                             const AxisTablesDev& ax,
                             typename CplxOf<UR>::type* U);
template <class Real>
void launch_gather_grad(Context& ctx, const Geom& g, int order,
                        const DevCatalogue& cat, const Real* grad, double* gw,
                        double* gx, double* gy, double* gz);
// Shot-noise adjoint (ell = 0).  Single-leg terms: U += fac[a] coef d for
// the listed modes of each two-point statistics bin a (stats plan lists).
template <class Real, class UR>
void launch_adjoint_stats(Context& ctx, const Geom& g, const Cube& cube,
                          const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                          int nbins, int max_count, const int* off,
                          const uint32_t* list, const double2* coef,
                          const double* fac, typename CplxOf<UR>::type* U);
// W(x) = sum_p mu_p j_0(ka_p |x|) j_0(kb_p |x|) on the full mesh (`table`:
// scratch of one double per integer key for cubic cells).
template <class Real>
void launch_shot_weight_field(Context& ctx, const Geom& g,
                              const SplineTable& sj, int np,
                              const double* ka, const double* kb,
                              const double* mu, double* table, Real* W);
// Pair terms: U += 2 scale FFT[W](k) / C_1(k) delta(k) on the half
// spectrum (k = 0: the legs' k = 0 values).
template <class Real>
void launch_adjoint_xi(Context& ctx, const Geom& g,
                       const typename CplxOf<Real>::type* Wh,
                       const FieldSpec<Real>& fa, const FieldSpec<Real>& fb,
                       const AxisTablesDev& ax, double scale,
                       typename CplxOf<Real>::type* U);

template <class Real>
void launch_radial_hist(Context& ctx, const Geom& g, const Real* xi_re,
                        const Real* xi_im, int ell_a, int m_a, int ell_b,
                        int m_b, double* hist /* 2 * nkeys */);

// With `ff` (and the tables' FP32 copies) the Bessel weights come from the
// float-float evaluation on the FP32 pipe, else from the FP64 spline.
void launch_pair_bessel_sums(Context& ctx, const Geom& g, int64_t nkeys,
                             const double* hist, const SplineTable& sja,
                             const SplineTable& sjb, const double* ka,
                             const double* kb, int npairs, bool ff,
                             double* out,
                             const double* rkey = nullptr);
// launch_pair_bessel_sums (float-float) as a Gram product over the
// distinct bins of each leg (ka_d[nka], kb_d[nkb]; pair p uses ka_d[pa[p]],
// kb_d[pb[p]]; same: one leg).  Returns false, launching nothing, when its
// tables do not fit in shared memory.
bool launch_pair_bessel_gram(Context& ctx, const Geom& g, int64_t nkeys,
                             const double* hist, const SplineTable& sja,
                             const SplineTable& sjb, const double* ka_d,
                             int nka, const double* kb_d, int nkb, bool same,
                             const int* pa, const int* pb, int npairs,
                             double* out, const double* rkey = nullptr);
// Sums of xi y_a y_b over cells of any shape, keyed by (|s_x|, |s_y|,
// |s_z|) on (n - n/2 + 1)^3 keys (per axis), with each key's radius in
// rkey.
template <class Real>
void launch_octant_cell_hist(Context& ctx, const Geom& g, const Real* xi_re,
                             const Real* xi_im, int ell_a, int m_a, int ell_b,
                             int m_b, double* hist, double* rkey);


template <class Real>
void launch_shotnoise_3pcf_bins(Context& ctx, const Geom& g, const Real* xi_re,
                                const Real* xi_im, int ell_a, int m_a,
                                int ell_b, int m_b, const BinsDev& bins,
                                long long* npairs, double* rsum, double* xi);

}  // namespace trvg
