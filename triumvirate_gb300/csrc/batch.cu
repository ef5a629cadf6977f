// Device-side bookkeeping of a replayed batch of periodic-box bispectra.
//
// A batch runs its largest mock as an ordinary estimate (which builds every
// cached table, plan and buffer), captures the sequence of one more mock
// into a CUDA graph, and replays that graph for the remaining mocks.  The
// captured sequence cannot read anything back to the host, so the scalars
// that differ from mock to mock live in a MockState in device memory:
//   * mock_begin_kernel selects the next mock (first particle, count, norm);
//   * mock_k0_kernel forms the exact k = 0 modes from the deposited sums;
//   * mock_term_kernel does what the host does per term after the pair,
//     two-point and shot-noise sums (threept.cpp:1675-2140): the B and
//     shot-noise combinations, accumulated per data-vector entry;
//   * mock_store_kernel applies the normalisation, writes the mock's data
//     vector and advances the batch position.
#include <algorithm>

#include "kernels.h"

namespace trvg {

namespace {

__global__ void mock_begin_kernel(MockState* st, const int64_t* order,
                                  const int64_t* offsets, const double* norms,
                                  double* acc, int nacc) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t m = order[st->index];
    st->mock = m;
    st->first = offsets[m];
    st->count = offsets[m + 1] - offsets[m];
    st->count_d[0] = double(st->count);
    st->count_d[1] = 0.;
    st->norm = norms[m];
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nacc;
       i += gridDim.x * blockDim.x)
    acc[i] = 0.;
}

// sums[0..1]: the deposited weight of the unit-weight mesh (re, im).
__global__ void mock_k0_kernel(MockState* st, const double* sums) {
  st->k0_nf[0] = sums[0];
  st->k0_nf[1] = sums[1];
  st->k0_dn[0] = sums[0] - st->count_d[0];  // delta n = n - nbar V
  st->k0_dn[1] = sums[1];
}

__device__ __forceinline__ cd cmul(cd a, cd b) {
  return cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// One statistics leg: (pk - S sn) / nmodes for bin b (zero without modes).
__device__ __forceinline__ cd stats_leg(const double* pk, const double* nst,
                                        const double* snsum, cd shot, int b) {
  const double n = nst[b];
  if (n == 0.) return cd{0., 0.};
  const cd pkb = {pk[2 * b] / n, pk[2 * b + 1] / n};
  const cd snb = cmul(shot, cd{snsum[2 * b], snsum[2 * b + 1]});
  return cd{pkb.re - snb.re / n, pkb.im - snb.im / n};
}

__global__ void mock_term_kernel(const MockState* st, MockTermArgs a,
                                 double* acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.ndv) return;
  const int r = a.prow[i], c = a.pcol[i];
  const cd sbar = {st->count_d[0], st->count_d[1]};
  // Raw bispectrum.
  const double den = a.nmodes[r] * a.nmodes[c];
  const cd B = {a.comp[2 * i] * a.fac / den, a.comp[2 * i + 1] * a.fac / den};
  const double cv = a.coupling * a.vol_cell;
  acc[4 * i] += cv * (B.re + a.mirror * B.re);
  acc[4 * i + 1] += cv * (B.im - a.mirror * B.im);
  // Shot noise.
  cd sn = {0., 0.};
  if (a.sn_const) sn = cd{a.coupling * sbar.re, a.coupling * sbar.im};
  if (a.pk_row != nullptr) {
    const cd s = stats_leg(a.pk_row, a.nst_row, a.snsum_row, sbar, r);
    const cd S = {a.coupling * s.re, a.coupling * s.im};
    sn = cd{sn.re + S.re + a.mirror * S.re, sn.im + S.im - a.mirror * S.im};
  }
  if (a.pk_col != nullptr) {
    const cd s = stats_leg(a.pk_col, a.nst_col, a.snsum_col, sbar, c);
    const cd S = {a.coupling * s.re, a.coupling * s.im};
    sn = cd{sn.re + S.re + a.mirror * S.re, sn.im + S.im - a.mirror * S.im};
  }
  const cd S = {a.coupling * (a.sij[2 * i] * a.vol_cell),
                a.coupling * (a.sij[2 * i + 1] * a.vol_cell)};
  const cd u = {S.re + a.mirror_w3j * S.re, S.im - a.mirror_w3j * S.im};
  const cd ph = cmul(cd{a.phase_re, a.phase_im}, u);
  acc[4 * i + 2] += sn.re + ph.re;
  acc[4 * i + 3] += sn.im + ph.im;
}

__global__ void mock_store_kernel(MockState* st, const double* acc, int ndv,
                                  double* raw, double* shot) {
  const int64_t m = st->mock;
  const double nf = st->norm;
  for (int i = threadIdx.x; i < ndv; i += blockDim.x) {
    raw[(m * ndv + i) * 2] = nf * acc[4 * i];
    raw[(m * ndv + i) * 2 + 1] = nf * acc[4 * i + 1];
    shot[(m * ndv + i) * 2] = nf * acc[4 * i + 2];
    shot[(m * ndv + i) * 2 + 1] = nf * acc[4 * i + 3];
  }
  __syncthreads();
  if (threadIdx.x == 0) st->index += 1;
}

}  // namespace

void launch_mock_begin(Context& ctx, MockState* st, const int64_t* order,
                       const int64_t* offsets, const double* norms,
                       double* acc, int nacc) {
  TRVG_KBEGIN(ctx, "batch_kernel");
  mock_begin_kernel<<<std::max(1, (nacc + 255) / 256), 256, 0, ctx.stream>>>(
      st, order, offsets, norms, acc, nacc);
  TRVG_LAUNCHED(ctx);
}

void launch_mock_k0(Context& ctx, MockState* st, const double* sums) {
  TRVG_KBEGIN(ctx, "batch_kernel");
  mock_k0_kernel<<<1, 1, 0, ctx.stream>>>(st, sums);
  TRVG_LAUNCHED(ctx);
}

void launch_mock_term(Context& ctx, const MockState* st,
                      const MockTermArgs& a, double* acc) {
  if (a.ndv <= 0) return;
  TRVG_KBEGIN(ctx, "batch_kernel");
  mock_term_kernel<<<(a.ndv + 255) / 256, 256, 0, ctx.stream>>>(st, a, acc);
  TRVG_LAUNCHED(ctx);
}

void launch_mock_store(Context& ctx, MockState* st, const double* acc,
                       int ndv, double* raw, double* shot) {
  TRVG_KBEGIN(ctx, "batch_kernel");
  mock_store_kernel<<<1, 256, 0, ctx.stream>>>(st, acc, ndv, raw, shot);
  TRVG_LAUNCHED(ctx);
}

}  // namespace trvg
