// FFTLog Hankel transforms (fftlog.cpp, include/fftlog.hpp:68-257), batched
// on the device.
//
// The forward biased Hankel transform
//   b(k) = int_0^inf k dr (k r)^q J_mu(k r) a(r)
// of samples a_j on log-spaced points r_j is, with FFTLog (Hamilton 2000),
// b = FFT[ u_m FFT[a] / N ] on the points k_j = (k r)_c exp(-dL) / r_{N-1-j},
// the kernel coefficients u_m following from ratios of complex gamma
// functions.  The plan (sample points, pivot, kernel) is set up once on the
// host in FP64; a transform of `batch` rows runs as two batched Z2Z cuFFT
// executions around one kernel multiplication, so the many rows of a
// double spherical-Bessel transform go in one call.
#include <algorithm>
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "internal.h"
#include "kernels.h"

namespace trvg {

namespace {

using zd = std::complex<double>;

// ln Gamma(z) away from the poles: the argument is moved to Re z >= 10 by
// Gamma(z) = Gamma(z + n) / (z (z + 1) ... (z + n - 1)), then the Stirling
// series with Bernoulli terms up to B_14 (remainder below 1e-16 there).
// The imaginary part is the phase of Gamma(z) up to a multiple of 2 pi,
// which is all the transform and the pivot condition use.
zd lngamma(zd z) {
  zd shift = 0.;
  while (z.real() < 10.) {
    shift += std::log(z);
    z += 1.;
  }
  const zd w1 = 1. / z, w2 = w1 * w1;
  // B_2k / (2k (2k - 1)) for k = 1..7.
  const double c[7] = {1. / 12., -1. / 360., 1. / 1260., -1. / 1680.,
                       1. / 1188., -691. / 360360., 1. / 156.};
  zd series = 0.;
  for (int k = 6; k >= 0; --k) series = series * w2 + c[k];
  series *= w1;
  return (z - 0.5) * std::log(z) - z + 0.5 * std::log(2. * M_PI) + series -
         shift;
}

// b[r][m] = a[r][m] * u[m] / n for every row r.
__global__ void hankel_kernel_mul(double2* buf, const double2* u, int n,
                                  int64_t total) {
  const double inv = 1. / double(n);
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < total;
       t += int64_t(gridDim.x) * blockDim.x) {
    const double2 a = buf[t], k = u[t % n];
    buf[t] = make_double2((a.x * k.x - a.y * k.y) * inv,
                          (a.x * k.y + a.y * k.x) * inv);
  }
}

}  // namespace

struct HankelPlan {
  double mu = 0., q = 0.;
  int n = 0;        // samples
  int n_trans = 0;  // transform length (with native extrapolation)
  int n_ext = 0;    // extra samples on either side
  int extrap = 0;   // 0 none, 1 zero, 2 pad, 3 lin, 4 loglin
  double logres = 0., pivot = 1.;
  std::vector<double> pre, post;  // sample points before / after
  std::vector<zd> kernel;         // u_m, m < n_trans
};

namespace {

// Pivot (k r)_c of the low-ringing condition (fftlog.cpp:254-295).
double lowring_pivot(double mu, double q, double dL, double kr_c) {
  const double y = M_PI / (2. * dL);
  if (kr_c > 0.) {
    const zd gp = lngamma(zd((mu + 1. + q) / 2., y));
    const zd gm = lngamma(zd((mu + 1. - q) / 2., y));
    const double argphase =
        std::log(2. / kr_c) / dL + (gp.imag() + gm.imag()) / M_PI;
    return kr_c * std::exp(dL * (argphase - std::round(argphase)));
  }
  // ln Gamma((mu + 1 + nu) / 2) - ln Gamma((mu + 1 - nu) / 2), nu = q + 2 i y.
  const zd nu(q, 2. * y);
  const zd lr = lngamma((mu + 1. + nu) / 2.) - lngamma((mu + 1. - nu) / 2.);
  const double lnkr = std::log(2.) + lr.imag() / (2. * y);
  return std::exp(lnkr - std::floor(lnkr / dL) * dL);
}

// u_m (fftlog.cpp:297-356): |u| = 2^q |Gamma(x+)| / |Gamma(x-)|,
// arg u = m t + arg Gamma(x+) + arg Gamma(x-), x+- = (mu + 1 +- q) / 2 +
// i m y, y = pi / (N dL), t = -2 y ln(kr_c / 2); u_{N-m} = conj(u_m) and a
// real u_{N/2}.
std::vector<zd> kernel_coeff(double mu, double q, int N, double dL,
                             double kr_c) {
  const double y = M_PI / (double(N) * dL);
  const double t = -2. * y * std::log(kr_c / 2.);
  std::vector<zd> u(N);
  for (int m = 0; m <= N / 2; ++m) {
    if (q == 0.) {
      const zd ge = lngamma(zd((mu + 1.) / 2., m * y));
      u[m] = std::polar(1., m * t + 2. * ge.imag());
    } else {
      const zd gp = lngamma(zd((mu + 1. + q) / 2., m * y));
      const zd gm = lngamma(zd((mu + 1. - q) / 2., m * y));
      u[m] = std::polar(std::exp(q * std::log(2.) + gp.real() - gm.real()),
                        m * t + gp.imag() + gm.imag());
    }
  }
  for (int m = N / 2 + 1; m < N; ++m) u[m] = std::conj(u[N - m]);
  if (N % 2 == 0) u[N / 2] = zd(u[N / 2].real(), 0.);
  return u;
}

// Extended copy of a real row (arrayops.cpp:94-203): constant (zero or
// end-value) padding, linear or log-linear continuation of the end steps.
void extend_row(const double* a, int n, int n_ext, int option, double* out) {
  for (int i = 0; i < n; ++i) out[n_ext + i] = a[i];
  for (int i = 0; i < n_ext; ++i) {
    const int dl = i - n_ext;        // -n_ext .. -1
    const int dr = i + 1;            // 1 .. n_ext
    double lo = 0., hi = 0.;
    switch (option) {
      case 1: break;
      case 2:
        lo = a[0];
        hi = a[n - 1];
        break;
      case 3:
        lo = a[0] + dl * (a[1] - a[0]);
        hi = a[n - 1] + dr * (a[n - 1] - a[n - 2]);
        break;
      default:  // 4: log-linear
        lo = a[0] * std::exp(dl * std::log(a[1] / a[0]));
        hi = a[n - 1] * std::exp(dr * std::log(a[n - 1] / a[n - 2]));
        break;
    }
    out[i] = lo;
    out[n_ext + n + i] = hi;
  }
}

}  // namespace

HankelPlan* hankel_plan_create(double mu, double q, const double* x, int n,
                               double kr_c, bool lowring, int extrap,
                               double extrap_exp) {
  if (((mu + 1. + q) <= 0. && std::floor(mu + 1. + q) == (mu + 1. + q)) ||
      ((mu + 1. - q) <= 0. && std::floor(mu + 1. - q) == (mu + 1. - q)))
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Invalid values of order `mu` and bias `q`: negative poles "
                "in the gamma function.");
  if (x == nullptr || n < 2)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "The number of sample points must be at least 2.");
  // Log-linear spacing (arrayops.cpp:60-92 with the library's isclose).
  const double d0 = std::log(x[1] / x[0]);
  for (int i = 0; i + 1 < n; ++i) {
    const double d = std::log(x[i + 1] / x[i]);
    if (!std::isfinite(d) || !(x[i] * x[i + 1] > 0.) ||
        std::fabs(d - d0) > 1.e-8 + 1.e-5 * std::fabs(d0))
      throw_error(TRVG_ERR_INVALID_PARAMETER,
                  "The sample points are not logarithmically spaced.");
  }
  if (extrap < 0 || extrap > 4)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Unsupported extrapolation option: %d.", extrap);
  auto* h = new HankelPlan();
  h->mu = mu;
  h->q = q;
  h->n = n;
  h->pre.assign(x, x + n);
  h->logres = std::log(x[n - 1] / x[0]) / double(n - 1);
  h->extrap = extrap;
  if (extrap != 0) {
    if (n % 2 != 0) {
      delete h;
      throw_error(TRVG_ERR_INVALID_PARAMETER,
                  "The number of sample points must be even for "
                  "extrapolation.");
    }
    h->n_trans = int(std::pow(2., std::ceil(std::log2(extrap_exp * n))));
    if (h->n_trans < n) {
      delete h;
      throw_error(TRVG_ERR_INVALID_PARAMETER,
                  "The sample size expansion factor results in a shrunken "
                  "sample size.");
    }
    h->n_ext = (h->n_trans - n) / 2;
  } else {
    h->n_trans = n;
  }
  if (lowring) {
    h->pivot = lowring_pivot(mu, q, h->logres, kr_c);
  } else {
    if (kr_c <= 0.) {
      delete h;
      throw_error(TRVG_ERR_INVALID_PARAMETER, "Pivot value must be positive.");
    }
    h->pivot = kr_c;
  }
  h->kernel = kernel_coeff(mu, q, h->n_trans, h->logres, h->pivot);
  const double kr = h->pivot * std::exp(-h->logres);
  h->post.resize(n);
  for (int j = 0; j < n; ++j) h->post[j] = kr / h->pre[n - j - 1];
  return h;
}

void hankel_plan_destroy(HankelPlan* h) { delete h; }

// b = the biased transform of `batch` rows of n complex samples (host,
// interleaved re / im; rows assumed real with native extrapolation).
void hankel_transform(Context& ctx, const HankelPlan& h, int batch,
                      const double* a, double* b) {
  if (batch <= 0) return;
  const int N = h.n, Nt = h.n_trans;
  const int64_t total = int64_t(batch) * Nt;
  std::vector<double> host(2 * size_t(total), 0.);
  std::vector<double> row(N), ext(Nt);
  for (int r = 0; r < batch; ++r) {
    double* dst = host.data() + 2 * size_t(r) * Nt;
    const double* src = a + 2 * size_t(r) * N;
    if (h.extrap == 0) {
      for (int j = 0; j < N; ++j) {
        dst[2 * j] = src[2 * j];
        dst[2 * j + 1] = src[2 * j + 1];
      }
      continue;
    }
    for (int j = 0; j < N; ++j) row[j] = src[2 * j];
    if (h.extrap == 4)
      for (int j = 0; j + 1 < N; ++j)
        if (!(row[j] * row[j + 1] > 0.))
          throw_error(TRVG_ERR_INVALID_PARAMETER,
                      "Sign change or zeros detected in the input array.");
    extend_row(row.data(), N, h.n_ext, h.extrap, ext.data());
    for (int j = 0; j < Nt; ++j) dst[2 * j] = ext[j];
  }
  double2* buf = ctx.buf<double2>("hankel.buf", size_t(total));
  double2* u = ctx.buf<double2>("hankel.kernel", size_t(Nt));
  std::vector<double2> uh(Nt);
  for (int m = 0; m < Nt; ++m)
    uh[m] = make_double2(h.kernel[m].real(), h.kernel[m].imag());
  TRVG_CUDA(cudaMemcpyAsync(u, uh.data(), Nt * sizeof(double2),
                            cudaMemcpyHostToDevice, ctx.stream));
  TRVG_CUDA(cudaMemcpyAsync(buf, host.data(), total * sizeof(double2),
                            cudaMemcpyHostToDevice, ctx.stream));
  cufftHandle plan = ctx.plan1d(CUFFT_Z2Z, Nt, batch);
  auto* z = reinterpret_cast<cufftDoubleComplex*>(buf);
  ctx.kbegin("cufft.z2z.hankel");
  TRVG_CUFFT(cufftExecZ2Z(plan, z, z, CUFFT_FORWARD));
  ctx.kend();
  TRVG_KBEGIN(ctx, "hankel_kernel");
  hankel_kernel_mul<<<int(std::min<int64_t>((total + 255) / 256, 152 * 16)),
                      256, 0, ctx.stream>>>(buf, u, Nt, total);
  TRVG_LAUNCHED(ctx);
  ctx.kbegin("cufft.z2z.hankel");
  TRVG_CUFFT(cufftExecZ2Z(plan, z, z, CUFFT_FORWARD));
  ctx.kend();
  ctx.fft_launches += 2;
  TRVG_CUDA(cudaMemcpyAsync(host.data(), buf, total * sizeof(double2),
                            cudaMemcpyDeviceToHost, ctx.stream));
  TRVG_CUDA(cudaStreamSynchronize(ctx.stream));
  for (int r = 0; r < batch; ++r)
    for (int j = 0; j < N; ++j) {
      const size_t s = 2 * (size_t(r) * Nt + h.n_ext + j);
      b[2 * (size_t(r) * N + j)] = host[s];
      b[2 * (size_t(r) * N + j) + 1] = host[s + 1];
    }
}

}  // namespace trvg

// ---- C ABI ------------------------------------------------------------------

struct trvg_hankel {
  trvg::HankelPlan* plan;
};

extern "C" {

int trvg_hankel_create(double mu, double q, const double* x, int n,
                       double kr_c, int lowring, int extrap,
                       double extrap_exp, trvg_hankel** out) {
  TRVG_API_BEGIN
  if (out == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null output handle.");
  *out = nullptr;
  trvg::HankelPlan* p = trvg::hankel_plan_create(
      mu, q, x, n, kr_c, lowring != 0, extrap, extrap_exp);
  *out = new trvg_hankel{p};
  TRVG_API_END
}

int trvg_hankel_info(const trvg_hankel* h, int* n, int* n_trans,
                     double* pivot, double* logres, double* pre_sampts,
                     double* post_sampts) {
  TRVG_API_BEGIN
  if (h == nullptr || h->plan == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null Hankel transform.");
  const trvg::HankelPlan& p = *h->plan;
  if (n) *n = p.n;
  if (n_trans) *n_trans = p.n_trans;
  if (pivot) *pivot = p.pivot;
  if (logres) *logres = p.logres;
  for (int j = 0; j < p.n; ++j) {
    if (pre_sampts) pre_sampts[j] = p.pre[j];
    if (post_sampts) post_sampts[j] = p.post[j];
  }
  TRVG_API_END
}

int trvg_hankel_transform(trvg_context* ctx, const trvg_hankel* h, int batch,
                          const double* a, double* b) {
  TRVG_API_BEGIN
  if (ctx == nullptr || h == nullptr || h->plan == nullptr || a == nullptr ||
      b == nullptr || batch < 0)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Invalid arguments.");
  TRVG_CUDA(cudaSetDevice(ctx->impl.device));
  ctx->impl.begin_call();
  trvg::hankel_transform(ctx->impl, *h->plan, batch, a, b);
  ctx->impl.finish_call();
  TRVG_API_END
}

int trvg_hankel_destroy(trvg_hankel* h) {
  TRVG_API_BEGIN
  if (h != nullptr) {
    trvg::hankel_plan_destroy(h->plan);
    delete h;
  }
  TRVG_API_END
}

}  // extern "C"
