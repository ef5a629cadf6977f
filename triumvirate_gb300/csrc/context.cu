// Context life cycle, device workspace, FFT plan cache, error reporting and
// the host-side maths entry points of the C ABI.
#include <cstdarg>
#include <cstring>
#include <iterator>
#include <string>

#include "internal.h"
#include "maths_host.h"

namespace trvg {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

[[noreturn]] void throw_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw Error(code, buf);
}

void* Context::buffer(const std::string& name, size_t bytes) {
  if (bytes == 0) bytes = 16;
  DeviceBuffer& b = buffers[name];
  if (b.bytes >= bytes) return b.ptr;
  if (b.ptr != nullptr) {
    TRVG_CUDA(cudaStreamSynchronize(stream));
    TRVG_CUDA(cudaFree(b.ptr));
    b.ptr = nullptr;
    b.bytes = 0;
  }
  cudaError_t e = cudaMalloc(&b.ptr, bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    b.ptr = nullptr;
    throw_error(TRVG_ERR_ALLOC,
                "Device allocation of %.3f GiB for '%s' failed: %s",
                double(bytes) / (1024. * 1024. * 1024.), name.c_str(),
                cudaGetErrorString(e));
  }
  b.bytes = bytes;
  return b.ptr;
}

cufftHandle Context::plan(int type, const int n[3], int batch) {
  PlanKey key{type, {n[0], n[1], n[2]}, batch};
  auto it = plans.find(key);
  if (it != plans.end()) return it->second;
  cufftHandle h;
  TRVG_CUFFT(cufftCreate(&h));
  TRVG_CUFFT(cufftSetStream(h, stream));
  long long nn[3] = {n[0], n[1], n[2]};
  size_t work = 0;
  long long odist = 0, idist = 0;
  const long long nfull = nn[0] * nn[1] * nn[2];
  const long long nhalf = nn[0] * nn[1] * (nn[2] / 2 + 1);
  switch (type) {
    case CUFFT_R2C:
    case CUFFT_D2Z:
      idist = nfull;
      odist = nhalf;
      break;
    case CUFFT_C2R:
    case CUFFT_Z2D:
      idist = nhalf;
      odist = nfull;
      break;
    default:
      idist = odist = nfull;
  }
  cufftResult r = cufftMakePlanMany64(h, 3, nn, nullptr, 1, idist, nullptr, 1,
                                      odist, cufftType(type), batch, &work);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(h);
    throw_error(r == CUFFT_ALLOC_FAILED ? TRVG_ERR_ALLOC : TRVG_ERR_CUFFT,
                "cuFFT plan (type %d, %d x %d x %d, batch %d) failed: %d",
                type, n[0], n[1], n[2], batch, int(r));
  }
  plans[key] = h;
  return h;
}

cufftHandle Context::plan1d(int type, int n, int batch) {
  PlanKey key{type, {n, -1, -1}, batch};
  auto it = plans.find(key);
  if (it != plans.end()) return it->second;
  cufftHandle h;
  TRVG_CUFFT(cufftCreate(&h));
  TRVG_CUFFT(cufftSetStream(h, stream));
  long long nn[1] = {n};
  size_t work = 0;
  cufftResult r = cufftMakePlanMany64(h, 1, nn, nullptr, 1, n, nullptr, 1, n,
                                      cufftType(type), batch, &work);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(h);
    throw_error(r == CUFFT_ALLOC_FAILED ? TRVG_ERR_ALLOC : TRVG_ERR_CUFFT,
                "cuFFT 1-d plan (type %d, length %d, batch %d) failed: %d",
                type, n, batch, int(r));
  }
  plans[key] = h;
  return h;
}

cufftHandle Context::plan_xy(int n0, int n1, int nz) {
  PlanKey key{-int(CUFFT_C2C), {n0, n1, nz}, nz};
  auto it = plans.find(key);
  if (it != plans.end()) return it->second;
  cufftHandle h;
  TRVG_CUFFT(cufftCreate(&h));
  TRVG_CUFFT(cufftSetStream(h, stream));
  long long nn[2] = {n0, n1};
  const long long plane = (long long)n0 * n1;
  size_t work = 0;
  cufftResult r = cufftMakePlanMany64(h, 2, nn, nullptr, 1, plane, nullptr,
                                      1, plane, CUFFT_C2C, nz, &work);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(h);
    throw_error(r == CUFFT_ALLOC_FAILED ? TRVG_ERR_ALLOC : TRVG_ERR_CUFFT,
                "cuFFT x-y plan (%d x %d, %d planes) failed: %d", n0, n1, nz,
                int(r));
  }
  plans[key] = h;
  return h;
}

namespace {
cudaEvent_t next_event(Context& c) {
  if (c.events_used == c.event_pool.size()) {
    cudaEvent_t e;
    TRVG_CUDA(cudaEventCreate(&e));
    c.event_pool.push_back(e);
  }
  return c.event_pool[c.events_used++];
}
}  // namespace

cudaStream_t Context::side_stream() {
  if (side == nullptr) {
    int prio = 0;
    if (side_priority != 0) {
      int least = 0, greatest = 0;
      TRVG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      prio = greatest;
    }
    TRVG_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking,
                                           prio));
  }
  if (ev_fork == nullptr) {
    TRVG_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    TRVG_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  }
  return side;
}

void Context::kbegin(const char* name) {
  if (!profiling) return;
  pending = name;
  pending_begin = next_event(*this);
  TRVG_CUDA(cudaEventRecord(pending_begin, stream));
}

void Context::kend() {
  if (!profiling || pending == nullptr) return;
  cudaEvent_t e = next_event(*this);
  TRVG_CUDA(cudaEventRecord(e, stream));
  records.push_back({pending, pending_begin, e});
  pending = nullptr;
}

void Context::begin_call() {
  kernel_launches = 0;
  fft_launches = 0;
  h2d_bytes = 0;
  graph_replays = 0;
  records.clear();
  events_used = 0;
  pending = nullptr;
}

void Context::finish_call() {
  ktimes.clear();
  for (const KernelRecord& r : records) {
    float ms = 0.f;
    TRVG_CUDA(cudaEventElapsedTime(&ms, r.begin, r.end));
    bool found = false;
    for (auto& kv : ktimes) {
      if (kv.first == r.name) {
        kv.second.first += ms;
        kv.second.second += 1;
        found = true;
        break;
      }
    }
    if (!found) ktimes.push_back({r.name, {double(ms), int64_t(1)}});
  }
  records.clear();
}

void Context::set_stream(cudaStream_t s) {
  stream = (s != nullptr) ? s : own_stream;
  for (auto& kv : plans) TRVG_CUFFT(cufftSetStream(kv.second, stream));
}

void Context::release() {
  if (stream) cudaStreamSynchronize(stream);
  for (auto& kv : plans) cufftDestroy(kv.second);
  plans.clear();
  for (auto& kv : buffers)
    if (kv.second.ptr) cudaFree(kv.second.ptr);
  buffers.clear();
  splines.clear();
  stats_plans.clear();
  mode_counts.clear();
}

void destroy_events(Context& c) {
  for (cudaEvent_t e : c.event_pool) cudaEventDestroy(e);
  c.event_pool.clear();
  c.events_used = 0;
}

void Context::log(int level, const char* fmt, ...) const {
  if (verbose < level) return;
  va_list ap;
  va_start(ap, fmt);
  std::fprintf(stderr, "[trvg] ");
  std::vfprintf(stderr, fmt, ap);
  std::fprintf(stderr, "\n");
  va_end(ap);
}

}  // namespace trvg

extern "C" {

const char* trvg_last_error(void) { return trvg::last_error(); }

const char* trvg_version(void) { return "triumvirate-gb300 0.1.0 (sm_103a)"; }

int trvg_context_create(int device, trvg_context** ctx) {
  TRVG_API_BEGIN
  if (ctx == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null context pointer.");
  int ndev = 0;
  TRVG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER,
                      "CUDA device %d unavailable (%d devices).", device,
                      ndev);
  TRVG_CUDA(cudaSetDevice(device));
  auto* c = new trvg_context();
  c->impl.device = device;
  TRVG_CUDA(cudaStreamCreateWithFlags(&c->impl.own_stream,
                                      cudaStreamNonBlocking));
  c->impl.stream = c->impl.own_stream;
  TRVG_CUDA(cudaEventCreate(&c->impl.ev_start));
  TRVG_CUDA(cudaEventCreate(&c->impl.ev_h2d));
  TRVG_CUDA(cudaEventCreate(&c->impl.ev_stop));
  *ctx = c;
  TRVG_API_END
}

int trvg_context_destroy(trvg_context* ctx) {
  TRVG_API_BEGIN
  if (ctx == nullptr) return TRVG_OK;
  cudaSetDevice(ctx->impl.device);
  ctx->impl.release();
  if (ctx->impl.ev_start) cudaEventDestroy(ctx->impl.ev_start);
  if (ctx->impl.ev_h2d) cudaEventDestroy(ctx->impl.ev_h2d);
  if (ctx->impl.ev_stop) cudaEventDestroy(ctx->impl.ev_stop);
  if (ctx->impl.ev_fork) cudaEventDestroy(ctx->impl.ev_fork);
  if (ctx->impl.ev_join) cudaEventDestroy(ctx->impl.ev_join);
  if (ctx->impl.side) cudaStreamDestroy(ctx->impl.side);
  trvg::destroy_events(ctx->impl);
  if (ctx->impl.own_stream) cudaStreamDestroy(ctx->impl.own_stream);
  delete ctx;
  TRVG_API_END
}

int trvg_release_workspace(trvg_context* ctx) {
  TRVG_API_BEGIN
  if (ctx == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null context.");
  TRVG_CUDA(cudaSetDevice(ctx->impl.device));
  ctx->impl.release();
  TRVG_API_END
}

int trvg_get_stats(const trvg_context* ctx, trvg_stats* out) {
  TRVG_API_BEGIN
  if (ctx == nullptr || out == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  const trvg::Context& c = ctx->impl;
  out->ms_total = c.ms_total;
  out->ms_h2d = c.ms_h2d;
  out->h2d_bytes = c.h2d_bytes;
  out->kernel_launches = c.kernel_launches;
  out->fft_launches = c.fft_launches;
  for (int i = 0; i < 3; ++i) out->pruned_grid[i] = c.pruned_grid[i];
  out->graph_replays = c.graph_replays;
  TRVG_API_END
}

int trvg_context_set_stream(trvg_context* ctx, void* stream) {
  TRVG_API_BEGIN
  if (ctx == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null context.");
  TRVG_CUDA(cudaSetDevice(ctx->impl.device));
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  ctx->impl.set_stream(static_cast<cudaStream_t>(stream));
  TRVG_API_END
}

int trvg_set_option(trvg_context* ctx, const char* key, int64_t value) {
  TRVG_API_BEGIN
  if (ctx == nullptr || key == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  const std::string k(key);
  if (k == "full_mesh_shells") {
    ctx->impl.full_mesh_shells = value != 0;
  } else if (k == "profiling") {
    ctx->impl.profiling = value != 0;
  } else if (k == "shotnoise_fp64") {
    ctx->impl.shotnoise_fp64 = value != 0;
  } else if (k == "shell_fields_fp64") {
    ctx->impl.shell_fields_fp64 = value != 0;
  } else if (k == "sort_catalogue") {
    ctx->impl.sort_catalogue = value != 0;
  } else if (k == "ff_transforms") {
    if (value < 0 || value > 2)
      trvg::throw_error(TRVG_ERR_INVALID_PARAMETER,
                        "ff_transforms must be 0, 1 or 2.");
    ctx->impl.ff_transforms = int(value);
  } else if (k == "gram_per_pair") {
    ctx->impl.gram_per_pair = value != 0;
  } else if (k == "graph_batch") {
    ctx->impl.graph_batch = value != 0;
  } else if (k == "autotune") {
    ctx->impl.autotune = value != 0;
    if (value == 0) ctx->impl.tuned.clear();
  } else if (k == "overlap") {
    ctx->impl.overlap = value != 0;
  } else if (k == "side_priority") {
    if (value < 0 || value > 1)
      trvg::throw_error(TRVG_ERR_INVALID_PARAMETER,
                        "side_priority must be 0 or 1.");
    if (ctx->impl.side != nullptr && ctx->impl.side_priority != int(value)) {
      TRVG_CUDA(cudaStreamSynchronize(ctx->impl.side));
      TRVG_CUDA(cudaStreamDestroy(ctx->impl.side));
      ctx->impl.side = nullptr;
    }
    ctx->impl.side_priority = int(value);
  } else if (k == "xi_octant") {
    ctx->impl.xi_octant = value != 0;
  } else if (k == "fused_ylm") {
    ctx->impl.fused_ylm = value != 0;
  } else if (k == "mesh_comp") {
    if (value < 0 || value > 2)
      trvg::throw_error(TRVG_ERR_INVALID_PARAMETER,
                        "mesh_comp must be 0, 1 or 2.");
    ctx->impl.mesh_comp = int(value);
  } else if (k == "mesh_renorm") {
    ctx->impl.mesh_renorm = value != 0;
  } else if (k == "assign_path") {
    if (value < 0 || value > 2)
      trvg::throw_error(TRVG_ERR_INVALID_PARAMETER,
                        "assign_path must be 0, 1 or 2.");
    ctx->impl.assign_path = int(value);
  } else {
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Unknown option '%s'.",
                      key);
  }
  TRVG_API_END
}

int trvg_kernel_time_count(const trvg_context* ctx, int* count) {
  TRVG_API_BEGIN
  if (ctx == nullptr || count == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  *count = int(ctx->impl.ktimes.size());
  TRVG_API_END
}

int trvg_kernel_time_get(const trvg_context* ctx, int index, char* name,
                         int name_len, double* ms, int64_t* launches) {
  TRVG_API_BEGIN
  if (ctx == nullptr || name == nullptr || name_len <= 0 || ms == nullptr ||
      launches == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  const auto& kt = ctx->impl.ktimes;
  if (index < 0 || index >= int(kt.size()))
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Index out of range.");
  std::snprintf(name, size_t(name_len), "%s", kt[index].first.c_str());
  *ms = kt[index].second.first;
  *launches = kt[index].second.second;
  TRVG_API_END
}

int trvg_tuned_count(const trvg_context* ctx, int* count) {
  TRVG_API_BEGIN
  if (ctx == nullptr || count == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  *count = int(ctx->impl.tuned.size());
  TRVG_API_END
}

int trvg_tuned_get(const trvg_context* ctx, int index, char* key,
                   int key_len, int64_t* value) {
  TRVG_API_BEGIN
  if (ctx == nullptr || key == nullptr || key_len <= 0 || value == nullptr)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  const auto& t = ctx->impl.tuned;
  if (index < 0 || index >= int(t.size()))
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Index out of range.");
  auto it = t.begin();
  std::advance(it, index);
  std::snprintf(key, size_t(key_len), "%s", it->first.c_str());
  *value = it->second;
  TRVG_API_END
}

double trvg_wigner_3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  return trvg::wigner_3j(j1, j2, j3, m1, m2, m3);
}

double trvg_sph_bessel(int ell, double x) { return trvg::sph_bessel(ell, x); }

int trvg_sph_bessel_spline(int ell, const double* x, int64_t n,
                           double* out) {
  TRVG_API_BEGIN
  if (ell < 0 || (n > 0 && (x == nullptr || out == nullptr)))
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Invalid arguments.");
  trvg::SplineHost s(ell);
  trvg::SplineTable t =
      s.table(s.y.data(), s.b.data(), s.c.data(), s.d.data());
  for (int64_t i = 0; i < n; ++i) {
    if (!(x[i] >= 0.))
      trvg::throw_error(TRVG_ERR_INVALID_PARAMETER,
                        "Spline argument must be non-negative.");
    out[i] = trvg::spline_eval(t, x[i]);
  }
  TRVG_API_END
}

int trvg_reduced_ylm(int ell, int m, const double* v3, int64_t n,
                     double* out_complex) {
  TRVG_API_BEGIN
  if (ell < 0 || m < -ell || m > ell ||
      (n > 0 && (v3 == nullptr || out_complex == nullptr)))
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Invalid arguments.");
  for (int64_t i = 0; i < n; ++i) {
    trvg::cd y = trvg::reduced_ylm(ell, m, v3[3 * i], v3[3 * i + 1],
                                   v3[3 * i + 2]);
    out_complex[2 * i] = y.re;
    out_complex[2 * i + 1] = y.im;
  }
  TRVG_API_END
}

int trvg_data_vector_dim(int shape, int num_bins, int idx_bin, int* dim) {
  TRVG_API_BEGIN
  if (dim == nullptr || num_bins <= 0)
    trvg::throw_error(TRVG_ERR_INVALID_PARAMETER, "Invalid arguments.");
  switch (shape) {
    case TRVG_SHAPE_DIAG:
    case TRVG_SHAPE_ROW:
      *dim = num_bins;
      break;
    case TRVG_SHAPE_OFFDIAG:
      *dim = num_bins - (idx_bin < 0 ? -idx_bin : idx_bin);
      break;
    case TRVG_SHAPE_FULL:
      *dim = num_bins * num_bins;
      break;
    case TRVG_SHAPE_TRIU:
      *dim = num_bins * (num_bins + 1) / 2;
      break;
    default:
      trvg::throw_error(TRVG_ERR_INVALID_PARAMETER,
                        "Three-point statistic form is not recognised: %d.",
                        shape);
  }
  TRVG_API_END
}

}  // extern "C"
