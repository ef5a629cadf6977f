// Device-resident particle catalogues: ingestion from text files and the
// O(N) preparation steps on the GPU (particles.cpp:94-510, 570-888;
// catalogue.py:437-676).
//
// A catalogue file is parsed on the host by a multi-threaded reader
// (std::from_chars, correctly rounded like the library's stream
// extraction) straight into the columns x, y, z, nz, ws, wc, which are
// copied to device memory once.  Everything after that runs on the
// device: the overall weight w = ws wc, the totals, the coordinate
// extents, offsets, centring and padding in a box, periodic wrapping and
// the lines of sight.  Element-wise steps use the library's operation
// order without contraction, so coordinates come out bit for bit as the
// reference's numpy code makes them.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"
#include "kernels.h"

struct trvg_dcat {
  int64_t n = 0;
  double* col[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double* w = nullptr;  // ws * wc
  double* los[3] = {nullptr, nullptr, nullptr};
  std::string source;
};

namespace trvg {

namespace {

enum { kX = 0, kY, kZ, kNZ, kWS, kWC };
const char* const kNames[6] = {"x", "y", "z", "nz", "ws", "wc"};

int grid_for(int64_t work) {
  int64_t g = (work + 255) / 256;
  return int(std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16)));
}

__global__ void product_kernel(int64_t n, const double* a, const double* b,
                               double* out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = __dmul_rn(a[i], b[i]);
}

__global__ void fill_kernel(int64_t n, double v, double* out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = v;
}

// Order-preserving integer image of a double (for atomic min / max).
__device__ __forceinline__ unsigned long long ordered(double v) {
  const unsigned long long b = __double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double from_ordered(unsigned long long u) {
  unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
  double v;
  std::memcpy(&v, &b, sizeof(v));
  return v;
}

// ext[2 a] = min, ext[2 a + 1] = max of axis a (ordered images).
__global__ void extents_kernel(int64_t n, const double* x, const double* y,
                               const double* z, unsigned long long* ext) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  const double* c[3] = {x, y, z};
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    for (int a = 0; a < 3; ++a) {
      const unsigned long long o = ordered(c[a][i]);
      lo[a] = o < lo[a] ? o : lo[a];
      hi[a] = o > hi[a] ? o : hi[a];
    }
  for (int a = 0; a < 3; ++a) {
    for (int s = 16; s > 0; s >>= 1) {
      const unsigned long long l = __shfl_down_sync(0xffffffffu, lo[a], s);
      const unsigned long long h = __shfl_down_sync(0xffffffffu, hi[a], s);
      lo[a] = l < lo[a] ? l : lo[a];
      hi[a] = h > hi[a] ? h : hi[a];
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(ext + 2 * a, lo[a]);
      atomicMax(ext + 2 * a + 1, hi[a]);
    }
  }
}

// Deterministic sums over the particles: kSumBlocks blocks each reduce a
// fixed stride in a fixed order, then one thread adds the partial sums in
// order (the same bits on every run).  Mode 0 sums (w, ws)
// (calc_total_weights, particles.cpp:570-602); modes 2 and 3 sum
// ws nz^(m-1) wc^m (twopt.cpp:56-99, threept.cpp:96-136) and count the
// particles with nz != 0.
constexpr int kSumBlocks = 152 * 2;

struct SumCols {
  const double* w;
  const double* ws;
  const double* nz;
  const double* wc;
  int mode;
};

__device__ __forceinline__ void sum_terms(const SumCols& c, int64_t i,
                                          double& a, double& b) {
  if (c.mode == 0) {
    a = c.w[i];
    b = c.ws[i];
    return;
  }
  const double nz = c.nz[i], wc = c.wc[i];
  if (c.mode == 2)
    a = __dmul_rn(__dmul_rn(c.ws[i], nz), __dmul_rn(wc, wc));
  else
    a = __dmul_rn(__dmul_rn(c.ws[i], __dmul_rn(nz, nz)), pow(wc, 3.));
  b = nz != 0. ? 1. : 0.;
}

__global__ void __launch_bounds__(256)
sums_kernel(int64_t n, SumCols cols, double* part) {
  __shared__ double sh[2][8];
  double a = 0., b = 0.;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    double ta, tb;
    sum_terms(cols, i, ta, tb);
    a += ta;
    b += tb;
  }
  for (int s = 16; s > 0; s >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, s);
    b += __shfl_down_sync(0xffffffffu, b, s);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = a;
    sh[1][threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0., tb = 0.;
    for (int k = 0; k < int(blockDim.x >> 5); ++k) {
      ta += sh[0][k];
      tb += sh[1][k];
    }
    part[2 * blockIdx.x] = ta;
    part[2 * blockIdx.x + 1] = tb;
  }
}

__global__ void sums_final_kernel(const double* part, int nblocks,
                                  double* out) {
  if (threadIdx.x == 0) {
    double a = 0., b = 0.;
    for (int k = 0; k < nblocks; ++k) {
      a += part[2 * k];
      b += part[2 * k + 1];
    }
    out[0] = a;
    out[1] = b;
  }
}

// x -= d (ParticleCatalogue::offset_coords).
__global__ void offset_kernel(int64_t n, double* x, double* y, double* z,
                              double dx, double dy, double dz) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    x[i] = __dsub_rn(x[i], dx);
    y[i] = __dsub_rn(y[i], dy);
    z[i] = __dsub_rn(z[i], dz);
  }
}

// ((x + L/2) - mid) mod L with numpy's float remainder (the divisor's
// sign; catalogue.py:648-676).
__device__ __forceinline__ double wrap_box(double x, double half, double mid,
                                           double L) {
  const double t = __dsub_rn(__dadd_rn(x, half), mid);
  double r = fmod(t, L);
  if (r != 0.) {
    if ((L < 0.) != (r < 0.)) r = __dadd_rn(r, L);
  } else {
    r = copysign(0., L);
  }
  return r;
}

__global__ void periodise_kernel(int64_t n, double* x, double* y, double* z,
                                 double3 L, double3 half, double3 mid) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    x[i] = wrap_box(x[i], half.x, mid.x, L.x);
    y[i] = wrap_box(y[i], half.y, mid.y, L.y);
    z[i] = wrap_box(z[i], half.z, mid.z, L.z);
  }
}

// Coordinates at or beyond L become fmod(x, L), negative ones
// fmod(x, L) + L (offset_coords_for_periodicity, particles.cpp:678-699).
__device__ __forceinline__ double wrap_fmod(double x, double L) {
  if (x >= L) return fmod(x, L);
  if (x < 0.) return __dadd_rn(fmod(x, L), L);
  return x;
}

__global__ void wrap_kernel(int64_t n, double* x, double* y, double* z,
                            double3 L) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    x[i] = wrap_fmod(x[i], L.x);
    y[i] = wrap_fmod(y[i], L.y);
    z[i] = wrap_fmod(z[i], L.z);
  }
}

// Unit end-point lines of sight x / |x| (|x| = 0 -> 1; catalogue.py:437).
__global__ void los_kernel(int64_t n, const double* x, const double* y,
                           const double* z, double* lx, double* ly,
                           double* lz) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(x[i], x[i]),
                                         __dmul_rn(y[i], y[i])),
                               __dmul_rn(z[i], z[i]));
    double r = __dsqrt_rn(s);
    if (r == 0.) r = 1.;
    lx[i] = __ddiv_rn(x[i], r);
    ly[i] = __ddiv_rn(y[i], r);
    lz[i] = __ddiv_rn(z[i], r);
  }
}

template <typename Kernel, typename... Args>
void run(Context& ctx, const char* name, int64_t n, Kernel kernel,
         Args... args) {
  if (n <= 0) return;
  TRVG_KBEGIN(ctx, name);
  kernel<<<grid_for(n), 256, 0, ctx.stream>>>(args...);
  TRVG_LAUNCHED(ctx);
}

double* dalloc(int64_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, size_t(std::max<int64_t>(n, 1)) * sizeof(double)) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    throw_error(TRVG_ERR_ALLOC, "Device allocation for %lld particles failed.",
                (long long)n);
  }
  return static_cast<double*>(p);
}

void dfree(trvg_dcat* c) {
  for (double*& p : c->col) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  if (c->w) cudaFree(c->w);
  c->w = nullptr;
  for (double*& p : c->los) {
    if (p) cudaFree(p);
    p = nullptr;
  }
}

bool ends_with(const std::string& s, const std::string& e) {
  return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}

// Sub-file paths joined by "::" (particles.cpp:160-162; monitor.cpp:59-85).
std::vector<std::string> split_paths(const std::string& s) {
  std::vector<std::string> out;
  if (s.empty()) return out;
  size_t b = 0, e;
  while ((e = s.find("::", b)) != std::string::npos) {
    out.push_back(s.substr(b, e - b));
    b = e + 2;
  }
  if (b < s.size()) out.push_back(s.substr(b));
  return out;
}

// Whole file in one read.
std::string slurp(const std::string& path) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (f == nullptr)
    throw_error(TRVG_ERR_INVALID_DATA, "Failed to open file: %s",
                path.c_str());
  std::string text;
  char chunk[1 << 16];
  if (std::fseek(f, 0, SEEK_END) == 0) {
    const long size = std::ftell(f);
    if (size > 0) text.reserve(size_t(size) + 1);
    std::fseek(f, 0, SEEK_SET);
  }
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0)
    text.append(chunk, got);
  std::fclose(f);
  return text;
}

inline bool is_blank(char c) {
  return c == ' ' || c == '\t' || c == '\v' || c == '\f' || c == '\r';
}

// Calls row(begin, end) for every line of text[lo, hi) that is neither
// empty nor a comment ('#' first); lines start in [lo, hi).
template <typename F>
void for_rows(const std::string& text, size_t lo, size_t hi, F&& row) {
  const char* base = text.data();
  size_t pos = lo;
  while (pos < hi) {
    const void* nl = std::memchr(base + pos, '\n', text.size() - pos);
    const size_t end = nl ? size_t(static_cast<const char*>(nl) - base)
                          : text.size();
    size_t stop = end;
    if (stop > pos && base[stop - 1] == '\r') --stop;
    if (stop > pos && base[pos] != '#') row(base + pos, base + stop);
    pos = end + 1;
  }
}

// Rows of whitespace-separated text files (particles.cpp:383-497): lines
// that are empty or start with '#' are skipped, and field k takes row
// entry index_of[k] (-1: absent).  Each file is split into one chunk per
// host thread at line boundaries; a counting pass and a prefix sum give
// every chunk its first row, and a second pass parses the chunk into the
// columns with std::from_chars, which rounds correctly as stream
// extraction does.
void parse_text(const std::vector<std::string>& paths, const int index_of[6],
                std::vector<std::vector<double>>& cols) {
  int need = 0;
  for (int k = 0; k < 6; ++k) need = std::max(need, index_of[k] + 1);
  const int nthr = int(std::max(1u, std::min(32u,
                                             std::thread::hardware_concurrency())));
  std::vector<std::string> texts;
  std::vector<std::vector<size_t>> bounds;
  std::vector<std::vector<int64_t>> first;
  int64_t n = 0;
  for (const std::string& path : paths) {
    texts.push_back(slurp(path));
    const std::string& text = texts.back();
    std::vector<size_t> b(nthr + 1, text.size());
    b[0] = 0;
    for (int t = 1; t < nthr; ++t) {
      size_t p = text.size() * size_t(t) / size_t(nthr);
      const void* nl = p < text.size()
                           ? std::memchr(text.data() + p, '\n', text.size() - p)
                           : nullptr;
      b[t] = nl ? size_t(static_cast<const char*>(nl) - text.data()) + 1
                : text.size();
      b[t] = std::max(b[t], b[t - 1]);
    }
    std::vector<int64_t> count(nthr, 0);
    std::vector<std::thread> pool;
    for (int t = 0; t < nthr; ++t)
      pool.emplace_back([&, t] {
        for_rows(text, b[t], b[t + 1],
                 [&](const char*, const char*) { ++count[t]; });
      });
    for (auto& th : pool) th.join();
    std::vector<int64_t> f(nthr + 1, n);
    for (int t = 0; t < nthr; ++t) f[t + 1] = f[t] + count[t];
    n = f[nthr];
    bounds.push_back(std::move(b));
    first.push_back(std::move(f));
  }
  for (int k = 0; k < 6; ++k)
    if (index_of[k] >= 0) cols[k].assign(size_t(n), 0.);
  std::vector<int64_t> bad(nthr, -1);
  for (size_t fi = 0; fi < texts.size(); ++fi) {
    std::vector<std::thread> pool;
    for (int t = 0; t < nthr; ++t)
      pool.emplace_back([&, t, fi] {
        int64_t i = first[fi][t];
        double row[6];
        for_rows(texts[fi], bounds[fi][t], bounds[fi][t + 1],
                 [&](const char* p, const char* e) {
                   int got = 0;
                   double v = 0.;
                   while (p < e && got < need) {
                     while (p < e && is_blank(*p)) ++p;
                     if (p >= e) break;
                     const char* q = (*p == '+') ? p + 1 : p;
                     const auto r = std::from_chars(q, e, v);
                     if (r.ec != std::errc() &&
                         r.ec != std::errc::result_out_of_range)
                       break;
                     for (int k = 0; k < 6; ++k)
                       if (index_of[k] == got) row[k] = v;
                     ++got;
                     p = r.ptr;
                   }
                   if (got < need) {
                     if (bad[t] < 0) bad[t] = i;
                   } else {
                     for (int k = 0; k < 6; ++k)
                       if (index_of[k] >= 0) cols[k][size_t(i)] = row[k];
                   }
                   ++i;
                 });
      });
    for (auto& th : pool) th.join();
    texts[fi].clear();
    texts[fi].shrink_to_fit();
  }
  for (int t = 0; t < nthr; ++t)
    if (bad[t] >= 0)
      throw_error(TRVG_ERR_INVALID_DATA,
                  "Catalogue row %lld has fewer than %d readable entries.",
                  (long long)bad[t], need);
}

void update_weights(Context& ctx, trvg_dcat* c) {
  run(ctx, "catalogue_kernel", c->n, product_kernel, c->n,
      (const double*)c->col[kWS], (const double*)c->col[kWC], c->w);
}

// Columns from host arrays; absent ones take the reference's defaults
// (nz: ntotal / volume, or 0; ws = wc = 1), and w = ws wc.
void upload_columns(Context& ctx, trvg_dcat* c, const double* const host[6],
                    double nz_default) {
  for (int k = 0; k < 6; ++k) {
    c->col[k] = dalloc(c->n);
    if (host[k] != nullptr) {
      if (c->n > 0)
        TRVG_CUDA(cudaMemcpyAsync(c->col[k], host[k],
                                  size_t(c->n) * sizeof(double),
                                  cudaMemcpyHostToDevice, ctx.stream));
    } else {
      const double v = (k == kNZ) ? nz_default : (k >= kWS ? 1. : 0.);
      run(ctx, "catalogue_kernel", c->n, fill_kernel, c->n, v, c->col[k]);
    }
  }
  c->w = dalloc(c->n);
  update_weights(ctx, c);
  TRVG_CUDA(cudaStreamSynchronize(ctx.stream));
}

void extents(Context& ctx, const trvg_dcat* c, double lo[3], double hi[3]) {
  if (c->n == 0) {
    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = 0.;
    return;
  }
  unsigned long long* d = ctx.buf<unsigned long long>("dcat.ext", 6);
  const unsigned long long init[6] = {~0ull, 0, ~0ull, 0, ~0ull, 0};
  TRVG_CUDA(cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice,
                            ctx.stream));
  run(ctx, "catalogue_kernel", c->n, extents_kernel, c->n,
      (const double*)c->col[kX], (const double*)c->col[kY],
      (const double*)c->col[kZ], d);
  unsigned long long h[6];
  TRVG_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost,
                            ctx.stream));
  TRVG_CUDA(cudaStreamSynchronize(ctx.stream));
  for (int a = 0; a < 3; ++a) {
    lo[a] = from_ordered(h[2 * a]);
    hi[a] = from_ordered(h[2 * a + 1]);
  }
}

void sums(Context& ctx, const trvg_dcat* c, int mode, double out[2]) {
  out[0] = out[1] = 0.;
  if (c->n == 0) return;
  double* part = ctx.buf<double>("dcat.sums", 2 * kSumBlocks + 2);
  const SumCols cols{c->w, c->col[kWS], c->col[kNZ], c->col[kWC], mode};
  TRVG_KBEGIN(ctx, "catalogue_kernel");
  sums_kernel<<<kSumBlocks, 256, 0, ctx.stream>>>(c->n, cols, part);
  TRVG_LAUNCHED(ctx);
  TRVG_KBEGIN(ctx, "catalogue_kernel");
  sums_final_kernel<<<1, 32, 0, ctx.stream>>>(part, kSumBlocks,
                                              part + 2 * kSumBlocks);
  TRVG_LAUNCHED(ctx);
  TRVG_CUDA(cudaMemcpyAsync(out, part + 2 * kSumBlocks, 2 * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx.stream));
  TRVG_CUDA(cudaStreamSynchronize(ctx.stream));
}

// Device column by name (nullptr for an unknown name).
double** column_slot(trvg_dcat* c, const char* column) {
  for (int k = 0; k < 6; ++k)
    if (std::strcmp(column, kNames[k]) == 0) return &c->col[k];
  if (std::strcmp(column, "w") == 0) return &c->w;
  if (std::strcmp(column, "los_x") == 0) return &c->los[0];
  if (std::strcmp(column, "los_y") == 0) return &c->los[1];
  if (std::strcmp(column, "los_z") == 0) return &c->los[2];
  return nullptr;
}

void offset(Context& ctx, trvg_dcat* c, const double d[3]) {
  run(ctx, "catalogue_kernel", c->n, offset_kernel, c->n, c->col[kX],
      c->col[kY], c->col[kZ], d[0], d[1], d[2]);
}

trvg_dcat* adopt(Context& ctx, int64_t n, const std::string& source,
                 const double* const host[6], double nz_default) {
  auto* c = new trvg_dcat();
  c->n = n;
  c->source = source;
  try {
    upload_columns(ctx, c, host, nz_default);
  } catch (...) {
    dfree(c);
    delete c;
    throw;
  }
  return c;
}

void check(trvg_context* ctx, const void* c) {
  if (ctx == nullptr || c == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  TRVG_CUDA(cudaSetDevice(ctx->impl.device));
}

}  // namespace

}  // namespace trvg

using namespace trvg;

extern "C" {

int trvg_dcat_read_text(trvg_context* ctx, const char* path,
                        const char* columns, double volume, trvg_dcat** out) {
  TRVG_API_BEGIN
  check(ctx, out);
  *out = nullptr;
  if (path == nullptr || columns == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  const std::string fpath(path);
  if (ends_with(fpath, ".h5") || ends_with(fpath, ".hdf5"))
    throw_error(TRVG_ERR_INVALID_DATA,
                "HDF5 file format is not supported in this build: %s", path);
  // Field k takes the first column named kNames[k] (particles.cpp:136-156).
  std::vector<std::string> names;
  std::stringstream cs(columns);
  std::string name;
  while (std::getline(cs, name, ',')) names.push_back(name);
  int index_of[6];
  for (int k = 0; k < 6; ++k) {
    const auto it = std::find(names.begin(), names.end(), kNames[k]);
    index_of[k] = it == names.end() ? -1 : int(it - names.begin());
  }
  if (index_of[kX] < 0 || index_of[kY] < 0 || index_of[kZ] < 0)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Catalogue columns must include 'x', 'y' and 'z'.");
  std::vector<std::vector<double>> cols(6);
  parse_text(split_paths(fpath), index_of, cols);
  const int64_t n = int64_t(cols[kX].size());
  const double* host[6];
  for (int k = 0; k < 6; ++k)
    host[k] = index_of[k] >= 0 ? cols[k].data() : nullptr;
  const double nz_default = volume > 0. ? double(n) / volume : 0.;
  *out = adopt(ctx->impl, n, "extfile:" + fpath, host, nz_default);
  TRVG_API_END
}

int trvg_dcat_from_host(trvg_context* ctx, int64_t n, const double* x,
                        const double* y, const double* z, const double* nz,
                        const double* ws, const double* wc, trvg_dcat** out) {
  TRVG_API_BEGIN
  check(ctx, out);
  *out = nullptr;
  if (n < 0 || (n > 0 && (x == nullptr || y == nullptr || z == nullptr)))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Invalid particle arrays.");
  const double* host[6] = {x, y, z, nz, ws, wc};
  *out = adopt(ctx->impl, n, "extdata", host, 0.);
  TRVG_API_END
}

int trvg_dcat_concat(trvg_context* ctx, const trvg_dcat* const* cats,
                     int count, trvg_dcat** out) {
  TRVG_API_BEGIN
  check(ctx, out);
  *out = nullptr;
  if (count < 0 || (count > 0 && cats == nullptr))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Invalid catalogue list.");
  int64_t n = 0;
  bool los = count > 0;
  for (int i = 0; i < count; ++i) {
    if (cats[i] == nullptr)
      throw_error(TRVG_ERR_INVALID_PARAMETER, "Null catalogue %d.", i);
    n += cats[i]->n;
    los = los && cats[i]->los[0] != nullptr;
  }
  auto* c = new trvg_dcat();
  c->n = n;
  c->source = "concatenated";
  try {
    for (int k = 0; k < 6; ++k) c->col[k] = dalloc(n);
    c->w = dalloc(n);
    if (los)
      for (double*& p : c->los) p = dalloc(n);
    int64_t at = 0;
    for (int i = 0; i < count; ++i) {
      const trvg_dcat* s = cats[i];
      const size_t bytes = size_t(s->n) * sizeof(double);
      if (bytes == 0) continue;
      for (int k = 0; k < 6; ++k)
        TRVG_CUDA(cudaMemcpyAsync(c->col[k] + at, s->col[k], bytes,
                                  cudaMemcpyDeviceToDevice, ctx->impl.stream));
      TRVG_CUDA(cudaMemcpyAsync(c->w + at, s->w, bytes,
                                cudaMemcpyDeviceToDevice, ctx->impl.stream));
      if (los)
        for (int a = 0; a < 3; ++a)
          TRVG_CUDA(cudaMemcpyAsync(c->los[a] + at, s->los[a], bytes,
                                    cudaMemcpyDeviceToDevice,
                                    ctx->impl.stream));
      at += s->n;
    }
    TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  } catch (...) {
    dfree(c);
    delete c;
    throw;
  }
  *out = c;
  TRVG_API_END
}

int trvg_dcat_info(trvg_context* ctx, const trvg_dcat* c, int64_t* n,
                   double* wtotal, double* wstotal, double* pos_min,
                   double* pos_max) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (n) *n = c->n;
  if (wtotal || wstotal) {
    double t[2];
    sums(ctx->impl, c, 0, t);
    if (wtotal) *wtotal = t[0];
    if (wstotal) *wstotal = t[1];
  }
  if (pos_min || pos_max) {
    double lo[3], hi[3];
    extents(ctx->impl, c, lo, hi);
    for (int a = 0; a < 3; ++a) {
      if (pos_min) pos_min[a] = lo[a];
      if (pos_max) pos_max[a] = hi[a];
    }
  }
  TRVG_API_END
}

int trvg_dcat_offset(trvg_context* ctx, trvg_dcat* c, const double* dpos) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (dpos == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  offset(ctx->impl, c, dpos);
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_centre(trvg_context* ctx, trvg_dcat* c, trvg_dcat* ref,
                     const double* boxsize) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (boxsize == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  // The mid-point of the reference's extents moves to the box centre, and
  // the same offset applies to both catalogues (particles.cpp:701-778;
  // catalogue.py:490-545).
  double lo[3], hi[3], d[3];
  extents(ctx->impl, ref ? ref : c, lo, hi);
  for (int a = 0; a < 3; ++a) d[a] = (lo[a] + hi[a]) / 2. - boxsize[a] / 2.;
  offset(ctx->impl, c, d);
  if (ref != nullptr) offset(ctx->impl, ref, d);
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_pad(trvg_context* ctx, trvg_dcat* c, trvg_dcat* ref,
                  const double* boxsize, const double* boxsize_pad,
                  const double* ngrid, const double* ngrid_pad) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (boxsize == nullptr ||
      (boxsize_pad == nullptr) == (ngrid_pad == nullptr) ||
      (ngrid_pad != nullptr && ngrid == nullptr))
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Give exactly one of the box-size and grid paddings.");
  // The reference's minimum coordinates move to the padding, and the same
  // offset applies to both catalogues (particles.cpp:780-888, whose
  // association this keeps; catalogue.py:547-646 divides first).
  double lo[3], hi[3], d[3];
  extents(ctx->impl, ref ? ref : c, lo, hi);
  for (int a = 0; a < 3; ++a) {
    d[a] = lo[a];
    if (boxsize_pad) d[a] -= boxsize_pad[a] * boxsize[a];
    if (ngrid_pad) d[a] -= ngrid_pad[a] * boxsize[a] / ngrid[a];
  }
  offset(ctx->impl, c, d);
  if (ref != nullptr) offset(ctx->impl, ref, d);
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_periodise(trvg_context* ctx, trvg_dcat* c,
                        const double* boxsize) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (boxsize == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  double lo[3], hi[3];
  extents(ctx->impl, c, lo, hi);
  const double3 L = make_double3(boxsize[0], boxsize[1], boxsize[2]);
  const double3 half =
      make_double3(boxsize[0] / 2., boxsize[1] / 2., boxsize[2] / 2.);
  const double3 mid = make_double3((hi[0] + lo[0]) / 2., (hi[1] + lo[1]) / 2.,
                                   (hi[2] + lo[2]) / 2.);
  run(ctx->impl, "catalogue_kernel", c->n, periodise_kernel, c->n, c->col[kX],
      c->col[kY], c->col[kZ], L, half, mid);
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_wrap_box(trvg_context* ctx, trvg_dcat* c,
                       const double* boxsize) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (boxsize == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  run(ctx->impl, "catalogue_kernel", c->n, wrap_kernel, c->n, c->col[kX],
      c->col[kY], c->col[kZ], make_double3(boxsize[0], boxsize[1], boxsize[2]));
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_compute_los(trvg_context* ctx, trvg_dcat* c) {
  TRVG_API_BEGIN
  check(ctx, c);
  for (double*& p : c->los)
    if (p == nullptr) p = dalloc(c->n);
  run(ctx->impl, "catalogue_kernel", c->n, los_kernel, c->n,
      (const double*)c->col[kX], (const double*)c->col[kY],
      (const double*)c->col[kZ], c->los[0], c->los[1], c->los[2]);
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_set_column(trvg_context* ctx, trvg_dcat* c, const char* column,
                         double value) {
  TRVG_API_BEGIN
  check(ctx, c);
  int k = -1;
  for (int i = kNZ; i <= kWC; ++i)
    if (column != nullptr && std::strcmp(column, kNames[i]) == 0) k = i;
  if (k < 0)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Only 'nz', 'ws' and 'wc' can be set to a constant.");
  run(ctx->impl, "catalogue_kernel", c->n, fill_kernel, c->n, value,
      c->col[k]);
  if (k != kNZ) update_weights(ctx->impl, c);
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_upload(trvg_context* ctx, trvg_dcat* c, const char* column,
                     const double* values) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (column == nullptr || (values == nullptr && c->n > 0))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  double** slot = column_slot(c, column);
  if (slot == nullptr || slot == &c->w)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Column '%s' cannot be uploaded.", column);
  if (*slot == nullptr) *slot = dalloc(c->n);
  if (c->n > 0)
    TRVG_CUDA(cudaMemcpyAsync(*slot, values, size_t(c->n) * sizeof(double),
                              cudaMemcpyHostToDevice, ctx->impl.stream));
  if (slot == &c->col[kWS] || slot == &c->col[kWC])
    update_weights(ctx->impl, c);
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_norm_sum(trvg_context* ctx, const trvg_dcat* c, int order,
                       double* sum, int64_t* nonzero_nz) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (order != 2 && order != 3)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Order must be 2 or 3.");
  double t[2];
  sums(ctx->impl, c, order, t);
  if (sum) *sum = t[0];
  if (nonzero_nz) *nonzero_nz = int64_t(t[1]);
  TRVG_API_END
}

int trvg_dcat_view(const trvg_dcat* c, trvg_catalogue* out) {
  TRVG_API_BEGIN
  if (c == nullptr || out == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  out->n = c->n;
  out->x = c->col[kX];
  out->y = c->col[kY];
  out->z = c->col[kZ];
  out->w = c->w;
  out->los_x = c->los[0];
  out->los_y = c->los[1];
  out->los_z = c->los[2];
  out->memory = TRVG_MEM_DEVICE;
  TRVG_API_END
}

int trvg_dcat_download(trvg_context* ctx, const trvg_dcat* c,
                       const char* column, double* out) {
  TRVG_API_BEGIN
  check(ctx, c);
  if (column == nullptr || (out == nullptr && c->n > 0))
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Null argument.");
  double* const* slot = column_slot(const_cast<trvg_dcat*>(c), column);
  const double* src = slot ? *slot : nullptr;
  if (src == nullptr)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Unknown or absent column '%s'.",
                column);
  if (c->n > 0)
    TRVG_CUDA(cudaMemcpyAsync(out, src, size_t(c->n) * sizeof(double),
                              cudaMemcpyDeviceToHost, ctx->impl.stream));
  TRVG_CUDA(cudaStreamSynchronize(ctx->impl.stream));
  TRVG_API_END
}

int trvg_dcat_destroy(trvg_dcat* c) {
  TRVG_API_BEGIN
  if (c != nullptr) {
    dfree(c);
    delete c;
  }
  TRVG_API_END
}

}  // extern "C"
