// Allocation-free grid-based power-law normalisation.
//
// Same computation as trvg_calc_grid_based_powlaw_norm at FP64 (assign the
// particles to a mesh, sum the mesh to the given power;
// MeshField::calc_grid_based_powlaw_norm, field.cpp:2017-2062), but the
// mesh and the reduction slots live in one file-scope device array instead
// of a context's grow-only workspace, and no context is created.
//
// Who needs it: callers that have handed all device memory to another pool
// (a framework's caching allocator, a runtime that preallocates most of
// the GPU) cannot let the library grow workspace of its own, and
// long-running pipelines avoid cudaMalloc / cudaFree after start-up because
// both synchronise the device and stall every other stream.
//
// Limits:
//  - at most kMaxCells = 2^21 mesh cells (128^3; 16 MiB of scratch);
//  - particle arrays must already be in device memory;
//  - the arithmetic is FP64 whatever params->precision says;
//  - one scratch array per device: calls that overlap on one device (from
//    different host threads, or on different streams before the previous
//    call returned) race on it and must be serialised by the caller;
//  - the call reads its result back and synchronises `stream`, so it must
//    not be made while `stream` (or, in global capture mode, any stream)
//    is being captured;
//  - the first call on a device looks up the scratch address on that
//    device (the one current on the calling thread) with
//    cudaGetSymbolAddress, a one-off host-side step.
#include <cmath>
#include <mutex>

#include "internal.h"
#include "kernels.h"

namespace trvg {
namespace {

constexpr int64_t kMaxCells = int64_t(1) << 21;
constexpr int64_t kTail = 32;  // [0, 4): assignment sums; [4]: power sum
constexpr int kMaxDevices = 64;

// Mesh cells [0, kMaxCells), then the reduction slots.  The call zeroes
// the part it uses on the caller's stream before the deposit, so nothing
// has to be zero on entry.
static __device__ __align__(256) double g_powlaw_scratch[kMaxCells + kTail];

std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on device `dev`, which must be the
// calling thread's current device.  Looked up once per device.
double* scratch_on(int dev) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    double* p = nullptr;
    const cudaError_t e =
        cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_powlaw_scratch);
    if (e != cudaSuccess || p == nullptr)
      throw_error(TRVG_ERR_CUDA,
                  "Cannot resolve the static scratch on device %d: %s.", dev,
                  cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

Geom geometry(const trvg_params& p) {
  Geom g;
  for (int i = 0; i < 3; ++i) {
    g.n[i] = p.ngrid[i];
    g.L[i] = p.boxsize[i];
    g.dk[i] = 2. * M_PI / p.boxsize[i];
    g.dr[i] = p.boxsize[i] / p.ngrid[i];
  }
  g.vol = p.boxsize[0] * p.boxsize[1] * p.boxsize[2];
  g.nmesh = int64_t(g.n[0]) * g.n[1] * g.n[2];
  g.vol_cell = g.vol / double(g.nmesh);
  g.nzh = g.n[2] / 2 + 1;
  g.nhalf = int64_t(g.n[0]) * g.n[1] * g.nzh;
  return g;
}

void check_inputs(const trvg_params* p, const trvg_catalogue* c, int order,
                  const double* norm_factor) {
  if (p == nullptr || c == nullptr || norm_factor == nullptr || order < 1)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Invalid arguments.");
  for (int i = 0; i < 3; ++i) {
    if (p->ngrid[i] < 2)
      throw_error(TRVG_ERR_INVALID_PARAMETER,
                  "Mesh number must be >= 2 in every dimension: %d.",
                  p->ngrid[i]);
    if (!(p->boxsize[i] > 0.) || !std::isfinite(p->boxsize[i]))
      throw_error(TRVG_ERR_INVALID_PARAMETER,
                  "Box size must be positive in every dimension.");
  }
  const double cells =
      double(p->ngrid[0]) * double(p->ngrid[1]) * double(p->ngrid[2]);
  if (cells > double(kMaxCells))
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Mesh of %.0f cells exceeds the %lld-cell static scratch of "
                "the allocation-free normalisation.",
                cells, (long long)kMaxCells);
  if (p->assignment_order < 1 || p->assignment_order > 4)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "Mesh assignment scheme must be 'ngp', 'cic', 'tsc' or "
                "'pcs' (order %d given).",
                p->assignment_order);
  if (c->memory != TRVG_MEM_DEVICE)
    throw_error(TRVG_ERR_INVALID_PARAMETER,
                "The allocation-free normalisation takes device-resident "
                "particle arrays only.");
  if (c->n < 0)
    throw_error(TRVG_ERR_INVALID_DATA, "Negative particle count.");
  if (c->n > 0 && (c->x == nullptr || c->y == nullptr || c->z == nullptr))
    throw_error(TRVG_ERR_INVALID_DATA, "Particle data are uninitialised.");
}

}  // namespace
}  // namespace trvg

extern "C" {

int trvg_calc_grid_based_powlaw_norm_noalloc(const trvg_params* params,
                                             const trvg_catalogue* particles,
                                             int order, void* stream,
                                             double* norm_factor) {
  TRVG_API_BEGIN
  using namespace trvg;
  check_inputs(params, particles, order, norm_factor);
  int dev = 0;
  TRVG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    throw_error(TRVG_ERR_INVALID_PARAMETER, "Device ordinal %d unsupported.",
                dev);
  double* scratch = scratch_on(dev);
  double* mesh = scratch;
  double* sums = scratch + kMaxCells;
  double* acc = sums + 4;

  const Geom g = geometry(*params);
  Context ctx;  // launch bookkeeping only: no stream, events or buffers
  ctx.device = dev;
  ctx.stream = static_cast<cudaStream_t>(stream);

  TRVG_CUDA(cudaMemsetAsync(mesh, 0, size_t(g.nmesh) * sizeof(double),
                            ctx.stream));
  TRVG_CUDA(cudaMemsetAsync(sums, 0, 5 * sizeof(double), ctx.stream));
  DevCatalogue cat;
  cat.n = particles->n;
  cat.x = particles->x;
  cat.y = particles->y;
  cat.z = particles->z;
  cat.w = particles->w;
  launch_assign<double>(ctx, g, params->assignment_order, false, cat,
                        WeightSpec(), mesh, nullptr, nullptr, nullptr, sums);
  launch_mesh_sum_pow<double>(ctx, mesh, g.nmesh, order, acc);
  // The launch helpers take their scratch from a context's workspace when
  // a path needs one; none may have been drawn here.
  if (!ctx.buffers.empty())
    throw_error(TRVG_ERR_ALLOC,
                "The allocation-free normalisation drew %zu workspace "
                "buffers.", ctx.buffers.size());
  double s = 0.;
  TRVG_CUDA(cudaMemcpyAsync(&s, acc, sizeof(double), cudaMemcpyDeviceToHost,
                            ctx.stream));
  TRVG_CUDA(cudaStreamSynchronize(ctx.stream));
  TRVG_CUDA(cudaGetLastError());
  // The mesh holds n dV; the library sums n^order over cells times dV.
  const double vint = s / std::pow(g.vol_cell, order) * g.vol_cell;
  *norm_factor = 1. / vint;
  TRVG_API_END
}

}  // extern "C"
