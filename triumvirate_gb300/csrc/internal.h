// Host-side internals: errors, device workspace, FFT plans, the context.
#pragma once

#include <cstdint>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <cufft.h>

#include "common.cuh"
#include "trvg.h"

namespace trvg {

// Error carrying a C-ABI status code.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] void throw_error(int code, const char* fmt, ...);
void set_last_error(const std::string& msg);
const char* last_error();

// Body wrappers of the C-ABI functions: exceptions become status codes and
// the thread's last-error message.
#define TRVG_API_BEGIN try {
#define TRVG_API_END                                        \
  }                                                         \
  catch (const ::trvg::Error& e) {                          \
    ::trvg::set_last_error(e.what());                       \
    return e.code;                                          \
  }                                                         \
  catch (const std::bad_alloc&) {                           \
    ::trvg::set_last_error("Host allocation failed.");      \
    return TRVG_ERR_ALLOC;                                  \
  }                                                         \
  catch (const std::exception& e) {                         \
    ::trvg::set_last_error(e.what());                       \
    return TRVG_ERR_INVALID_DATA;                           \
  }                                                         \
  ::trvg::set_last_error("");                               \
  return TRVG_OK;

#define TRVG_CUDA(call)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess)                                                  \
      ::trvg::throw_error(TRVG_ERR_CUDA, "%s failed at %s:%d: %s", #call,   \
                          __FILE_NAME__, __LINE__, cudaGetErrorString(e_));      \
  } while (0)

#define TRVG_CUFFT(call)                                                    \
  do {                                                                      \
    cufftResult r_ = (call);                                                \
    if (r_ != CUFFT_SUCCESS)                                                \
      ::trvg::throw_error(TRVG_ERR_CUFFT, "%s failed at %s:%d: cufft %d",   \
                          #call, __FILE_NAME__, __LINE__, int(r_));              \
  } while (0)

// Bracket a launch: TRVG_KBEGIN records the start event when profiling,
// TRVG_LAUNCHED checks the launch (configuration errors surface here;
// faults in the kernel surface at the next synchronising call), counts it
// and records the end event.
#define TRVG_KBEGIN(ctx, name) (ctx).kbegin(name)
#define TRVG_LAUNCHED(ctx)                                                  \
  do {                                                                      \
    TRVG_CUDA(cudaGetLastError());                                          \
    (ctx).kernel_launches++;                                                \
    (ctx).kend();                                                           \
  } while (0)

// A named, grow-only device buffer.  Buffers persist across calls on one
// context so that repeated estimates allocate nothing.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

// cuFFT plan key.
struct PlanKey {
  int type;       // cufftType
  int n[3];
  int batch;
  bool operator<(const PlanKey& o) const {
    if (type != o.type) return type < o.type;
    for (int i = 0; i < 3; ++i)
      if (n[i] != o.n[i]) return n[i] < o.n[i];
    return batch < o.batch;
  }
};

// One timed launch of the current call (profiling mode).
struct KernelRecord {
  const char* name;
  cudaEvent_t begin, end;
};

// Mode list of the fine-binned two-point statistics for one mesh, binning
// and degree pair (device arrays are named buffers under `tag`).
struct StatsPlan {
  std::string tag;
  int max_count = 0;
  std::vector<long long> nmodes;
  std::vector<double> ksum;
  std::vector<double> snsum;  // re, im per bin
  // Device copies of nmodes (as doubles) and snsum for replayed batches.
  const double* dev_nmodes = nullptr;
  const double* dev_snsum = nullptr;
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;       // stream in use
  cudaStream_t own_stream = nullptr;   // stream created with the context
  std::map<std::string, DeviceBuffer> buffers;
  std::map<PlanKey, cufftHandle> plans;
  cudaEvent_t ev_start = nullptr, ev_h2d = nullptr, ev_stop = nullptr;
  // Second stream for memory-bound work next to FP32-issue-bound work of
  // the same estimate (created on first use), with its fork / join events.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool overlap = true;
  // Priority of the second stream: 0 the default, 1 the device's greatest
  // (its blocks are dispatched first whenever an SM has room).
  int side_priority = 0;
  cudaStream_t side_stream();
  int verbose = 0;
  // Counters of the current / last call.
  int64_t kernel_launches = 0;
  int64_t fft_launches = 0;
  int64_t h2d_bytes = 0;
  double ms_total = 0., ms_h2d = 0.;
  int pruned_grid[3] = {0, 0, 0};
  // Options.
  bool full_mesh_shells = false;  // evaluate shell fields on the full mesh
  // FP32-mixed precision choices: shot-noise field / shell fields in FP64.
  bool shotnoise_fp64 = false;
  bool shell_fields_fp64 = false;
  // Order large catalogues by mesh tile before the deposit.
  bool sort_catalogue = true;
  // FP32-mixed: float-float transforms of the shell fields (0 none, 1 both
  // directions, 2 the forward transform of the mesh only).
  int ff_transforms = 1;
  // FP32 pair sums one pair per thread instead of the register-tiled Gram
  // form (a comparison switch; both accumulate in float-float).
  bool gram_per_pair = false;
  // Batches: replay one captured mock as a CUDA graph (batch.cu).
  bool graph_batch = true;
  // Autotuner: launch shapes picked by timing (tile side of the catalogue
  // sort, bin batch of the pair reduction), cached by key.
  bool autotune = true;
  std::map<std::string, int> tuned;
  // Shot-noise field of m = 0, even-degree legs on one octant (FP32).
  bool xi_octant = true;
  // Y_lm-weighted fields of every order in one fused pass (FP32 meshes).
  bool fused_ylm = true;
  // Deposit of sorted catalogues: 0 tuned, 1 tiled (shared memory),
  // 2 global atomics.
  int assign_path = 0;
  // FP32-mixed meshes deposited with float-float windows and compensated
  // atomics into a second FP32 mesh: 0 never, 1 always, 2 fields built
  // from several catalogues (data minus randoms, which cancel).  The tiled
  // deposit serves uncompensated meshes only.
  int mesh_comp = 2;
  // Round every compensated mesh to its correctly rounded FP32 sum before
  // the FP32 transforms (always done for fields of several catalogues).
  bool mesh_renorm = false;
  // Mocks replayed from the captured graph by the last batch call.
  int64_t graph_replays = 0;
  // Deposits made so far (FieldSpec::mesh_gen).
  int64_t mesh_gen = 0;
  // Profiling: per-launch events of the current call, per-name totals of
  // the last call.
  bool profiling = false;
  std::vector<cudaEvent_t> event_pool;
  size_t events_used = 0;
  std::vector<KernelRecord> records;
  const char* pending = nullptr;
  cudaEvent_t pending_begin = nullptr;
  std::vector<std::pair<std::string, std::pair<double, int64_t>>> ktimes;
  // j_ell spline tables by ell (device arrays are named buffers).
  std::map<int, SplineTable> splines;
  // Two-point statistics mode lists by key.
  std::map<std::string, StatsPlan> stats_plans;
  // Shell mode counts and k sums (nmodes, k_eff) by mesh and bin edges.
  std::map<std::string, std::pair<std::vector<long long>,
                                  std::vector<double>>> mode_counts;

  void kbegin(const char* name);
  void kend();
  void begin_call();
  void finish_call();   // after the stream is synchronised
  void set_stream(cudaStream_t s);

  // Grow-only named buffer of at least `bytes` bytes.
  void* buffer(const std::string& name, size_t bytes);
  template <class T>
  T* buf(const std::string& name, size_t count) {
    return static_cast<T*>(buffer(name, count * sizeof(T)));
  }
  cufftHandle plan(int type, const int n[3], int batch);
  // Batched 1-D plan of length n (cached with the 3-D ones).
  cufftHandle plan1d(int type, int n, int batch);
  // In-place C2C of nz contiguous n0 x n1 planes (element (z, x, y) at
  // (z n0 + x) n1 + y): the x and y transforms that complete an R2C whose
  // z transform is done.
  cufftHandle plan_xy(int n0, int n1, int nz);
  void release();
  void log(int level, const char* fmt, ...) const;
};

void destroy_events(Context& c);

}  // namespace trvg

struct trvg_context {
  trvg::Context impl;
};
