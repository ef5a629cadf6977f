// Spatial counting sort of a particle catalogue by mesh tile.
//
// The assignment deposits every particle into order^3 mesh cells with
// atomics.  In input order (e.g. uniformly random) consecutive particles
// touch unrelated cache lines of a mesh far larger than L2, so most atomics
// miss.  Sorting by mesh tile first (one counting pass, one scan, one
// scatter) makes the deposits of neighbouring threads share lines, and the
// mesh streams through L2 about once.  The tile side, 2^shift cells, is
// picked by the autotuner (default 8).  The order of deposits does not
// change the result beyond floating-point association.
#include <algorithm>

#include "kernels.h"

namespace trvg {

namespace {

// Approximate cell (the tile only orders the deposits): one multiply by
// n / L, no division.
__device__ __forceinline__ int cell_of(double x, int n, double ratio) {
  int i = int(x * ratio);
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

__global__ void tile_key_kernel(DevCatalogue cat, int n0, int n1, int n2,
                                double r0, double r1, double r2, int t1,
                                int t2, int shift, int* key, int* rank,
                                int* count) {
  const int64_t np = cat.count(), p0 = cat.first();
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < np;
       p += int64_t(gridDim.x) * blockDim.x) {
    const int tx = cell_of(cat.x[p0 + p], n0, r0) >> shift;
    const int ty = cell_of(cat.y[p0 + p], n1, r1) >> shift;
    const int tz = cell_of(cat.z[p0 + p], n2, r2) >> shift;
    const int k = (tx * t1 + ty) * t2 + tz;
    key[p] = k;
    rank[p] = atomicAdd(count + k, 1);
  }
}

// Exclusive scan of count[0..n) in place: per-block scans of 2048
// elements, a scan of the block totals, then the block offsets added.
constexpr int kScanBlock = 1024;
constexpr int kScanTile = 2 * kScanBlock;

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh) {
  // Inclusive Hillis-Steele scan in shared memory, returned exclusive.
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < int(blockDim.x); off <<= 1) {
    const int t = (int(threadIdx.x) >= off) ? sh[threadIdx.x - off] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  const int incl = sh[threadIdx.x];
  __syncthreads();
  return incl - v;
}

__global__ void __launch_bounds__(kScanBlock)
scan_tiles_kernel(int* count, int n, int* tile_sum) {
  __shared__ int sh[kScanBlock];
  const int64_t base = int64_t(blockIdx.x) * kScanTile;
  const int64_t i0 = base + 2 * threadIdx.x, i1 = i0 + 1;
  const int a = (i0 < n) ? count[i0] : 0;
  const int b = (i1 < n) ? count[i1] : 0;
  const int ex = block_exclusive_scan(a + b, sh);
  if (i0 < n) count[i0] = ex;
  if (i1 < n) count[i1] = ex + a;
  if (threadIdx.x == blockDim.x - 1) tile_sum[blockIdx.x] = ex + a + b;
}

// Exclusive scan of the tile totals (at most 1024 * 2048 tiles handled by
// looping one block over them).
__global__ void __launch_bounds__(kScanBlock)
scan_sums_kernel(int* tile_sum, int ntiles) {
  __shared__ int sh[kScanBlock];
  int carry = 0;
  for (int base = 0; base < ntiles; base += kScanBlock) {
    const int i = base + threadIdx.x;
    const int v = (i < ntiles) ? tile_sum[i] : 0;
    const int ex = block_exclusive_scan(v, sh);
    if (i < ntiles) tile_sum[i] = carry + ex;
    __shared__ int total;
    if (threadIdx.x == blockDim.x - 1) total = ex + v;
    __syncthreads();
    carry += total;
    __syncthreads();
  }
}

__global__ void add_offsets_kernel(int* count, int n, const int* tile_sum) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) count[i] += tile_sum[i / kScanTile];
}

struct SortedOut {
  double* x;
  double* y;
  double* z;
  double* w;
  double* lx;
  double* ly;
  double* lz;
};

__global__ void scatter_kernel(DevCatalogue in, const int* key,
                               const int* rank, const int* offset,
                               SortedOut out) {
  const int64_t np = in.count(), p0 = in.first();
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < np;
       p += int64_t(gridDim.x) * blockDim.x) {
    const int64_t d = int64_t(offset[key[p]]) + rank[p];
    const int64_t q = p0 + p;
    out.x[d] = in.x[q];
    out.y[d] = in.y[q];
    out.z[d] = in.z[q];
    if (out.w != nullptr) out.w[d] = in.w[q];
    if (out.lx != nullptr) {
      out.lx[d] = in.lx[q];
      out.ly[d] = in.ly[q];
      out.lz[d] = in.lz[q];
    }
  }
}

int grid_for(int64_t work, int block) {
  int64_t g = (work + block - 1) / block;
  const int64_t cap = 152 * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return int(g);
}

}  // namespace

DevCatalogue sort_catalogue(Context& ctx, const Geom& g, const DevCatalogue& in,
                            const std::string& tag, int shift) {
  if (in.n < 2) return in;
  if (in.n > int64_t(2147483647))
    throw_error(TRVG_ERR_INVALID_DATA, "Catalogue larger than 2^31 particles.");
  const int side = 1 << shift;
  const int t0 = (g.n[0] + side - 1) >> shift;
  const int t1 = (g.n[1] + side - 1) >> shift;
  const int t2 = (g.n[2] + side - 1) >> shift;
  const int64_t ntiles = int64_t(t0) * t1 * t2;
  if (ntiles > int64_t(1) << 30) return in;
  int* key = ctx.buf<int>(tag + ".sort.key", size_t(in.n));
  int* rank = ctx.buf<int>(tag + ".sort.rank", size_t(in.n));
  int* count = ctx.buf<int>(tag + ".sort.count", size_t(ntiles));
  TRVG_CUDA(cudaMemsetAsync(count, 0, size_t(ntiles) * sizeof(int),
                            ctx.stream));
  TRVG_KBEGIN(ctx, "tile_key_kernel");
  tile_key_kernel<<<grid_for(in.n, 256), 256, 0, ctx.stream>>>(
      in, g.n[0], g.n[1], g.n[2], g.n[0] / g.L[0], g.n[1] / g.L[1],
      g.n[2] / g.L[2], t1, t2, shift, key, rank, count);
  TRVG_LAUNCHED(ctx);
  const int nscan = int((ntiles + kScanTile - 1) / kScanTile);
  int* tile_sum = ctx.buf<int>(tag + ".sort.tiles", size_t(nscan));
  TRVG_KBEGIN(ctx, "scan_kernel");
  scan_tiles_kernel<<<nscan, kScanBlock, 0, ctx.stream>>>(count, int(ntiles),
                                                          tile_sum);
  TRVG_LAUNCHED(ctx);
  TRVG_KBEGIN(ctx, "scan_kernel");
  scan_sums_kernel<<<1, kScanBlock, 0, ctx.stream>>>(tile_sum, nscan);
  TRVG_LAUNCHED(ctx);
  TRVG_KBEGIN(ctx, "scan_kernel");
  add_offsets_kernel<<<int((ntiles + 255) / 256), 256, 0, ctx.stream>>>(
      count, int(ntiles), tile_sum);
  TRVG_LAUNCHED(ctx);
  SortedOut o;
  const size_t n = size_t(in.n);
  o.x = ctx.buf<double>(tag + ".sorted.x", n);
  o.y = ctx.buf<double>(tag + ".sorted.y", n);
  o.z = ctx.buf<double>(tag + ".sorted.z", n);
  o.w = in.w ? ctx.buf<double>(tag + ".sorted.w", n) : nullptr;
  o.lx = in.lx ? ctx.buf<double>(tag + ".sorted.lx", n) : nullptr;
  o.ly = in.lx ? ctx.buf<double>(tag + ".sorted.ly", n) : nullptr;
  o.lz = in.lx ? ctx.buf<double>(tag + ".sorted.lz", n) : nullptr;
  TRVG_KBEGIN(ctx, "scatter_kernel");
  scatter_kernel<<<grid_for(in.n, 256), 256, 0, ctx.stream>>>(in, key, rank,
                                                              count, o);
  TRVG_LAUNCHED(ctx);
  DevCatalogue d;
  d.n = in.n;
  d.x = o.x;
  d.y = o.y;
  d.z = o.z;
  d.w = o.w;
  d.lx = o.lx;
  d.ly = o.ly;
  d.lz = o.lz;
  d.dev_n = in.dev_n;  // the sorted copy starts at its first element
  d.tile_start = count;
  d.tile_shift = shift;
  return d;
}

}  // namespace trvg
