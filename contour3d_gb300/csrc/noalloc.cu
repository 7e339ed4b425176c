/*
 * noalloc.cu -- per-cell triangle offsets of one iso-level without any device
 * allocation: contour3d_gb300_cell_offsets_noalloc (include/contour3d_gb300.h).
 *
 * Some callers cannot let a library allocate device memory: an in-situ solver
 * that has reserved the GPU's memory for its own pool (a cudaMalloc would fail
 * or would break the pool's accounting), or a time-stepping loop that must
 * not stall on the implicit device synchronisation of cudaFree.  This entry
 * point serves them.  The caller passes the field and the output arrays; the
 * only other memory the kernel touches -- the tile states of the single-pass
 * scan -- lives in the file-scope array below, which every GPU that loads the
 * library holds (kScratchBytes) until the process exits.
 *
 * The kernel is a single-pass scan with decoupled look-back that computes
 * each cell's triangle count from the field itself (the classification rule
 * of kernels.cu) instead of reading a codes array, so no intermediate buffer
 * is needed.  Tiles are taken in order from an atomic counter, so every tile
 * a block waits on is running or done; the wait is bounded (2^22 polls) and
 * raises an error flag that the host reports.
 *
 * Contract:
 *   - at most kMaxCells cells ((nx-1)(ny-1)(nz-1)); larger fields are
 *     rejected with an error before anything is launched;
 *   - the first call on a device looks up the scratch array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture on that device;
 *   - every call shares the one scratch array and clears the part it uses at
 *     its start; calls that overlap on the GPU (other streams, other host
 *     threads) race on it and must be serialised by the caller;
 *   - `stream` must belong to the current device (checked);
 *   - every call copies the 4-byte error word back to the host and
 *     synchronises `stream` before it returns, so the return code covers the
 *     device work too;
 *   - the cached device address is only valid for the device context it was
 *     taken in: the library must not be used across a cudaDeviceReset;
 *   - no cudaMalloc, cudaFree or allocating library routine is called.
 */
#include <cuda_runtime.h>
#include <cuda/atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include "contour3d_gb300.h"
#include "c3d_common.cuh"
#include "c3d_host.h"

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr long long kTile = kThreads * kItems;
constexpr long long kMaxTiles = 1 << 16;
/* the scan also writes the offset after the last cell, so tiles cover n + 1 positions */
constexpr long long kMaxCells = kMaxTiles * kTile - 1;
constexpr int kMaxDevices = 64;
constexpr unsigned long long kAgg = 1ULL << 62;
constexpr unsigned long long kPrefix = 2ULL << 62;
constexpr unsigned long long kValue = (1ULL << 62) - 1;
constexpr unsigned kErrTimeout = 1u;

/* word 0: tile counter, word 1: error flags, words 2..: one state per tile */
constexpr size_t kScratchWords = 2 + (size_t)kMaxTiles;
constexpr size_t kScratchBytes = kScratchWords * sizeof(unsigned long long);
static __device__ __align__(256) unsigned long long g_scratch[kScratchWords];

/* cube corners of the six tetrahedra, and triangles per folded mask (triangulate.c:145-270) */
__constant__ unsigned char c_tet[6][4] = {{0, 7, 3, 1}, {0, 7, 1, 5}, {0, 7, 5, 4},
                                          {0, 7, 4, 6}, {0, 7, 6, 2}, {0, 7, 2, 3}};
__constant__ unsigned char c_ntri[8] = {0, 1, 1, 2, 1, 2, 2, 1};

struct Grid {
  const void* data;
  long long nx, ny, nz;
  long long thr_key;
  int thr_nan;
};

template <typename T>
__device__ __forceinline__ unsigned cell_count(const Grid& g, long long c) {
  const long long ncx = g.nx - 1, ncy = g.ny - 1;
  const long long i = c % ncx, j = (c / ncx) % ncy, k = c / (ncx * ncy);
  const T* f = static_cast<const T*>(g.data);
  const long long base = (k * g.ny + j) * g.nx + i;
  unsigned code = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const long long idx = base + ((q & 1) ? 1 : 0) + ((q & 2) ? g.nx : 0) + ((q & 4) ? g.nx * g.ny : 0);
    const double v = (double)f[idx];
    const bool above = !g.thr_nan && !c3d::d_isnan(v) && c3d::d_key(v) > g.thr_key;
    code |= (unsigned)above << q;
  }
  unsigned n = 0;
#pragma unroll
  for (int t = 0; t < 6; t++) {
    unsigned m = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) m |= ((code >> c_tet[t][q]) & 1u) << q;
    if (m >= 8) m = 15 - m;
    n += c_ntri[m];
  }
  return n;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_offsets_noalloc(Grid g, long long n, unsigned* __restrict__ offsets, unsigned long long* __restrict__ total,
                  unsigned long long* __restrict__ scratch) {
  __shared__ unsigned s_tile;
  __shared__ unsigned long long s_warp[kThreads / 32];
  __shared__ unsigned long long s_excl;
  unsigned* counter = reinterpret_cast<unsigned*>(scratch);
  unsigned* err = reinterpret_cast<unsigned*>(scratch + 1);
  unsigned long long* state = scratch + 2;
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const unsigned tile = s_tile;
  const long long base = (long long)tile * kTile + (long long)threadIdx.x * kItems;
  unsigned char cnt[kItems];
  unsigned sum = 0;
#pragma unroll
  for (int q = 0; q < kItems; q++) {
    const long long c = base + q;
    cnt[q] = c < n ? (unsigned char)cell_count<T>(g, c) : 0;
    sum += cnt[q];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long incl = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < kThreads / 32 ? s_warp[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, d);
      if (lane >= d) w += y;
    }
    if (lane < kThreads / 32) s_warp[lane] = w;
  }
  __syncthreads();
  const unsigned long long agg = s_warp[kThreads / 32 - 1];
  const unsigned long long texcl = (warp ? s_warp[warp - 1] : 0) + incl - sum;
  if (warp == 0) {
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> mine(state[tile]);
    if (lane == 0) mine.store((tile == 0 ? kPrefix : kAgg) | agg, cuda::memory_order_release);
    unsigned long long excl = 0;
    if (tile > 0) {
      long long pred = (long long)tile - 1;
      int spins = 0;
      bool done = false;
      while (!done) {
        const long long p = pred - lane;
        unsigned long long st = 0;
        if (p >= 0) {
          cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> ps(state[p]);
          st = ps.load(cuda::memory_order_acquire);
        }
        const unsigned invalid = __ballot_sync(0xFFFFFFFFu, p >= 0 && (st >> 62) == 0);
        const unsigned prefix = __ballot_sync(0xFFFFFFFFu, p >= 0 && (st >> 62) == 2);
        const unsigned fi = invalid ? __ffs(invalid) - 1 : 32;
        const unsigned fp = prefix ? __ffs(prefix) - 1 : 32;
        unsigned take = 0;
        if (fp < fi) {
          take = fp + 1;
          done = true;
        } else if (fi > 0) {
          take = fi;
        }
        if (take) {
          unsigned long long v = (lane < (int)take && p >= 0) ? (st & kValue) : 0;
#pragma unroll
          for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
          excl += v;
          pred -= take;
          if (pred < 0) done = true;
        } else if (++spins > (1 << 22)) {
          if (lane == 0) atomicOr(err, kErrTimeout);
          done = true;
        } else {
          __nanosleep(64);
        }
      }
      if (lane == 0) mine.store(kPrefix | ((excl + agg) & kValue), cuda::memory_order_release);
    }
    if (lane == 0) s_excl = excl;
  }
  __syncthreads();
  unsigned long long run = s_excl + texcl;
#pragma unroll
  for (int q = 0; q < kItems; q++) {
    const long long c = base + q;
    if (c <= n) offsets[c] = (unsigned)run;
    if (c == n) *total = run;
    run += cnt[q];
  }
}

std::mutex g_mu;
unsigned long long* g_scratch_ptr[kMaxDevices] = {};

long long host_key(double x) {
  long long b;
  memcpy(&b, &x, sizeof b);
  if ((b << 1) == 0) b = 0;
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}

}  // namespace

extern "C" int contour3d_gb300_cell_offsets_noalloc(const void* device_field, int dtype, const size_t sizes[3],
                                                    double threshold, uint32_t* device_offsets,
                                                    unsigned long long* device_total, void* stream) {
  if (!device_field || !sizes || !device_offsets || !device_total ||
      (dtype != CONTOUR3D_GB300_F64 && dtype != CONTOUR3D_GB300_F32)) {
    c3d::log_error("cell_offsets_noalloc: null pointer or unknown dtype");
    return 1;
  }
  if (sizes[0] < 2 || sizes[1] < 2 || sizes[2] < 2) {
    c3d::log_error("cell_offsets_noalloc: every size must be at least 2 nodes");
    return 1;
  }
  const double cells = (double)(sizes[0] - 1) * (double)(sizes[1] - 1) * (double)(sizes[2] - 1);
  if (cells > (double)kMaxCells) {
    c3d::log_error("cell_offsets_noalloc: %.0f cells exceed the no-allocation limit of %lld cells "
                   "(%zu bytes of static scratch); use contour3d_gb300_render_device instead",
                   cells, kMaxCells, kScratchBytes);
    return 1;
  }
  const long long n = (long long)(sizes[0] - 1) * (long long)(sizes[1] - 1) * (long long)(sizes[2] - 1);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    c3d::log_error("cell_offsets_noalloc: no usable current device");
    return 1;
  }
  unsigned long long* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
      /* once per device, with that device current: the host-side name of the
         array is not its device address */
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess || !p) {
        c3d::log_error("cell_offsets_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return 1;
      }
      g_scratch_ptr[dev] = static_cast<unsigned long long*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st) {
    int sdev = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess || sdev != dev) {
      cudaGetLastError();
      c3d::log_error("cell_offsets_noalloc: the stream does not belong to the current device %d", dev);
      return 1;
    }
  }
  const long long tiles = (n + kTile) / kTile;
  /* the counter, the error word and the tile states this call uses start at zero */
  if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * (size_t)(2 + tiles), st) != cudaSuccess) {
    c3d::log_error("cell_offsets_noalloc: clearing the scratch failed");
    return 1;
  }
  Grid g;
  g.data = device_field;
  g.nx = (long long)sizes[0];
  g.ny = (long long)sizes[1];
  g.nz = (long long)sizes[2];
  g.thr_key = host_key(threshold);
  g.thr_nan = std::isnan(threshold) ? 1 : 0;
  if (dtype == CONTOUR3D_GB300_F64)
    k_offsets_noalloc<double><<<(unsigned)tiles, kThreads, 0, st>>>(g, n, device_offsets, device_total, scratch);
  else
    k_offsets_noalloc<float><<<(unsigned)tiles, kThreads, 0, st>>>(g, n, device_offsets, device_total, scratch);
  cudaError_t e = cudaGetLastError();
  unsigned errw = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&errw, scratch + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    c3d::log_error("cell_offsets_noalloc: %s", cudaGetErrorString(e));
    return 1;
  }
  if (errw) {
    c3d::log_error("cell_offsets_noalloc: the device scan did not complete (flags 0x%x)", errw);
    return 1;
  }
  return 0;
}
