/*
 * kernels.cu -- sm_103a kernels of the isosurface-to-image path.
 *
 * The contour objects of one field are classified together, then each
 * object is processed in z-slabs of cells, then shaded once:
 *   k_classify_tma  cell codes of up to four thresholds per pass over the
 *                   field (TMA node planes; k_classify where TMA cannot
 *                   address the field)                         (HBM: field read)
 * per slab of an object:
 *   k_scan          packed (triangle, vertex) counts per segment of cells,
 *                   the segment's prefix by decoupled look-back, then every
 *                   cell's offsets and the triangle -> cell map, in one pass
 *   k_vertices      one FP32 screen vertex per crossed edge, with certified
 *                   bounds (two FP64 subtractions per vertex)
 *   k_emit          one thread per triangle: its three vertices through their
 *                   owner cells, culling, and the raster route (cover list,
 *                   sliver list, tiny list, or dropped)
 *   k_raster        one thread per listed triangle, over the cover list
 *                   and then the sliver list: FP32 coverage and depth
 *                   intervals over its pixel range; certainly drawn
 *                   fragments raise a per-pixel depth floor, the rest become
 *                   candidates; slivers (area the reference may clamp) the
 *                   bounds cannot settle go to the tiny list
 *   k_finish        drops candidates below the final depth floor, then one
 *                   thread per remaining candidate: the reference's
 *                   vertices (recomputed from the field), projection,
 *                   barycentric test and harmonic depth in FP64, then a
 *                   128-bit (depth, order) max into the z-buffer; then one
 *                   thread per tiny-list triangle (too small for FP32
 *                   bounds): the reference's arithmetic for its few pixels
 * per object, after its slabs:
 *   k_winners       the pixels the object owns
 *   k_shade_f       FP32 vertex normals and colour with certified bounds
 *                   (block-shared triangle normals)
 *   k_nb_list, k_nb_wn, k_shade
 *                   the reference's FP64 colour for the pixels FP32 cannot
 *                   settle: neighbour triangles in normal.c's order, their
 *                   weighted normals, ordered sums and the shading
 * and once per frame k_canvas_init, k_lines and k_resolve.  k_exact_all and
 * k_normals compute every triangle's exact data for inspection only.
 *
 * The FP64 work runs one item per thread on compacted lists so that warps
 * stay converged: on GB300 an FP64 warp instruction costs the same whether 2
 * or 32 lanes are active.  Exact vertices are needed only for fragments that
 * can win, and weighted normals only around the triangles that finally own a
 * pixel, so they are computed for those alone.
 *
 * Reference correspondence (file:line of the reference tree):
 *   k_classify*, scan, k_emit   src/contour3d/contour/triangulate.c:95-342
 *   k_vertices, exact vertices  src/contour3d/contour/triangulate.c:40-73
 *   k_shade_f, k_nb_*, k_shade, k_normals
 *                               src/contour3d/contour/normal.c:6-165
 *   k_raster, k_finish, shading factor
 *                               src/contour3d/contour/render.c:38-163,
 *                               src/contour3d/project.c:9-67
 *   k_lines                     src/contour3d/line.c:26-119
 *   k_resolve                   src/contour3d/output.c:10-30, 113-123
 *   slab / interior             src/contour3d/contour/main.c:38-112
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <cuda/atomic>
#include "c3d_common.cuh"
#include "c3d_kernels.h"

namespace c3d {

__constant__ unsigned char c_code_count[256];
/* normal.c:78-158: per cube edge, the (dk, dj, di, local edge id) of the
   cells sharing it, in the reference's accumulation order */
__constant__ signed char c_nb[19][4][4];
__constant__ unsigned char c_nb_count[19];
/* per code and cube edge: bit r set when the cell's triangle of rank r has
   a vertex on that edge (read by lanes with different codes: global, cached) */
__device__ unsigned short g_edge_tris[256 * 19];

/* ------------------------------------------------------------------ */
/* field access                                                        */
/* ------------------------------------------------------------------ */
template <typename T>
__device__ __forceinline__ double load_value(const T* f, long long idx) {
  return (double)__ldg(f + idx);
}
template <>
__device__ __forceinline__ double load_value<double>(const double* f, long long idx) {
  return __longlong_as_double(ld_bits(f + idx));
}

/* bit c of the result: threshold < value at corner c of cell (i, j, k) */
template <typename T>
__device__ __forceinline__ unsigned cell_code(const FieldDev& F, long long i, long long j, long long k,
                                              double vals[8]) {
  const T* f = static_cast<const T*>(F.data);
  const long long sx = 1, sy = F.nx, sz = F.nx * F.ny;
  const long long base = k * sz + j * sy + i;
  unsigned code = 0;
  const long long tk = F.thr_key;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const long long idx = base + ((c & 1) ? sx : 0) + ((c & 2) ? sy : 0) + ((c & 4) ? sz : 0);
    const double v = load_value<T>(f, idx);
    vals[c] = v;
    const bool above = !F.thr_nan && !d_isnan(v) && d_key(v) > tk;
    code |= (unsigned)above << c;
  }
  return code;
}

__device__ __forceinline__ unsigned fast_div(unsigned n, const FastDiv& d) {
  const unsigned t = __umulhi(d.m, n);
  return (t + ((n - t) >> d.s1)) >> d.s2;
}

/* cell (i, j, k-in-slab) of a slab-local linear cell index; 32-bit arithmetic */
__device__ __forceinline__ void cell_ijk(const FieldDev& F, unsigned c, unsigned& i, unsigned& j, unsigned& kl) {
  const unsigned ncx = (unsigned)(F.nx - 1), ncy = (unsigned)(F.ny - 1);
  const unsigned r = fast_div(c, F.div_cx);
  i = c - r * ncx;
  kl = fast_div(r, F.div_cy);
  j = r - kl * ncy;
}

/* ------------------------------------------------------------------ */
/* counts per cell                                                     */
/* ------------------------------------------------------------------ */
/*
 * Per cell, its triangle count and the number of its owned vertices (edges
 * from its corner 0 that the iso-level crosses), packed as tri | vert << 31:
 * every sum over a slab stays below 2^31 in both fields for slabs of at most
 * kMaxSlabCells cells, so packed additions never carry.  The scan runs over
 * segments of kScanTile cells, one block each (k_scan).
 *
 * Vertices are owned by cells: cell c owns the crossed edges that start at
 * its corner 0 and run to corner m = 1..7 (+x, +y, +x+y, +z, +x+z, +y+z,
 * +x+y+z).  Every edge of the six-tetrahedra split joins corners a, b with
 * a & b = a or b, so it starts at corner a & b of its cell and runs in
 * direction a ^ b: it is the edge m = a ^ b owned by the cell at offset a & b.
 */
constexpr int kScanThreads = 256;
constexpr int kScanItems = 32;  /* cells per thread */
constexpr int kScanTile = kScanThreads * kScanItems;
static_assert(kScanTile == 1 << kVSegShift, "vertex offsets are relative to scan segments");
constexpr unsigned long long kTriMask = (1ULL << 31) - 1;

/* the vertex offset of cell c */
__device__ __forceinline__ unsigned voff_at(const VOffDev& o, long long c) {
  return o.seg[c >> kVSegShift] + o.rel[c];
}

/* bit m - 1: the iso-level crosses edge m of the cell's corner 0 */
__device__ __forceinline__ unsigned owned_edges(unsigned code) {
  const unsigned flip = code ^ (0u - (code & 1u));
  return (flip >> 1) & 0x7Fu;
}

/* triangles | vertices << 16 of every code, in shared memory */
__device__ __forceinline__ void load_count_lut(unsigned* lut) {
  for (int q = threadIdx.x; q < 256; q += blockDim.x)
    lut[q] = (unsigned)c_code_count[q] | ((unsigned)__popc(owned_edges((unsigned)q)) << 16);
}

__device__ __forceinline__ unsigned long long packed_count(unsigned c) {
  return (unsigned long long)(c & 0xFFFFu) | ((unsigned long long)(c >> 16) << 31);
}

/* ------------------------------------------------------------------ */
/* k_classify                                                          */
/* ------------------------------------------------------------------ */
/*
 * Tiled over (x, y) and marching in z: each node's "above" bit is computed
 * once into shared memory (two planes, double-buffered), and each cell
 * assembles its 8-bit code from the bits of its corners.  The codes are
 * kept: the scan maps them to triangle counts, and the later passes read
 * them instead of comparing the eight corner values again.  A block owns
 * kClsX x kClsY cells of kClsZ consecutive slices.
 */
constexpr int kClsX = 128;
constexpr int kClsY = 8;
constexpr int kClsZ = 32; /* default slices per brick (LaunchShape::cls_z) */

template <typename T>
__device__ __forceinline__ unsigned char node_above(const FieldDev& F, const T* f, long long idx);
template <>
__device__ __forceinline__ unsigned char node_above<double>(const FieldDev& F, const double* f, long long idx) {
  const long long b = ld_bits(f + idx);
  return (!F.thr_nan && !d_isnan_bits(b) && d_key_bits(b) > F.thr_key) ? 1 : 0;
}
template <>
__device__ __forceinline__ unsigned char node_above<float>(const FieldDev& F, const float* f, long long idx) {
  /* threshold < (double)v  <=>  v >= the least float above the threshold */
  const float v = __ldg(f + idx);
  return (F.thr_f_ok && v == v && f_key(v) >= F.thr_f_key) ? 1 : 0;
}

/* the same test against threshold t of a set (k_classify_tma classifies the
   objects of one field together), on the value's bit pattern: the
   sign-folded key, then one unsigned range check (ThrSet) */
template <typename T>
struct NodeBits;
template <>
struct NodeBits<double> {
  using type = long long;
};
template <>
struct NodeBits<float> {
  using type = int;
};
__device__ __forceinline__ bool node_above_thr(const ThrSet& ts, int t, long long b) {
  const long long key = b ^ (long long)((unsigned long long)(b >> 63) >> 1);
  return (unsigned long long)key - ts.lo[t] < ts.cnt[t];
}
__device__ __forceinline__ bool node_above_thr(const ThrSet& ts, int t, int b) {
  const int key = b ^ (int)((unsigned)(b >> 31) >> 1);
  return (unsigned)key - ts.flo[t] < ts.fcnt[t];
}

/* the cell codes of one brick (kClsX x kClsY cells, S.cls_z slices) */
template <typename T>
__device__ __forceinline__ void classify_brick(const FieldDev& F, const SlabDev& S, unsigned char* __restrict__ codes,
                                               unsigned bx, unsigned by, unsigned bz,
                                               unsigned char (*bits)[kClsY + 1][kClsX + 1]) {
  const T* f = static_cast<const T*>(F.data);
  const unsigned ncx = (unsigned)(F.nx - 1), ncy = (unsigned)(F.ny - 1);
  const unsigned i0 = bx * kClsX, j0 = by * kClsY;
  const long long k0 = (long long)bz * S.cls_z;
  const long long k1 = min(k0 + S.cls_z, S.nslices);
  const long long sx = F.nx, sxy = F.nx * F.ny;
  auto load_plane = [&](int buf, long long k) {
    for (int q = threadIdx.x; q < (kClsY + 1) * (kClsX + 1); q += blockDim.x) {
      const unsigned jj = (unsigned)q / (kClsX + 1), ii = (unsigned)q - jj * (kClsX + 1);
      const long long gi = (long long)i0 + ii, gj = (long long)j0 + jj;
      unsigned char b = 0;
      if (gi < F.nx && gj < F.ny) b = node_above<T>(F, f, k * sxy + gj * sx + gi);
      bits[buf][jj][ii] = b;
    }
  };
  load_plane(0, S.kfirst + k0);
  for (long long kl = k0; kl < k1; kl++) {
    const int cur = (int)((kl - k0) & 1), nxt = cur ^ 1;
    load_plane(nxt, S.kfirst + kl + 1);
    __syncthreads();
    const unsigned i = i0 + threadIdx.x;
    const bool in_x = i < ncx;
    const int tx = threadIdx.x;
#pragma unroll
    for (int jj = 0; jj < kClsY; jj++) {
      const unsigned j = j0 + jj;
      if (j >= ncy) break; /* the same for the whole block */
      const unsigned code = bits[cur][jj][tx] | (bits[cur][jj][tx + 1] << 1) | (bits[cur][jj + 1][tx] << 2) |
                            (bits[cur][jj + 1][tx + 1] << 3) | (bits[nxt][jj][tx] << 4) |
                            (bits[nxt][jj][tx + 1] << 5) | (bits[nxt][jj + 1][tx] << 6) |
                            (bits[nxt][jj + 1][tx + 1] << 7);
      if (in_x) codes[((size_t)kl * ncy + j) * ncx + i] = (unsigned char)code;
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(kClsX) k_classify(FieldDev F, SlabDev S, unsigned char* __restrict__ codes) {
  pdl_enter();
  __shared__ unsigned char bits[2][kClsY + 1][kClsX + 1];
  classify_brick<T>(F, S, codes, blockIdx.x, blockIdx.y, blockIdx.z, bits);
}

/*
 * k_classify_queue: the cell codes of many fields (the frames of a batch) in
 * one launch of a persistent grid.  A work item is one field with up to
 * kMaxThr thresholds; its bricks are numbered item by item
 * (ClsItem::first).  Each block takes the next brick number from a device
 * counter, finds its item by binary search over the items' first numbers,
 * and classifies that brick for all of the item's thresholds in one pass
 * over its nodes.  A node's values of the next plane are loaded into
 * registers before the current plane pair is turned into codes, so the
 * loads are in flight during that work.  Node masks hold bit t for
 * threshold t; a cell's code for threshold t gathers bit t of its eight
 * corner masks with one multiply (the corner masks as the bytes of a 64-bit
 * word: bit t of byte c moves to bit c of the top byte).  Every brick number
 * is taken once, so the loop ends after at most nunits / grid bricks per
 * block.
 */
constexpr int kQPlane = (kClsY + 1) * (kClsX + 1); /* nodes of a brick's plane */
constexpr int kQPer = (kQPlane + kClsX - 1) / kClsX; /* of them per thread */

/* what a block keeps of its current item, in shared memory */
struct QueueBrick {
  const void* data;
  unsigned char* codes[kMaxThr];
  long long nx, ny, kfirst, k0, k1;
  unsigned i0, j0, ncx, ncy;
  int nt;
};

template <typename T>
__device__ __forceinline__ void classify_queue_brick(const QueueBrick& qb, const ThrSet& ts,
                                                     unsigned char (*bits)[kClsY + 1][kClsX + 1]) {
  using K = typename NodeBits<T>::type;
  const K* __restrict__ f = static_cast<const K*>(qb.data);
  const long long nx = qb.nx, ny = qb.ny, sxy = nx * ny;
  const unsigned i0 = qb.i0, j0 = qb.j0, ncx = qb.ncx, ncy = qb.ncy;
  const long long k0 = qb.k0, k1 = qb.k1, kfirst = qb.kfirst;
  const int nt = qb.nt;
  /* the thresholds as key ranges (see ThrSet) */
  unsigned long long tlo[kMaxThr], tcnt[kMaxThr];
#pragma unroll
  for (int t = 0; t < kMaxThr; t++) {
    tlo[t] = sizeof(T) == 8 ? ts.lo[t] : ts.flo[t];
    tcnt[t] = t < nt ? (sizeof(T) == 8 ? ts.cnt[t] : ts.fcnt[t]) : 0ULL;
  }
  K v[kQPer];
  unsigned valid = 0;
  auto fetch = [&](long long k) {
    valid = 0;
#pragma unroll
    for (int r = 0; r < kQPer; r++) {
      const int q = threadIdx.x + r * kClsX;
      const unsigned jj = (unsigned)q / (kClsX + 1), ii = (unsigned)q - jj * (kClsX + 1);
      const long long gi = (long long)i0 + ii, gj = (long long)j0 + jj;
      const bool ok = q < kQPlane && gi < nx && gj < ny;
      v[r] = ok ? __ldg(f + k * sxy + gj * nx + gi) : K(0);
      valid |= (unsigned)ok << r;
    }
  };
  auto store = [&](int buf) {
    unsigned char* dst = &bits[buf][0][0];
#pragma unroll
    for (int r = 0; r < kQPer; r++) {
      const int q = threadIdx.x + r * kClsX;
      if (q < kQPlane) {
        unsigned m = 0;
        if ((valid >> r) & 1u) {
          /* sign-folded key, then one unsigned range check per threshold */
          const K b = v[r];
          const K key = b ^ (K)((typename std::make_unsigned<K>::type)(b >> (8 * sizeof(K) - 1)) >> 1);
#pragma unroll
          for (int t = 0; t < kMaxThr; t++) {
            if (sizeof(T) == 8)
              m |= (unsigned)((unsigned long long)key - tlo[t] < tcnt[t]) << t;
            else
              m |= (unsigned)((unsigned)key - (unsigned)tlo[t] < (unsigned)tcnt[t]) << t;
          }
        }
        dst[q] = (unsigned char)m;
      }
    }
  };
  fetch(kfirst + k0);
  store(0);
  fetch(kfirst + k0 + 1);
  const unsigned i = i0 + threadIdx.x;
  const bool in_x = i < ncx;
  const int tx = threadIdx.x;
  for (long long kl = k0; kl < k1; kl++) {
    const int cur = (int)((kl - k0) & 1), nxt = cur ^ 1;
    store(nxt); /* node plane kl + 1 */
    __syncthreads();
    if (kl + 1 < k1) fetch(kfirst + kl + 2);
#pragma unroll
    for (int jj = 0; jj < kClsY; jj++) {
      const unsigned j = j0 + jj;
      if (j >= ncy) break; /* the same for the whole block */
      const unsigned lo = (unsigned)bits[cur][jj][tx] | ((unsigned)bits[cur][jj][tx + 1] << 8) |
                          ((unsigned)bits[cur][jj + 1][tx] << 16) | ((unsigned)bits[cur][jj + 1][tx + 1] << 24);
      const unsigned hi = (unsigned)bits[nxt][jj][tx] | ((unsigned)bits[nxt][jj][tx + 1] << 8) |
                          ((unsigned)bits[nxt][jj + 1][tx] << 16) | ((unsigned)bits[nxt][jj + 1][tx + 1] << 24);
      const unsigned long long w = (unsigned long long)lo | ((unsigned long long)hi << 32);
      const size_t at = ((size_t)kl * ncy + j) * ncx + i;
#pragma unroll
      for (int t = 0; t < kMaxThr; t++) {
        if (t < nt && in_x) {
          const unsigned code = (unsigned)((((w >> t) & 0x0101010101010101ULL) * 0x0102040810204080ULL) >> 56);
          qb.codes[t][at] = (unsigned char)code;
        }
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kClsX, 6)
k_classify_queue(const ClsItem* __restrict__ items, int nitems, unsigned long long nunits,
                 unsigned long long* __restrict__ next) {
  pdl_enter();
  __shared__ unsigned char bits[2][kClsY + 1][kClsX + 1];
  __shared__ QueueBrick s_qb;
  __shared__ ThrSet s_ts;
  __shared__ int s_item;
  __shared__ unsigned long long s_unit;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long u = atomicAdd(next, 1ULL);
      s_unit = u;
      if (u < nunits) {
        int lo = 0, hi = nitems - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (items[mid].first <= u) lo = mid;
          else hi = mid - 1;
        }
        const ClsItem& it = items[lo];
        const unsigned long long r = u - it.first;
        const unsigned bx = (unsigned)(r % it.nbx), by = (unsigned)((r / it.nbx) % it.nby);
        const unsigned bz = (unsigned)(r / ((unsigned long long)it.nbx * it.nby));
        s_item = lo;
        s_qb.data = it.data;
        for (int t = 0; t < kMaxThr; t++) s_qb.codes[t] = it.out.codes[t];
        s_qb.nx = it.nx;
        s_qb.ny = it.ny;
        s_qb.kfirst = it.S.kfirst;
        s_qb.k0 = (long long)bz * it.S.cls_z;
        s_qb.k1 = min(s_qb.k0 + it.S.cls_z, it.S.nslices);
        s_qb.i0 = bx * kClsX;
        s_qb.j0 = by * kClsY;
        s_qb.ncx = (unsigned)(it.nx - 1);
        s_qb.ncy = (unsigned)(it.ny - 1);
        s_qb.nt = it.ts.n;
        s_ts = it.ts;
      }
    }
    __syncthreads();
    if (s_unit >= nunits) return;
    if (items[s_item].is_f32) classify_queue_brick<float>(s_qb, s_ts, bits);
    else classify_queue_brick<double>(s_qb, s_ts, bits);
    /* the brick ends with a barrier: thread 0 may overwrite s_qb */
  }
}

/*
 * k_classify_multi: the codes of up to kMaxThr objects of one field in one
 * pass over its nodes, one brick per block (the brick code of
 * k_classify_queue) -- the classification of fields whose rows TMA cannot
 * address (a row pitch that is not a multiple of 16 bytes, such as an odd
 * node count along x for a double field).
 */
template <typename T>
__global__ void __launch_bounds__(kClsX, 6)
k_classify_multi(const void* __restrict__ data, long long nx, long long ny, SlabDev S, ThrSet ts, CodeOut out) {
  pdl_enter();
  __shared__ unsigned char bits[2][kClsY + 1][kClsX + 1];
  /* the brick's description in shared memory, as k_classify_queue keeps it
     (in registers it spilled) */
  __shared__ QueueBrick s_qb;
  __shared__ ThrSet s_ts;
  if (threadIdx.x == 0) {
    s_qb.data = data;
    for (int t = 0; t < kMaxThr; t++) s_qb.codes[t] = out.codes[t];
    s_qb.nx = nx;
    s_qb.ny = ny;
    s_qb.kfirst = S.kfirst;
    s_qb.k0 = (long long)blockIdx.z * S.cls_z;
    s_qb.k1 = min(s_qb.k0 + S.cls_z, S.nslices);
    s_qb.i0 = blockIdx.x * kClsX;
    s_qb.j0 = blockIdx.y * kClsY;
    s_qb.ncx = (unsigned)(nx - 1);
    s_qb.ncy = (unsigned)(ny - 1);
    s_qb.nt = ts.n;
    s_ts = ts;
  }
  __syncthreads();
  classify_queue_brick<T>(s_qb, s_ts, bits);
}

/*
 * k_classify_tma: the same codes, with the node planes staged by TMA.  A
 * block owns kClsX x kClsY cells of kClsZ slices; each of its node planes
 * (TmaBox<T>::kX x (kClsY + 1) nodes, x from the tile start, so the copy starts on
 * a 16-byte boundary) is one cp.async.bulk.tensor copy into a ring of
 * TmaBox<T>::kStages shared-memory buffers, each completed on its own
 * mbarrier, so that many planes are in flight while the block turns the
 * current one into node bits and the previous pair into cell codes.  Fewer
 * stages let more blocks share an SM: the bytes in flight per SM stay about
 * the same, and more warps hide the latency of the bit work.  Copies beyond
 * the field read zeros (those nodes belong to no cell of the tile).  Every
 * wait is bounded: on a timeout the block records kErrClassifyTimeout, waits
 * (again bounded) for its own copies in flight, and returns.
 *
 * Node bits are warp ballots: per plane, row and threshold, word w holds the
 * nodes x = 32w .. 32w + 31 of the tile and word kClsX / 32 the node
 * x = kClsX.  A cell's code takes its two x-adjacent corners of each of its
 * four (row, plane) pairs with one funnel shift of two adjacent words.
 */
/* f64: 2 stages (19.7 KB, 11 blocks per SM) measured 0.326 ms on the 512^3
   two-level field, 3 stages 0.331, 4 stages 0.342; f32 blocks are limited
   by registers first */
constexpr int kTmaStagesF64 = 2;
constexpr int kTmaStagesF32 = 4;
constexpr int kTmaWaitLimit = 1 << 22;
constexpr int kClsWords = kClsX / 32 + 1;

template <typename T>
struct TmaBox {
  static constexpr int kX = sizeof(T) == 8 ? 130 : 132; /* >= kClsX + 1, a multiple of 16 bytes */
  static constexpr int kBytes = kX * (kClsY + 1) * (int)sizeof(T);
  static constexpr int kStride = (kBytes + 127) / 128 * 128; /* every stage starts on 128 bytes */
  static constexpr int kStages = sizeof(T) == 8 ? kTmaStagesF64 : kTmaStagesF32;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

/* bounded wait; false when the limit was reached */
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (int it = 0; it < kTmaWaitLimit; it++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <typename T, int NT>
__global__ void __launch_bounds__(kClsX)
k_classify_tma(const __grid_constant__ CUtensorMap tmap, FieldDev F, SlabDev S, ThrSet ts, CodeOut out,
               unsigned* __restrict__ err) {
  pdl_enter();
  static_assert(kClsX % 32 == 0 && kClsY + 1 <= 32, "classify tile: whole warps, a column of rows in one warp");
  using B = typename NodeBits<T>::type;
  constexpr int BX = TmaBox<T>::kX;
  constexpr int kStages = TmaBox<T>::kStages;
  __shared__ __align__(128) unsigned char stage_mem[kStages][TmaBox<T>::kStride];
  /* mask[plane parity][row][threshold][word] */
  __shared__ unsigned mask[2][kClsY + 1][NT][kClsWords];
  __shared__ __align__(8) unsigned long long bar[kStages];
  __shared__ int s_fail;
  const unsigned ncx = (unsigned)(F.nx - 1), ncy = (unsigned)(F.ny - 1);
  const int i0 = blockIdx.x * kClsX, j0 = blockIdx.y * kClsY;
  const long long k0 = (long long)blockIdx.z * S.cls_z;
  const long long k1 = min(k0 + S.cls_z, S.nslices);
  const int nplanes = (int)(k1 - k0) + 1; /* node planes k0 .. k1 of the slab */
  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int q = 0; q < kStages; q++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[q])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int p) { /* thread 0: plane p into stage p % kStages */
    const int st = p % kStages;
    const unsigned b = smem_u32(&bar[st]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(TmaBox<T>::kBytes)
                 : "memory");
    const int z = (int)(S.kfirst + k0 + p);
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(&stage_mem[st][0])), "l"(&tmap), "r"(i0), "r"(j0), "r"(z), "r"(b)
        : "memory");
  };
  if (threadIdx.x == 0)
    for (int p = 0; p < kStages && p < nplanes; p++) issue(p);
  const int tx = threadIdx.x, lane = tx & 31, warp = tx >> 5;
  const unsigned i = (unsigned)(i0 + tx);
  const bool in_x = i < ncx;
  for (int p = 0; p < nplanes; p++) {
    const int st = p % kStages;
    if (!mbar_wait(smem_u32(&bar[st]), (unsigned)((p / kStages) & 1))) s_fail = 1;
    /* also orders the previous plane's code reads before this plane's mask writes */
    __syncthreads();
    if (s_fail) {
      /* give up: record it, let the copies in flight land (bounded), return */
      if (threadIdx.x == 0) {
        atomicOr(err, kErrClassifyTimeout);
        for (int q = p; q < nplanes && q < p + kStages; q++)
          mbar_wait(smem_u32(&bar[q % kStages]), (unsigned)((q / kStages) & 1));
      }
      return;
    }
    /* node bits of plane p: warp w takes word w of every row; the node column
       x = kClsX goes to the last warp's lanes 0 .. kClsY */
    {
      const B(*vp)[BX] = reinterpret_cast<const B(*)[BX]>(&stage_mem[st][0]);
      unsigned(*mp)[NT][kClsWords] = mask[p & 1];
#pragma unroll
      for (int jj = 0; jj <= kClsY; jj++) {
        const B v = vp[jj][32 * warp + lane];
#pragma unroll
        for (int t = 0; t < NT; t++) {
          const unsigned m = __ballot_sync(0xFFFFFFFFu, node_above_thr(ts, t, v));
          if (lane == t) mp[jj][t][warp] = m;
        }
      }
      if (warp == kClsX / 32 - 1 && lane <= kClsY) {
        const B v = vp[lane][kClsX];
#pragma unroll
        for (int t = 0; t < NT; t++) mp[lane][t][kClsWords - 1] = node_above_thr(ts, t, v) ? 1u : 0u;
      }
    }
    __syncthreads();
    /* stage st is free again: refill it with plane p + kStages */
    if (threadIdx.x == 0 && p + kStages < nplanes) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(p + kStages);
    }
    if (p >= 1) {
      /* cell codes of slice k0 + p - 1 from the masks of planes p - 1 and p:
         bits 0-1 row jj of plane p - 1 (x, x + 1), 2-3 row jj + 1, 4-7 the
         same rows of plane p */
      const unsigned(*m0)[NT][kClsWords] = mask[(p - 1) & 1];
      const unsigned(*m1)[NT][kClsWords] = mask[p & 1];
      const int sh = lane;
      const long long kl = k0 + p - 1;
      unsigned a0[NT], a1[NT]; /* row jj of planes p - 1 and p, shifted to x */
#pragma unroll
      for (int t = 0; t < NT; t++) {
        a0[t] = __funnelshift_r(m0[0][t][warp], m0[0][t][warp + 1], sh);
        a1[t] = __funnelshift_r(m1[0][t][warp], m1[0][t][warp + 1], sh);
      }
#pragma unroll
      for (int jj = 0; jj < kClsY; jj++) {
        const unsigned j = (unsigned)(j0 + jj);
        if (j >= ncy) break; /* the same for the whole block */
        const size_t at = ((size_t)kl * ncy + j) * ncx + i;
#pragma unroll
        for (int t = 0; t < NT; t++) {
          const unsigned b0 = __funnelshift_r(m0[jj + 1][t][warp], m0[jj + 1][t][warp + 1], sh);
          const unsigned b1 = __funnelshift_r(m1[jj + 1][t][warp], m1[jj + 1][t][warp + 1], sh);
          const unsigned code = (a0[t] & 3u) | ((b0 & 3u) << 2) | ((a1[t] & 3u) << 4) | ((b1 & 3u) << 6);
          if (in_x) out.codes[t][at] = (unsigned char)code;
          a0[t] = b0;
          a1[t] = b1;
        }
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* the scan: segment offsets, then every cell's offsets                 */
/* ------------------------------------------------------------------ */
/* the thread's kScanItems codes, 4 per word (a code past the end reads as 0:
   no triangles, no vertices) */
__device__ __forceinline__ void load_scan_codes(const unsigned char* __restrict__ codes, long long base, long long n,
                                                unsigned wv[kScanItems / 4]) {
  if (base + kScanItems <= n) {
    /* 16-byte loads (base is a multiple of 32, the buffer 256-byte aligned) */
#pragma unroll
    for (int h = 0; h < kScanItems / 16; h++) {
      const uint4 v = *reinterpret_cast<const uint4*>(codes + base + 16 * h);
      wv[4 * h] = v.x;
      wv[4 * h + 1] = v.y;
      wv[4 * h + 2] = v.z;
      wv[4 * h + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int w = 0; w < kScanItems / 4; w++) {
      unsigned x = 0;
      for (int b = 0; b < 4; b++) {
        const long long c = base + 4 * w + b;
        if (c < n) x |= (unsigned)codes[c] << (8 * b);
      }
      wv[w] = x;
    }
  }
}

/*
 * The scan in one pass with decoupled look-back (Merrill and Garland,
 * "Single-pass Parallel Prefix Scan with Decoupled Look-back", NVIDIA
 * technical report NVR-2016-002).  Segment s's state word holds a packed
 * (triangle, vertex) sum in bits 0-61 and a status in bits 62-63: 1 = the
 * segment's own total, 2 = the total of segments 0..s.  A block takes the
 * next segment number from a ticket counter (the word after the states), so
 * every segment it waits for belongs to a block that is already running and
 * publishes its own total without waiting on anyone.  Warp 0 then walks back
 * 32 states at a time, adding own totals until it meets an inclusive one.
 * The walk is bounded: after kScanWaitLimit rounds the block records
 * kErrScanTimeout and goes on with what it has; its writes stay inside their
 * buffers whatever the prefix (the map is written only where it fits).
 */
constexpr unsigned long long kStAgg = 1ULL << 62, kStIncl = 2ULL << 62, kStValue = (1ULL << 62) - 1;
constexpr int kScanWaitLimit = 1 << 20;

__device__ __forceinline__ unsigned long long ld_state(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_state(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

/* the exclusive prefix of segment seg >= 1 (warp 0; every lane returns it) */
__device__ __forceinline__ unsigned long long look_back(const unsigned long long* state, long long seg,
                                                        unsigned* err) {
  const int lane = threadIdx.x & 31;
  unsigned long long prefix = 0;
  long long p = seg - 1; /* the nearest state not yet added */
  for (int rounds = 0;;) {
    const long long q = p - lane;
    const unsigned long long v = q >= 0 ? ld_state(state + q) : kStIncl; /* before segment 0: an inclusive 0 */
    const unsigned stt = (unsigned)(v >> 62);
    if (__any_sync(0xFFFFFFFFu, stt == 0)) {
      if (++rounds > kScanWaitLimit) {
        if (lane == 0) atomicOr(err, kErrScanTimeout);
        break;
      }
      __nanosleep(64);
      continue;
    }
    const unsigned incl = __ballot_sync(0xFFFFFFFFu, stt == 2);
    const int stop = incl ? __ffs(incl) - 1 : 31; /* lanes 0..stop are added */
    unsigned long long x = lane <= stop ? (v & kStValue) : 0ULL;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, d);
    prefix += x;
    if (incl) break;
    p -= 32;
  }
  return prefix;
}

/*
 * One block per segment: the segment's sum, its prefix by look-back, every
 * cell's vertex offsets (and triangle offsets when asked for), and the
 * segment's part of the triangle -> cell map when it fits tri_cap.  A thread
 * owns 32 consecutive cells; its offsets go through a per-warp shared-memory
 * stage (rows of kStagePitch words) so that every global store of a warp
 * covers 512 contiguous bytes.  The vertex offsets are stored relative to
 * the segment (VOffDev), so every warp stores them before the prefix is
 * known, warp 0 then looks back and stores the segment's first offset.  The
 * map goes through a shared list of the segment's triangles when they fit
 * it (positions relative to the segment, then a coalesced copy), else it is
 * written directly once the prefix is known.  The block of the last segment
 * writes the slab totals and the end entries (triangle offset of cell n,
 * vertex offset of cell n).
 */
constexpr int kFillList = 8192; /* triangles of a segment listed in shared memory (4 blocks per SM) */
constexpr int kStagePitch = 33;  /* words per staged row: conflict-free transposes */
constexpr size_t kScanWriteSmem =
    sizeof(unsigned) * (kScanThreads / 32) * 32 * kStagePitch + sizeof(unsigned short) * kFillList;

/* a warp's 1024 staged values plus `add` into dst[wbase ..] (cells past n are skipped) */
__device__ __forceinline__ void store_stage(unsigned* __restrict__ dst, const unsigned* stage, long long wbase,
                                            long long n, unsigned add) {
  const int lane = threadIdx.x & 31;
  if (wbase + 32 * kScanItems <= n) {
    /* each store instruction writes 512 contiguous bytes (lane L: cells
       4L .. 4L + 3 of a 128-cell chunk, all in one staged row; wbase is a
       multiple of 1024, dst 256-byte aligned) */
#pragma unroll 4
    for (int k = 0; k < 8; k++) {
      const int e = 128 * k + 4 * lane, row = e >> 5, col = e & 31;
      const unsigned* sr = stage + kStagePitch * row + col;
      reinterpret_cast<uint4*>(dst + wbase)[32 * k + lane] =
          make_uint4(sr[0] + add, sr[1] + add, sr[2] + add, sr[3] + add);
    }
  } else {
    for (int k = 0; k < 32; k++) {
      const long long c = wbase + 32 * k + lane;
      if (c < n) dst[c] = stage[kStagePitch * k + lane] + add;
    }
  }
}

/* a warp's 1024 staged values (below 2^16) into dst[wbase ..] as 16-bit
   words (cells past n are skipped) */
__device__ __forceinline__ void store_stage16(unsigned short* __restrict__ dst, const unsigned* stage, long long wbase,
                                              long long n) {
  const int lane = threadIdx.x & 31;
  if (wbase + 32 * kScanItems <= n) {
    /* each store instruction writes 512 contiguous bytes (lane L: cells
       8L .. 8L + 7 of a 256-cell chunk, all in one staged row; wbase is a
       multiple of 1024, dst 256-byte aligned) */
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int e = 256 * k + 8 * lane, row = e >> 5, col = e & 31;
      const unsigned* sr = stage + kStagePitch * row + col;
      reinterpret_cast<uint4*>(dst + wbase)[32 * k + lane] =
          make_uint4(sr[0] | (sr[1] << 16), sr[2] | (sr[3] << 16), sr[4] | (sr[5] << 16), sr[6] | (sr[7] << 16));
    }
  } else {
    for (int k = 0; k < 32; k++) {
      const long long c = wbase + 32 * k + lane;
      if (c < n) dst[c] = (unsigned short)stage[kStagePitch * k + lane];
    }
  }
}

__global__ void __launch_bounds__(kScanThreads, 4)
k_scan(const unsigned char* __restrict__ codes, long long n, long long nseg, unsigned long long* __restrict__ state,
       unsigned* __restrict__ offsets, VOffDev voff, unsigned long long* __restrict__ totals,
       unsigned* __restrict__ tri_cell, unsigned long long tri_cap, int want_offsets, unsigned* __restrict__ ovf,
       unsigned* __restrict__ err) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char scan_smem[];
  __shared__ unsigned long long s_warp[kScanThreads / 32];
  __shared__ unsigned s_cnt[256];
  __shared__ unsigned long long s_prefix;
  __shared__ unsigned s_seg;
  __shared__ unsigned s_first[kFillList / 32]; /* bit e: list slot e starts a cell's triangles */
  unsigned* stage_all = reinterpret_cast<unsigned*>(scan_smem);
  unsigned short* s_list = /* segment-local cell of each of the segment's triangles */
      reinterpret_cast<unsigned short*>(scan_smem + sizeof(unsigned) * (kScanThreads / 32) * 32 * kStagePitch);
  if (threadIdx.x == 0) s_seg = (unsigned)atomicAdd(state + nseg, 1ULL);
  load_count_lut(s_cnt);
  __syncthreads();
  const long long seg = s_seg;
  const long long c0 = seg * kScanTile;
  const long long base = c0 + (long long)threadIdx.x * kScanItems;
  unsigned wv[kScanItems / 4];
  load_scan_codes(codes, base, n, wv);
  /* per-thread sums in the 16-bit fields of the table entries (at most 384
     triangles and 224 vertices in a thread's 32 cells) */
  unsigned s32 = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) s32 += s_cnt[(wv[q >> 2] >> (8 * (q & 3))) & 255];
  const unsigned long long sum = packed_count(s32);
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
    unsigned long long w = lane < kScanThreads / 32 ? s_warp[lane] : 0ULL;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, d);
      if (lane >= d) w += y;
    }
    if (lane < kScanThreads / 32) s_warp[lane] = w;
    /* the segment's own total goes out at once */
    const unsigned long long agg = __shfl_sync(0xFFFFFFFFu, w, kScanThreads / 32 - 1);
    if (lane == 0) st_state(state + seg, (seg == 0 ? kStIncl : kStAgg) | agg);
  }
  __syncthreads();
  const unsigned long long agg = s_warp[kScanThreads / 32 - 1];
  const unsigned seg_tris = (unsigned)(agg & kTriMask);
  /* the thread's first offsets relative to the segment (both below 2^31) */
  const unsigned long long rel = (warp ? s_warp[warp - 1] : 0ULL) + incl - sum;
  const unsigned rel_t = (unsigned)(rel & kTriMask), rel_v = (unsigned)(rel >> 31);
  const bool can_list = seg_tris <= (unsigned)kFillList;
  if (can_list) {
    /* the shared list: each cell writes its first triangle's slot and marks
       it in s_first; a slot finds its cell's first slot there */
    for (unsigned e = threadIdx.x; e < (seg_tris + 31) / 32; e += kScanThreads) s_first[e] = 0u;
    __syncthreads();
  }
  unsigned* stage = stage_all + warp * 32 * kStagePitch;
  const long long wbase = c0 + (long long)warp * 32 * kScanItems; /* the warp's first cell */
  /* the vertex offsets (relative to the segment) and the list */
  auto fill_stage = [&]() {
    unsigned run = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; q++) {
      const unsigned cnt = s_cnt[(wv[q >> 2] >> (8 * (q & 3))) & 255];
      stage[kStagePitch * lane + q] = rel_v + (run >> 16);
      /* cells past n read as code 0: no triangles */
      if (can_list && (cnt & 0xFFFFu)) {
        const unsigned slot = rel_t + (run & 0xFFFFu);
        s_list[slot] = (unsigned short)(base + q - c0);
        atomicOr(&s_first[slot >> 5], 1u << (slot & 31));
      }
      run += cnt;
    }
  };
  /* the vertex offsets are relative to the segment: each warp stores its
     own at once; warp 0 then looks back */
  fill_stage();
  __syncwarp();
  store_stage16(voff.rel, stage, wbase, n);
  if (warp == 0) {
    unsigned long long prefix = 0;
    if (seg > 0) {
      prefix = look_back(state, seg, err);
      if (lane == 0) st_state(state + seg, kStIncl | ((prefix + agg) & kStValue));
    }
    if (lane == 0) {
      s_prefix = prefix;
      voff.seg[seg] = (unsigned)(prefix >> 31);
      if (seg == nseg - 1) {
        const unsigned long long tot = prefix + agg;
        totals[0] = tot & kTriMask;
        totals[1] = tot >> 31;
        offsets[n] = (unsigned)(tot & kTriMask);
        /* cell n: the end of this segment, or the start of segment nseg */
        voff.seg[nseg] = (unsigned)(tot >> 31);
        voff.rel[n] = n - c0 < kScanTile ? (unsigned short)(agg >> 31) : (unsigned short)0;
      }
    }
  }
  __syncthreads();
  const unsigned long long seg0 = s_prefix;
  const unsigned ta = (unsigned)(seg0 & kTriMask);
  const bool fill = (unsigned long long)ta + seg_tris <= tri_cap;
  /* a map that does not fit: the caller runs the scan again with a larger
     map, or, when the buffers were sized before the count was known (ovf
     given), renders the frame again */
  if (!fill && ovf && threadIdx.x == 0) atomicOr(ovf, kOvfTriangles);
  if (want_offsets || (fill && !can_list)) {
    /* triangle offsets (inspection) and the direct map: the prefix is known */
    __syncwarp();
    unsigned run = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; q++) {
      const unsigned cnt = s_cnt[(wv[q >> 2] >> (8 * (q & 3))) & 255];
      const unsigned t0 = ta + rel_t + (run & 0xFFFFu);
      stage[kStagePitch * lane + q] = t0;
      if (fill && !can_list && base + q < n)
        for (unsigned r = 0; r < (cnt & 0xFFFFu); r++) tri_cell[t0 + r] = (unsigned)(base + q) | (r << kTcRankShift);
      run += cnt;
    }
    __syncwarp();
    if (want_offsets) store_stage(offsets, stage, wbase, n, 0u);
  }
  if (fill && can_list) {
    /* the list was complete at the barrier above */
    for (unsigned e = threadIdx.x; e < seg_tris; e += kScanThreads) {
      /* the cell's first slot: the last marked slot at or before e (a cell
         has at most 12 triangles and slot 0 starts one, so it lies in e's
         word of s_first or the word before); the rank is the distance */
      const unsigned wd = e >> 5;
      unsigned m = s_first[wd] & (0xFFFFFFFFu >> (31 - (e & 31)));
      unsigned first = 32 * wd + 31 - __clz(m);
      if (m == 0u && wd > 0) first = 32 * (wd - 1) + 31 - __clz(s_first[wd - 1]);
      tri_cell[ta + e] = ((unsigned)c0 + s_list[first]) | ((e - first) << kTcRankShift);
    }
  }
}

/* ------------------------------------------------------------------ */
/* exact triangles on demand (triangulate.c:40-93)                      */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ d3 corner_pos(const FieldDev& F, long long i, long long j, long long k, int c) {
  const long long ii = i + (c & 1), jj = j + ((c >> 1) & 1), kk = k + (c >> 2);
  if (F.nodes) {
    const double* p = F.nodes + 3 * ((kk * F.ny + jj) * F.nx + ii);
    return {p[0], p[1], p[2]};
  }
  return {F.gx[ii], F.gy[jj], F.gz[kk]};
}

/* triangulate.c:40-73 */
__device__ __forceinline__ d3 interpolate(double vt, d3 p0, double v0, d3 p1, double v1) {
  const double dv = dsub(v1, v0);
  if (abs_lt_1e8(dv)) return p0;
  const double f = ddiv(dsub(vt, v0), dv);
  return v_add(p0, v_mul(f, v_sub(p1, p0)));
}

/* value at corner c of cell (i, j, k) */
__device__ __forceinline__ double corner_value(const FieldDev& F, long long i, long long j, long long k, int c) {
  const long long idx = ((k + (c >> 2)) * F.ny + j + ((c >> 1) & 1)) * F.nx + i + (c & 1);
  return F.is_f32 ? (double)__ldg(static_cast<const float*>(F.data) + idx)
                  : __ldg(static_cast<const double*>(F.data) + idx);
}

/* corner values and code of cell (i, j, k), element type chosen at run time */
__device__ __forceinline__ unsigned cell_code_any(const FieldDev& F, long long i, long long j, long long k,
                                                  double vals[8]) {
  return F.is_f32 ? cell_code<float>(F, i, j, k, vals) : cell_code<double>(F, i, j, k, vals);
}

/*
 * The reference's triangle (vertices in winding order) for emission index t
 * of the slab, recomputed from the field: the same operations as k_emit's
 * FP32 estimate stands for.  Returns the cube-edge ids in *edges.
 */
__device__ __forceinline__ void exact_vertices(const Geo& G, long long t, d3 v[3]) {
  const unsigned tc = G.tri_cell[t];
  const unsigned c = tc & kTcCellMask, r = tc >> kTcRankShift;
  unsigned ui, uj, ukl;
  cell_ijk(G.F, c, ui, uj, ukl);
  const long long i = ui, j = uj, k = G.S.kfirst + ukl;
  const unsigned code = G.codes[c];
  const unsigned long long e = __ldg(G.lut + code * 12 + r);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const int a = (int)((e >> (6 * q)) & 7), b = (int)((e >> (6 * q + 3)) & 7);
    v[q] = interpolate(G.F.threshold, corner_pos(G.F, i, j, k, a), corner_value(G.F, i, j, k, a),
                       corner_pos(G.F, i, j, k, b), corner_value(G.F, i, j, k, b));
  }
}

/* triangulate.c:75-93 and normal.c:39-40: face normal, area, area * face normal */
__device__ __forceinline__ void face_normal(const d3 v[3], d3& fn, double& area, d3& wn) {
  fn = v_cross(v_sub(v[1], v[0]), v_sub(v[2], v[0]));
  area = dsqrt(v_dot(fn, fn));
  fn = v_mul(drcp(area), fn);
  wn = v_mul(area, fn);
}

/* ------------------------------------------------------------------ */
/* k_emit: single-precision triangles with certified bounds             */
/* ------------------------------------------------------------------ */
/* x >= 0 (or -1, -2) as a bfloat16 no smaller than x (bits of the high half) */
__device__ __forceinline__ unsigned bf16_up(float x) {
  const unsigned b = __float_as_uint(x);
  return (b >> 16) + ((b & 0xFFFFu) != 0u && !(b >> 31) ? 1u : 0u);
}
__device__ __forceinline__ float bf16_value(unsigned h) { return __uint_as_float(h << 16); }

/* a field value as a float and the bound on its conversion error */
__device__ __forceinline__ float value_f(double v, float& e) {
  const float a = to_f(v); /* truncation: < 2u |a|, or < 2^-126 when flushed */
  e = 2.f * kU32 * fabsf(a) + 1.2e-38f;
  return a;
}
__device__ __forceinline__ float value_f(float v, float& e) {
  e = 0.f;
  return v;
}

/*
 * The interpolation parameter f = (vt - v0) / (v1 - v0) of triangulate.c:40-73
 * in FP32 with a bound e_f on its distance to the reference's value.
 * Returns 1 (f valid), 0 (the reference keeps p0: |v1 - v0| < 1e-8) or -1
 * (the bounds cannot decide that test).
 *   double fields: the two differences are formed in FP64 exactly as the
 *     reference forms them, then truncated to float (2u each), so the 1e-8
 *     test is exact and cancellation costs no accuracy (k_vertices: issue
 *     bound, two FP64 subtractions cost fewer slots than float pairs);
 *   float fields: the values are exact floats and the differences are FP32
 *     (u each), with the 1e-8 test decided by the bounds.
 * interp_shade below is the FP64-free form for double fields.
 */
__device__ __forceinline__ int interp_param(double vt, float, float, double v0, double v1, float& f, float& e_f) {
  const double dvd = dsub(v1, v0);
  if (abs_lt_1e8(dvd)) return 0;
  const float dv = to_f(dvd), dt = to_f(dsub(vt, v0));
  const float adv = fabsf(dv);
  const float e_dv = 2.f * kU32 * adv + 1.2e-38f, e_dt = 2.f * kU32 * fabsf(dt) + 1.2e-38f;
  if (!(adv > 1e-30f) || adv > 1e30f) return -1;
  const float rdv = __fdividef(1.f, adv); /* 2 ulp on [1e-30, 1e30] */
  const float xr = e_dv * rdv;
  f = __fdividef(dt, dv);
  const float fmax_ = 1.01f * (fabsf(dt) + e_dt) * rdv * (1.f + 1.02f * xr);
  e_f = 1.1f * (1.01f * (e_dt + fmax_ * e_dv) * rdv + 4.f * kU32 * fabsf(f));
  return 1;
}
__device__ __forceinline__ int interp_param(double, float vt, float e_vt, float v0, float v1, float& f, float& e_f) {
  const float dv = v1 - v0;
  const float e_dv = 1.01f * kU32 * fabsf(dv);
  const float adv = fabsf(dv);
  if (!(adv - e_dv > 1.00001e-8f)) return adv + e_dv < 0.99999e-8f ? 0 : -1;
  if (adv > 1e30f) return -1;
  /* 1 / |dv| to 2 ulp; 1 / (|dv| - e_dv) <= rdv (1 + 1.02 x) for x = e_dv rdv < 0.01 */
  const float rdv = __fdividef(1.f, adv);
  const float xr = e_dv * rdv;
  if (!(xr < 0.01f)) return -1;
  const float dt = vt - v0;
  const float e_dt = e_vt + 1.01f * kU32 * fabsf(dt);
  f = __fdividef(dt, dv); /* 2 ulp */
  /* |dt/dv - DT/DV| <= (e_dt + |DT/DV| e_dv) / |dv|, |DT/DV| <= fmax */
  const float fmax_ = 1.01f * (fabsf(dt) + e_dt) * rdv * (1.f + 1.02f * xr);
  e_f = 1.1f * (1.01f * (e_dt + fmax_ * e_dv) * rdv + 4.f * kU32 * fabsf(f));
  return 1;
}

/*
 * A double as an unevaluated float pair hi + lo, by integer operations (the
 * FP64 pipe stays free): hi carries the top 24 significand bits, lo up to 24
 * of the next 29, both truncated; |hi + lo - v| <= 2^-47 |v| + 2^-126.  False
 * for NaN, infinities and magnitudes beyond float.
 */
__device__ __forceinline__ bool split_bits(unsigned long long b, float& hi, float& lo) {
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int ex = (int)((b >> 52) & 0x7FF);
  hi = lo = 0.f;
  if (ex == 0x7FF || ex - 1023 > 127) return false;
  const int fe = ex - 1023 + 127;
  if (fe <= 0) { /* below 2^-126: flushed */
    hi = __uint_as_float(sign);
    return true;
  }
  hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
  /* lo = rem 2^(ex - 1075), rem the low 29 bits, truncated to 24 significant
     bits (an error below 2^-47 |v|); flushed to 0 below 2^-126 */
  const unsigned rem = (unsigned)(b & 0x1FFFFFFFu);
  if (rem == 0) return true;
  const int lz = __clz(rem);                      /* 3 .. 31 */
  const int le = (31 - lz) + (ex - 1075) + 127;   /* biased exponent of lo */
  if (le <= 0) return true;
  lo = __uint_as_float(sign | ((unsigned)le << 23) | ((rem << (lz + 1)) >> 9));
  return true;
}

__device__ __forceinline__ bool split_f(double v, float& hi, float& lo) {
  return split_bits((unsigned long long)__double_as_longlong(v), hi, lo);
}

/* s + t = a - b exactly (Knuth's two-sum; no fused operations in this build) */
__device__ __forceinline__ void two_diff(float a, float b, float& s, float& t) {
  s = a - b;
  const float bb = s - a;
  t = (a - (s - bb)) - (b + bb);
}

/* (ah + al) - (bh + bl) in FP32 and a bound on its distance to the
   difference of the two doubles the pairs stand for */
__device__ __forceinline__ float pair_diff(float ah, float al, float bh, float bl, float& e) {
  float s, t;
  two_diff(ah, bh, s, t);
  const float dl = al - bl, u = t + dl, d = s + u;
  e = 1.01f * (kU32 * (fabsf(dl) + fabsf(u) + fabsf(d)) + 1.43e-14f * (fabsf(ah) + fabsf(bh)) + 3e-38f);
  return d;
}

/* the threshold in the forms the shading pass uses */
struct ThrF {
  float vt, e_vt; /* rounded to float, with its bound (float fields) */
  float hi, lo;   /* split (double fields) */
};
__device__ __forceinline__ ThrF thr_f(double t) {
  ThrF r;
  r.vt = value_f(t, r.e_vt);
  if (!split_f(t, r.hi, r.lo)) r.hi = r.lo = __int_as_float(0x7fc00000);
  return r;
}

/* interp_param for the shading pass, FP32 operations only: for a double
   field the differences are formed from float pairs (pair_diff), accurate to
   a few float ulps of the differences themselves */
__device__ __forceinline__ int interp_shade(const FieldDev& F, const ThrF& th, long long v0, long long v1, float& f,
                                            float& e_f) {
  float h0, l0, h1, l1;
  if (!split_bits((unsigned long long)v0, h0, l0) || !split_bits((unsigned long long)v1, h1, l1) || th.hi != th.hi)
    return -1;
  float e_dv, e_dt;
  const float dv = pair_diff(h1, l1, h0, l0, e_dv);
  const float adv = fabsf(dv);
  /* triangulate.c:40-73: |v1 - v0| < 1e-8 keeps p0 */
  if (!(adv - e_dv > 1.00001e-8f)) return adv + e_dv < 0.99999e-8f ? 0 : -1;
  if (adv > 1e30f) return -1;
  const float rdv = __fdividef(1.f, adv);
  const float xr = e_dv * rdv;
  if (!(xr < 0.01f)) return -1;
  const float dt = pair_diff(th.hi, th.lo, h0, l0, e_dt);
  f = __fdividef(dt, dv); /* 2 ulp */
  const float fmax_ = 1.01f * (fabsf(dt) + e_dt) * rdv * (1.f + 1.02f * xr);
  e_f = 1.1f * (1.01f * (e_dt + fmax_ * e_dv) * rdv + 4.f * kU32 * fabsf(f));
  return 1;
}
__device__ __forceinline__ int interp_shade(const FieldDev& F, const ThrF& th, float v0, float v1, float& f,
                                            float& e_f) {
  return interp_param(F.threshold, th.vt, th.e_vt, v0, v1, f, e_f);
}

/* a corner value as the shading pass takes it: a double's bit pattern, a float itself */
template <typename T>
struct ShadeVal;
template <>
struct ShadeVal<double> {
  typedef long long type;
  static __device__ __forceinline__ long long load(const double* f, long long idx) { return ld_bits(f + idx); }
};
template <>
struct ShadeVal<float> {
  typedef float type;
  static __device__ __forceinline__ float load(const float* f, long long idx) { return __ldg(f + idx); }
};


/*
 * FP32 estimate of one vertex (triangulate.c:40-73) relative to the camera,
 * q = vertex - camera, with a bound per component on the distance to the
 * reference's FP64 value: p = p0 + f (p1 - p0) with f from interp_param.
 * Returns false when interp_param cannot decide the reference's 1e-8 test
 * (the triangle then takes the FP64 path).
 */
template <typename T>
__device__ __forceinline__ bool vertex_q(const SceneDev& s, const FieldDev& F, const ThrF& th, const float x0[3],
                                         T v0, const float x1[3], T v1, float ce, float q[3], float eq[3]) {
  /* x0, x1: corner coordinates rounded to float with error <= ce u |x| */
  const float pc[3] = {s.f_cam[0], s.f_cam[1], s.f_cam[2]};
  float f = 0.f, e_f = 0.f;
  const int st = interp_param(F.threshold, th.vt, th.e_vt, v0, v1, f, e_f);
  if (st < 0) return false;
  if (st == 0) {
    /* the reference keeps p0 itself */
#pragma unroll
    for (int i = 0; i < 3; i++) {
      q[i] = x0[i] - pc[i];
      eq[i] = 1.1f * kU32 * (ce * fabsf(x0[i]) + fabsf(pc[i]) + fabsf(q[i])) + 1e-30f;
    }
    return true;
  }
  const float af = fabsf(f);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    /* fused multiply-adds round once where the bound allows for two
       roundings, so every bound below still holds */
    const float d = x1[i] - x0[i];
    const float p = __fmaf_rn(f, d, x0[i]);
    q[i] = p - pc[i];
    const float cx0 = ce * fabsf(x0[i]);
    const float inner = __fmaf_rn(2.2f, fabsf(d), __fmaf_rn(ce, fabsf(x1[i]), cx0));
    const float ep = __fmaf_rn(e_f, fabsf(d), kU32 * __fmaf_rn(af, inner, cx0 + fabsf(p)));
    eq[i] = __fmaf_rn(1.1f, __fmaf_rn(kU32, fabsf(pc[i]) + fabsf(q[i]), ep), 1e-30f);
  }
  return true;
}

/* corner coordinates as floats, and the bound factor of their rounding */
__device__ __forceinline__ float corner_pos_f(const FieldDev& F, long long i, long long j, long long k, int c,
                                              float x[3]) {
  const long long ii = i + (c & 1), jj = j + ((c >> 1) & 1), kk = k + (c >> 2);
  if (F.nodes) {
    const double* p = F.nodes + 3 * ((kk * F.ny + jj) * F.nx + ii);
    x[0] = to_f(p[0]);
    x[1] = to_f(p[1]);
    x[2] = to_f(p[2]);
    return 2.f;
  }
  x[0] = __ldg(F.gxf + ii);
  x[1] = __ldg(F.gyf + jj);
  x[2] = __ldg(F.gzf + kk);
  return 1.f;
}

/*
 * Screen projection in single precision from q (bounded per component).
 * Uses the identity (exact in real arithmetic) of project.c:9-67
 *   x = [(cam - centre) . lx + D (q . lx) / (n . q)] / (lx . lx),
 *   D = n . centre - n . cam,  depth = n . q,  t = D / (n . q)
 * Each FP32 dot product a . q is within sum|a_i| eq_i + 4.2 u sum|a_i q_i|
 * of the real one.  Returns 1 = certainly projects, 0 = certainly fails
 * (render.c:62-72 drops the triangle), -1 = too close to a threshold of
 * project.c:39-46.
 */
__device__ __forceinline__ int project_f(const SceneDev& s, const float q[3], const float eq[3], float ref_eps,
                                         float& X, float& Y, float& Z, float& exy, float& ez) {
  const float ax = fabsf(q[0]), ay = fabsf(q[1]), az = fabsf(q[2]);
  /* dot products and their bounds with fused multiply-adds: one rounding
     fewer per step than the unfused sums the bounds allow for */
  const float nq = __fmaf_rn(s.f_n[2], q[2], __fmaf_rn(s.f_n[1], q[1], s.f_n[0] * q[0]));
  const float lq = __fmaf_rn(s.f_lx[2], q[2], __fmaf_rn(s.f_lx[1], q[1], s.f_lx[0] * q[0]));
  const float mq = __fmaf_rn(s.f_ly[2], q[2], __fmaf_rn(s.f_ly[1], q[1], s.f_ly[0] * q[0]));
  auto bound = [&](const float a[3]) {
    const float se = __fmaf_rn(fabsf(a[2]), eq[2], __fmaf_rn(fabsf(a[1]), eq[1], fabsf(a[0]) * eq[0]));
    const float sq = __fmaf_rn(fabsf(a[2]), az, __fmaf_rn(fabsf(a[1]), ay, fabsf(a[0]) * ax));
    return __fmaf_rn(4.2f * kU32, sq, se);
  };
  const float e_nq = bound(s.f_n), e_lq = bound(s.f_lx), e_mq = bound(s.f_ly);
  const float anq = fabsf(nq);
  Z = nq;
  ez = 1.1f * e_nq + 1e-30f;
  if (!isfinite(nq) || !isfinite(lq) || !isfinite(mq)) return -1;
  /* project.c:39-46: |nr| < 1e-8 or t outside (0, 1) => the point is dropped */
  if (anq + e_nq < 0.99e-8f) return 0;
  if (anq - e_nq <= 1.01e-8f || anq > 1e30f) return -1;
  /* r = 1 / nq to 2 ulp (__fdividef, |nq| in [1e-8, 1e30]); with
     x = e_nq |r| < 0.01, 1 / (|nq| - e_nq) <= |r| (1 + 1.02 x) (1 + 4u) */
  const float r = __fdividef(1.f, nq);
  const float x = e_nq * fabsf(r);
  if (!(x < 0.01f)) return -1;
  const float rin = 1.01f * fabsf(r) * (1.f + 1.02f * x);
  const float t = s.f_dq * r;
  const float et = fabsf(t) * (1.02f * x + 6.f * kU32) + 1e-30f;
  if (t + et < 0.f || t - et > 1.f) return 0;
  if (t - et <= 0.f || t + et >= 1.f) return -1;
  const float rx = lq * r, ry = mq * r;
  const float erx = __fmaf_rn(__fmaf_rn(fabsf(rx), e_nq, e_lq), rin, 6.f * kU32 * fabsf(rx));
  const float ery = __fmaf_rn(__fmaf_rn(fabsf(ry), e_nq, e_mq), rin, 6.f * kU32 * fabsf(ry));
  X = __fmaf_rn(s.f_bx, rx, s.f_ax);
  Y = __fmaf_rn(s.f_by, ry, s.f_ay);
  const float ex = __fmaf_rn(fabsf(s.f_bx), erx,
                             __fmaf_rn(kU32, __fmaf_rn(2.f, fabsf(s.f_bx * rx), fabsf(s.f_ax)) + fabsf(X), ref_eps));
  const float ey = __fmaf_rn(fabsf(s.f_by), ery,
                             __fmaf_rn(kU32, __fmaf_rn(2.f, fabsf(s.f_by * ry), fabsf(s.f_ay)) + fabsf(Y), ref_eps));
  exy = 1.1f * fmaxf(ex, ey);
  return 1;
}

/* inspection: every triangle's exact vertices, face normal, area and weighted normal */
__global__ void __launch_bounds__(256) k_exact_all(Geo G, const unsigned long long* __restrict__ total_p, TriDev tri) {
  pdl_enter();
  const long long T_ = (long long)*total_p;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T_;
       t += (long long)gridDim.x * blockDim.x) {
    d3 v[3], fn, wn;
    double area;
    exact_vertices(G, t, v);
    face_normal(v, fn, area, wn);
    tri.wn[0][t] = wn.x;
    tri.wn[1][t] = wn.y;
    tri.wn[2][t] = wn.z;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      tri.vert[3 * q + 0][t] = v[q].x;
      tri.vert[3 * q + 1][t] = v[q].y;
      tri.vert[3 * q + 2][t] = v[q].z;
    }
    tri.dbg_fn[3 * t + 0] = fn.x;
    tri.dbg_fn[3 * t + 1] = fn.y;
    tri.dbg_fn[3 * t + 2] = fn.z;
    tri.dbg_area[t] = area;
  }
}

/* ------------------------------------------------------------------ */
/* vertex normals (normal.c:6-165)                                      */
/* ------------------------------------------------------------------ */
/*
 * Sum of area * face normal over the triangles of the cells sharing cube
 * edge `e` of cell `c`, visited in the reference's order (ascending cell,
 * then triangle order), then normalised.  wn must be present for every
 * triangle touching the edge.
 */
__device__ __forceinline__ d3 vertex_normal(long long c, int e, long long ncx, long long ncy,
                                            const unsigned* __restrict__ offsets, const TriDev& tri) {
  d3 sum = {0., 0., 0.};
  const int nn = c_nb_count[e];
  for (int q = 0; q < nn; q++) {
    const long long nc = c + (long long)c_nb[e][q][0] * ncx * ncy + (long long)c_nb[e][q][1] * ncx +
                         (long long)c_nb[e][q][2];
    const unsigned le = (unsigned)c_nb[e][q][3];
    const unsigned u0 = offsets[nc], u1 = offsets[nc + 1];
    for (unsigned u = u0; u < u1; u++) {
      const unsigned om = tri.meta[u];
      if (((om & 31) == le) || (((om >> 5) & 31) == le) || (((om >> 10) & 31) == le)) {
        const d3 w = {tri.wn[0][u], tri.wn[1][u], tri.wn[2][u]};
        sum = v_add(sum, w);
      }
    }
  }
  return v_normalise(sum);
}

/* inspection: every rendered triangle's vertex normals */
__global__ void __launch_bounds__(256)
k_normals(FieldDev F, SlabDev S, const unsigned* __restrict__ offsets, const unsigned* __restrict__ tri_cell,
          const unsigned long long* __restrict__ total_p, TriDev tri) {
  pdl_enter();
  const long long T_ = (long long)*total_p;
  const long long ncx = F.nx - 1, ncy = F.ny - 1;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T_;
       t += (long long)gridDim.x * blockDim.x) {
    const unsigned meta = tri.meta[t];
    if (!(meta & kMetaRendered)) continue;
    const long long c = tri_cell[t] & kTcCellMask;
#pragma unroll 1
    for (int m = 0; m < 3; m++) {
      const d3 n = vertex_normal(c, (meta >> (5 * m)) & 31, ncx, ncy, offsets, tri);
      tri.vn[3 * m + 0][t] = n.x;
      tri.vn[3 * m + 1][t] = n.y;
      tri.vn[3 * m + 2][t] = n.z;
    }
  }
}

/* ------------------------------------------------------------------ */
/* raster: exact fragment arithmetic (render.c:48-163)                  */
/* ------------------------------------------------------------------ */
/* the reference's projected triangle, bounding box and inverse area */
struct ExactTri {
  d3 v0, v1, v2;
  long long imin, imax, jmin, jmax;
  double area;
  double area_inv;
};

/* the projected triangle and its inverse area (the box is left unset) */
__device__ __forceinline__ bool exact_tri_core(const SceneDev& s, const d3 w[3], ExactTri& x) {
  if (!project(s, w[0], x.v0) || !project(s, w[1], x.v1) || !project(s, w[2], x.v2)) return false;
  x.area = edge_fn(x.v0, x.v1, x.v2);
  x.area_inv = drcp(x.area < 0. ? fmin(x.area, -1.e-16) : fmax(x.area, +1.e-16));
  return true;
}

/* the reference's bounding box of a projected triangle */
__device__ __forceinline__ void exact_box(const SceneDev& s, ExactTri& x) {
  const long long W = s.width, H = s.height;
  const long long xmin = (long long)dsub(dmul(dadd(0.5, fmin(x.v0.x, fmin(x.v1.x, x.v2.x))), (double)W), 1.);
  const long long xmax = (long long)dadd(dmul(dadd(0.5, fmax(x.v0.x, fmax(x.v1.x, x.v2.x))), (double)W), 1.);
  const long long ymin = (long long)dsub(dmul(dadd(0.5, fmin(x.v0.y, fmin(x.v1.y, x.v2.y))), (double)H), 1.);
  const long long ymax = (long long)dadd(dmul(dadd(0.5, fmax(x.v0.y, fmax(x.v1.y, x.v2.y))), (double)H), 1.);
  x.imin = min(W - 1, max(0LL, xmin));
  x.imax = min(W - 1, max(0LL, xmax));
  x.jmin = min(H - 1, max(0LL, ymin));
  x.jmax = min(H - 1, max(0LL, ymax));
}

__device__ __forceinline__ bool exact_tri(const SceneDev& s, const d3 w[3], ExactTri& x) {
  if (!exact_tri_core(s, w, x)) return false;
  exact_box(s, x);
  return true;
}

/* the reference's barycentric weights at pixel (i, j) of its box; false when
   outside the triangle */
__device__ __forceinline__ bool exact_weights_in(const ExactTri& x, long long i, long long j, const double* xs,
                                                 const double* ys, double& w0, double& w1, double& w2) {
  const d3 v3 = {xs[i], ys[j], 0.};
  w0 = dmul(x.area_inv, edge_fn(x.v1, x.v2, v3));
  w1 = dmul(x.area_inv, edge_fn(x.v2, x.v0, v3));
  w2 = dmul(x.area_inv, edge_fn(x.v0, x.v1, v3));
  return !(w0 < -1.e-8 || w1 < -1.e-8 || w2 < -1.e-8);
}

/* the same at any pixel; false when outside the box or the triangle */
__device__ __forceinline__ bool exact_weights(const ExactTri& x, long long i, long long j, const double* xs,
                                              const double* ys, double& w0, double& w1, double& w2) {
  if (i < x.imin || i > x.imax || j < x.jmin || j > x.jmax) return false;
  return exact_weights_in(x, i, j, xs, ys, w0, w1, w2);
}

__device__ __forceinline__ double exact_depth(const ExactTri& x, double w0, double w1, double w2) {
  return drcp(dadd(dadd(ddiv(w0, x.v0.z), ddiv(w1, x.v1.z)), ddiv(w2, x.v2.z)));
}

__device__ __forceinline__ unsigned long long order_of(const Geo& G, unsigned long long order_base, long long t) {
  const unsigned tc = G.tri_cell[t];
  return order_base + 12ULL * (tc & kTcCellMask) + (tc >> kTcRankShift);
}

/* the winning fragment's exact weights for shading (see RasterDev::winfo) */
__device__ __forceinline__ void keep_weights(const RasterDev& R, long long p, unsigned long long order, double w0,
                                             double w1, double w2) {
  const unsigned long long tag = (order << 24) | R.epoch;
  ulonglong2* w = R.winfo + 3 * p;
  store128_atomic(w, (unsigned long long)__double_as_longlong(w0), tag);
  store128_atomic(w + 1, (unsigned long long)__double_as_longlong(w1), tag);
  store128_atomic(w + 2, (unsigned long long)__double_as_longlong(w2), tag);
}

/*
 * One candidate fragment through the reference's test and the (depth, order)
 * z-buffer.  Candidates come from the cover list only: triangles whose area
 * is certainly not clamped, so a pixel that passes the weight test lies in
 * the triangle's extent and so inside the reference's box, whose margins are
 * a pixel wide; the box is not computed (CHECK: it is, and a pixel outside it
 * counts as a violation and is not drawn).
 */
template <bool CHECK>
__device__ __forceinline__ void exact_fragment(const Geo& G, const SceneDev& s, long long t, long long i, long long j,
                                               const RasterDev& R, unsigned long long order_base,
                                               unsigned* checks) {
  d3 w[3];
  exact_vertices(G, t, w);
  ExactTri x;
  if (!exact_tri_core(s, w, x)) return;
  double w0, w1, w2;
  if (!exact_weights_in(x, i, j, R.xs, R.ys, w0, w1, w2)) return;
  if (CHECK) {
    exact_box(s, x);
    if (i < x.imin || i > x.imax || j < x.jmin || j > x.jmax) {
      atomicAdd(checks + 2, 1u);
      return;
    }
  }
  const double dist0 = exact_depth(x, w0, w1, w2);
  const unsigned long long order = order_of(G, order_base, t);
  const long long p = j * s.width + i;
  if (slot_max(R.canvas + p, depth_key(dist0), order << 24, R.zerr)) keep_weights(R, p, order, w0, w1, w2);
}

/* ------------------------------------------------------------------ */
/* k_cover: single-precision coverage / depth filter                   */
/* ------------------------------------------------------------------ */
/*
 * Per rendered triangle, every pixel whose centre can lie in the triangle
 * is classified with certified FP32 bounds:
 *   certainly outside        -> dropped
 *   certainly inside         -> raises the pixel's depth floor (zlo) to a
 *                               certain lower bound of its depth, and is a
 *                               candidate
 *   undecided                -> candidate
 * A candidate carries an upper bound of its depth; k_exact drops it when
 * that bound is below the final floor (a certainly drawn fragment is nearer,
 * so it cannot win), and runs the reference's arithmetic otherwise.
 */
struct EdgeF {
  float ax, ay, dby, dbx, e_dby, e_dbx;
};

__device__ __forceinline__ EdgeF edge_f(float ax, float ay, float bx, float by, float eps) {
  EdgeF E;
  E.ax = ax;
  E.ay = ay;
  E.dby = by - ay;
  E.dbx = bx - ax;
  E.e_dby = 2.f * eps + kU32 * fabsf(E.dby);
  E.e_dbx = 2.f * eps + kU32 * fabsf(E.dbx);
  return E;
}

/* render.c:38-46 at a point known to +-e_p, edge vertex a known to +-eps_a; value and error bound */
__device__ __forceinline__ float edge_eval(const EdgeF& E, float px, float py, float e_p, float eps_a, float& err) {
  const float u = px - E.ax, v = py - E.ay;
  const float eu = __fmaf_rn(kU32, fabsf(u), e_p + eps_a), ev = __fmaf_rn(kU32, fabsf(v), e_p + eps_a);
  /* u dby - v dbx with one rounding of the product v dbx and one of the
     fused result; the bound keeps a term for a rounding of u dby as well */
  const float p2 = v * E.dbx;
  const float e = __fmaf_rn(u, E.dby, -p2);
  const float pr = fabsf(u) * fabsf(E.dby) + fabsf(p2) + fabsf(e);
  float b = __fmaf_rn(fabsf(u), E.e_dby, kU32 * pr);
  b = __fmaf_rn(fabsf(E.dby) + E.e_dby, eu, b);
  b = __fmaf_rn(fabsf(v), E.e_dbx, b);
  b = __fmaf_rn(fabsf(E.dbx) + E.e_dbx, ev, b);
  err = 1.25f * b;
  return e;
}

constexpr float kWOut = -1.0e-8f * (1.f + 1e-5f); /* certainly below -1e-8 */
constexpr float kWIn = -1.0e-8f * (1.f - 1e-5f);  /* certainly above -1e-8 */

/*
 * Block-wide reservation of list slots for two lists at once: every thread of
 * the block calls it at the same point with its item counts (block totals
 * below 65536 per list).  One global atomic per block and list instead of
 * one per warp: the list counters are single addresses that every block
 * appends to, and same-address atomics serialise in the L2.
 */
template <int kThreads>
__device__ __forceinline__ void block_reserve2(unsigned long long* count0, unsigned n0, unsigned long long* count1,
                                               unsigned n1, unsigned long long& r0, unsigned long long& r1) {
  __shared__ unsigned s_w[kThreads / 32];
  __shared__ unsigned long long s_b[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned x = n0 | (n1 << 16);
  unsigned incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) {
      const unsigned v = s_w[w];
      s_w[w] = run;
      run += v;
    }
    const unsigned t0 = run & 0xFFFFu, t1 = run >> 16;
    s_b[0] = t0 ? atomicAdd(count0, (unsigned long long)t0) : 0ULL;
    s_b[1] = t1 ? atomicAdd(count1, (unsigned long long)t1) : 0ULL;
  }
  __syncthreads();
  const unsigned ex = s_w[warp] + incl - x;
  r0 = s_b[0] + (ex & 0xFFFFu);
  r1 = s_b[1] + (ex >> 16);
  __syncthreads();
}

template <int kThreads>
__device__ __forceinline__ unsigned long long block_reserve(unsigned long long* count, unsigned n) {
  unsigned long long r0, r1;
  block_reserve2<kThreads>(count, n, count, 0u, r0, r1);
  return r0;
}

/* pixel index range whose centres (i + 0.5) / n - 0.5 may lie in [lo, hi] */
__device__ __forceinline__ void centre_range(float lo, float hi, long long n, long long& a, long long& b) {
  const float fa = fmaxf(-4.f, fminf((float)n + 4.f, (0.5f + lo) * (float)n - 0.5f - 1e-3f));
  const float fb = fmaxf(-4.f, fminf((float)n + 4.f, (0.5f + hi) * (float)n - 0.5f + 1e-3f));
  /* 32-bit conversions (the 64-bit ones run on the FP64 pipe); NaN gives an empty range */
  const int ia = __float2int_ru(fa), ib = __float2int_rd(fb);
  a = fa == fa ? max(0LL, (long long)ia) : 1;
  b = fb == fb ? min(n - 1, (long long)ib) : 0;
}

/*
 * k_vertices: the FP32 screen position of every crossed edge of the slab,
 * once per edge (a surface vertex is shared by about six triangles).  A block
 * takes kVTile consecutive cells, lists their owned crossed edges in shared
 * memory at their global vertex indices (the scan's vertex offsets), and
 * computes them with all its threads.  Each record: X, Y, Z, the bound on |X, Y - the
 * reference's value| and, in aux, the relative depth bound (>= 0), or -1 when
 * the projection certainly fails, -2 when the bounds cannot decide it.  The
 * edge runs from the owning corner to corner m; the reference interpolates a
 * triangle's vertex from its own tail corner, which gives the same point up
 * to FP64 rounding -- except where it keeps the tail because |v1 - v0| <
 * 1e-8, so that case is left undecided.
 */
constexpr int kVThreads = 128; /* 64, 128, 256 threads (tiles of 512 .. 2048 cells): 1.19, 1.10, 1.13 ms per frame */
constexpr int kVItems = 8;
constexpr int kVTile = kVThreads * kVItems;

template <typename T>
__global__ void __launch_bounds__(kVThreads)
k_vertices(FieldDev F, SlabDev S, SceneDev scene, const unsigned char* __restrict__ codes,
           VOffDev voff, long long n, VertDev V) {
  pdl_enter();
  __shared__ unsigned short list[kVTile * 7];
  const long long c0 = (long long)blockIdx.x * kVTile;
  if (c0 >= n) return;
  const long long c1 = min(c0 + kVTile, n);
  const unsigned va = voff_at(voff, c0), vb = voff_at(voff, c1);
  if (vb > V.cap) {
    /* more crossed edges than records (buffers sized before the count was known) */
    if (threadIdx.x == 0) atomicOr(V.ovf, kOvfVertices);
    return;
  }
  {
    /* the thread's kVItems cells: one 8-byte load of their codes (a code
       past the end reads as 0: no owned edges); their vertices are
       consecutive from the first cell's offset */
    const long long cf = c0 + (long long)threadIdx.x * kVItems;
    unsigned long long cw = 0;
    if (cf + kVItems <= c1) {
      cw = *reinterpret_cast<const unsigned long long*>(codes + cf); /* cf is a multiple of 8 */
    } else {
      for (int q = 0; q < kVItems; q++)
        if (cf + q < c1) cw |= (unsigned long long)codes[cf + q] << (8 * q);
    }
    if (cw != 0ULL && cw != ~0ULL) { /* all-outside or all-inside cells own no crossed edge */
      unsigned at = (cf < c1 ? voff_at(voff, cf) : vb) - va;
#pragma unroll
      for (int q = 0; q < kVItems; q++) {
        unsigned mask = owned_edges((unsigned)(cw >> (8 * q)) & 255u);
        const unsigned lc = threadIdx.x * kVItems + q;
        while (mask) {
          const unsigned m = (unsigned)__ffs(mask); /* edge to corner m */
          mask &= mask - 1;
          list[at++] = (unsigned short)(lc | (m << 11));
        }
      }
    }
  }
  __syncthreads();
  const T* fd = static_cast<const T*>(F.data);
  const ThrF th = thr_f(F.threshold);
  for (unsigned e = threadIdx.x; e < vb - va; e += kVThreads) {
    const unsigned entry = list[e];
    const unsigned m = entry >> 11;
    unsigned ui, uj, ukl;
    cell_ijk(F, (unsigned)(c0 + (entry & 2047)), ui, uj, ukl);
    const long long i = ui, j = uj, k = S.kfirst + ukl;
    float xa[3], xb[3], qv[3], eq[3];
    const float ce = corner_pos_f(F, i, j, k, 0, xa);
    corner_pos_f(F, i, j, k, (int)m, xb);
    const long long i0 = (k * F.ny + j) * F.nx + i;
    const long long i1 = i0 + (long long)(m & 1u) + ((m >> 1) & 1u) * F.nx + (long long)(m >> 2) * F.nx * F.ny;
    const bool vok = vertex_q<T>(scene, F, th, xa, __ldg(fd + i0), xb, __ldg(fd + i1), ce, qv, eq);
    float X = 0.f, Y = 0.f, Z = 0.f, exy = 0.f, ez = 0.f;
    const int st = vok ? project_f(scene, qv, eq, fmaxf(1e-12f, F.proj_eps), X, Y, Z, exy, ez) : -1;
    /* |Z| in [1e-8, 1e30] when the projection succeeds: __fdividef is within 2 ulp */
    const float aux = st > 0 ? 1.01f * __fdividef(ez, fabsf(Z)) : (st == 0 ? -1.f : -2.f);
    V.pos[va + e] = make_float4(X, Y, Z, __uint_as_float((bf16_up(exy) << 16) | bf16_up(aux)));
  }
}

/*
 * One thread per triangle.  The render form gathers a rendered triangle's
 * FP32 screen vertices and their bounds (from k_vertices) and picks the
 * raster path that settles it: the tiny list (FP64 throughout) when the
 * bounds cannot decide its culling, the sliver list when its area may be
 * clamped, none when no pixel centre can lie in it, the cover list
 * otherwise -- only cover and sliver triangles are written, to the compact
 * lists k_raster reads.  The inspection form keeps the cube-edge ids and
 * flags of every triangle (tri.meta) and routes nothing.
 */
/* what k_emit decided for one triangle */
struct EmitOut {
  int route; /* 0 no fragment, 1 k_tiny, 2 k_cover, 3 k_sliver */
  float X[3], Y[3], Z[3], exy, zr;
};

/*
 * One triangle.  RENDER: for a rendered triangle, its FP32 screen vertices
 * (gathered from k_vertices), its bounds and its raster route; nothing is
 * stored per triangle.  Otherwise (inspection): the cube-edge ids, the
 * rendered flag and the rank in the cell, stored in tri.meta.
 */
template <typename T, bool CHECK, bool RENDER, typename LutT>
__device__ __forceinline__ void emit_one(const FieldDev& F, const SlabDev& S, const SceneDev& scene,
                                         const LutT* lut, const unsigned char* __restrict__ codes,
                                         const VOffDev& voff, const unsigned* __restrict__ tri_cell,
                                         const TriDev& tri, const RasterDev& R, const VertDev& V,
                                         unsigned* __restrict__ checks, long long t, EmitOut& out) {
  const unsigned ncx = (unsigned)(F.nx - 1), ncy = (unsigned)(F.ny - 1);
  const long long W = scene.width, H = scene.height;
  const unsigned ncxy = ncx * ncy;
  int& route = out.route;
  float* X = out.X;
  float* Y = out.Y;
  float* Z = out.Z;
  float& exy = out.exy;
  float& zr = out.zr;
  route = 0;
  exy = 0.f;
  zr = 0.f;
#pragma unroll
  for (int q = 0; q < 3; q++) X[q] = Y[q] = Z[q] = 0.f;
  const unsigned tc = tri_cell[t];
  const unsigned c = tc & kTcCellMask, r = tc >> kTcRankShift;
  unsigned ui, uj, ukl;
  cell_ijk(F, c, ui, uj, ukl);
  /* slab slices fit 32 bits (a slab holds fewer than 2^28 cells) */
  const unsigned uk = (unsigned)S.kfirst + ukl;
  const unsigned code = codes[c];
  const unsigned long long e = RENDER ? __ldg(lut + code * 12 + r) : lut[code * 12 + r];
  /* rendered set: interior cells of the slab's own slices (contour/main.c:70-112) */
  const bool rendered = ui >= 1u && ui + 2u <= ncx && uj >= 1u && uj + 2u <= ncy && uk >= (unsigned)S.krender0 &&
                        uk < (unsigned)S.krender1;
  if (!RENDER) {
    unsigned edges = 0;
#pragma unroll
    for (int q = 0; q < 3; q++) edges |= (unsigned)((e >> (18 + 5 * q)) & 31) << (5 * q);
    tri.meta[t] = edges | (rendered ? kMetaRendered : 0u) | (r << kMetaRankShift);
    return;
  }
  if (!rendered) return;
  /* the three vertices from k_vertices: vertex q lies on the edge from
     corner a to corner b, owned by the cell at corner a & b */
  int status = 1;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const unsigned a = (unsigned)((e >> (6 * q)) & 7), b = (unsigned)((e >> (6 * q + 3)) & 7);
    const unsigned o = a & b, m = a ^ b;
    const unsigned oc = c + (o & 1u) + ((o >> 1) & 1u) * ncx + (o >> 2) * ncxy;
    const unsigned vi = voff_at(voff, oc) + __popc(owned_edges(codes[oc]) & ((1u << (m - 1)) - 1u));
    const float4 p = __ldg(V.pos + vi);
    const unsigned pk = __float_as_uint(p.w);
    const float aux = bf16_value(pk & 0xFFFFu);
    X[q] = p.x;
    Y[q] = p.y;
    Z[q] = p.z;
    exy = fmaxf(exy, bf16_value(pk >> 16));
    if (aux >= 0.f) zr = fmaxf(zr, aux);
    else if (aux == -1.f) status = 0;
    else if (status != 0) status = -1;
  }
  const long long i = ui, j = uj, k = uk;
  d3 v[3];
  bool ok = true;
  if (CHECK) {
    /* the reference's own vertices and projection */
    d3 p[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const int a = (int)((e >> (6 * q)) & 7), b = (int)((e >> (6 * q + 3)) & 7);
      v[q] = interpolate(F.threshold, corner_pos(F, i, j, k, a), corner_value(F, i, j, k, a),
                         corner_pos(F, i, j, k, b), corner_value(F, i, j, k, b));
    }
#pragma unroll
    for (int q = 0; q < 3; q++) ok = project(scene, v[q], p[q]) && ok;
    if (status >= 0 && (status == 1) != ok) atomicAdd(checks + 0, 1u);
    if (status == 1 && ok) {
#pragma unroll
      for (int q = 0; q < 3; q++)
        if (fabs((double)X[q] - p[q].x) > exy || fabs((double)Y[q] - p[q].y) > exy ||
            fabs((double)Z[q] - p[q].z) > (double)zr * fabs((double)Z[q]))
          atomicAdd(checks + 1, 1u);
    }
  }
  if (status == 0) return;
  const EdgeF E2 = edge_f(X[0], Y[0], X[1], Y[1], exy);
  float errA;
  const float A = edge_eval(E2, X[2], Y[2], exy, exy, errA);
  const bool decided = status > 0 && isfinite(A) && isfinite(exy) && exy < 1e-3f && zr < 1e-3f;
  if (!decided) {
    route = 1;
  } else if (!(fabsf(A) - errA > 1e-15f)) {
    /* the area may be clamped to +-1e-16 (render.c:108-111): the sliver
       pass tests the reference's whole box */
    route = 3;
  } else {
    /* the reference's area is certainly not clamped: its weights are
       barycentric up to the -1e-8 slack, so every covered pixel centre
       lies in the triangle's extent */
    const float xext = fmaxf(X[0], fmaxf(X[1], X[2])) - fminf(X[0], fminf(X[1], X[2]));
    const float yext = fmaxf(Y[0], fmaxf(Y[1], Y[2])) - fminf(Y[0], fminf(Y[1], Y[2]));
    const float mb = exy + 1e-6f * (xext + yext) + 1e-12f;
    long long imin, imax, jmin, jmax;
    centre_range(fminf(X[0], fminf(X[1], X[2])) - mb, fmaxf(X[0], fmaxf(X[1], X[2])) + mb, W, imin, imax);
    centre_range(fminf(Y[0], fminf(Y[1], Y[2])) - mb, fmaxf(Y[0], fmaxf(Y[1], Y[2])) + mb, H, jmin, jmax);
    route = imin <= imax && jmin <= jmax ? 2 : 0;
    if (CHECK && route == 0 && ok) {
      /* no pixel of the reference's box may be covered */
      ExactTri ex;
      if (exact_tri(scene, v, ex))
        for (long long jj = ex.jmin; jj <= ex.jmax; jj++)
          for (long long ii = ex.imin; ii <= ex.imax; ii++) {
            double w0, w1, w2;
            if (exact_weights(ex, ii, jj, R.xs, R.ys, w0, w1, w2)) atomicAdd(checks + 2, 1u);
          }
    }
  }
}

/* triangles per thread and iteration: one.  k_emit hides its gathers by
   occupancy, and it reaches all 64 warps per SM only at 32 registers or
   fewer: two or three chains per thread, or loading the next triangle's
   entry one iteration ahead, cost registers and measured slower */
constexpr int kEmitPer = 1;

/*
 * List appends without block barriers: each warp takes chunks of entries
 * from a list's counter (one atomic per chunk) and fills them with warp
 * ballots; a batch that does not fit the chunk's rest starts the next
 * chunk.  At the warp's end the rest of its last chunk is marked empty
 * (kNoTri), so a list holds its entries and fewer than one chunk of empty
 * ones per warp; the raster passes skip those.  A chunk is the smallest
 * multiple of the list's unit that holds the rest of a batch; the sparse
 * sliver list (about 2 % of the triangles) takes a small unit so that its
 * empty entries stay few.
 */
/* cover chunk units of 32, 64 and 128 measured alike (5.57 +- 0.01 ms per frame) */
constexpr unsigned kCoverChunk = 32, kSliverChunk = 8;
/* runs of 32 consecutive triangles per warp and window: 1 (grid-stride), 2,
   4 and 8 measured 5.57, 5.56, 5.51 and 5.51 ms per bench frame */
constexpr unsigned kEmitRun = 4;
constexpr unsigned kNoTri = 0xFFFFFFFFu;

/* record entries beyond the triangles that a grid of `blocks` k_emit blocks
   may leave empty (two lists, one partial chunk per warp and list) */
__host__ __device__ __forceinline__ unsigned long long emit_slack_for(unsigned long long blocks) {
  return (unsigned long long)(kCoverChunk + kSliverChunk) * blocks * (256 / 32);
}

/* the list slot of this lane's entry (when `take`), every lane of the warp
   calling with the same chunk state */
template <unsigned kChunk>
__device__ __forceinline__ unsigned long long warp_append(unsigned long long* count, bool take, unsigned lane,
                                                          unsigned below, unsigned long long& cbase,
                                                          unsigned& cfill, unsigned& csize,
                                                          unsigned long long& taken) {
  const unsigned m = __ballot_sync(0xFFFFFFFFu, take);
  if (m == 0u) return 0ULL;
  const unsigned n = __popc(m), rank = __popc(m & below), room = csize - cfill;
  taken += n;
  unsigned long long slot = cbase + cfill + rank;
  if (n > room) {
    /* the next chunk: whole multiples of kChunk holding the batch's rest */
    const unsigned size = (n - room + kChunk - 1) / kChunk * kChunk;
    unsigned long long nb = 0;
    if (lane == 0) nb = atomicAdd(count, (unsigned long long)size);
    nb = __shfl_sync(0xFFFFFFFFu, nb, 0);
    if (rank >= room) slot = nb + (rank - room);
    cbase = nb;
    cfill = n - room;
    csize = size;
  } else {
    cfill += n;
  }
  return slot;
}

template <typename T, bool CHECK, bool RENDER>
__global__ void __launch_bounds__(256, CHECK ? 1 : 8)
k_emit(FieldDev F, SlabDev S, SceneDev scene, const unsigned long long* __restrict__ lut_g,
       const unsigned char* __restrict__ codes, const unsigned* __restrict__ offsets,
       VOffDev voff, const unsigned* __restrict__ tri_cell,
       const unsigned long long* __restrict__ total_p, TriDev tri, RasterDev R, VertDev V,
       unsigned* __restrict__ checks) {
  pdl_trigger(); /* the table below does not depend on the preceding kernel */
  (void)offsets;
  /* the render form reads the table through L1 (one 24 KB copy per SM)
     rather than from a copy in each block's shared memory, which took L1
     from the gathers and shared memory from the other lane's kernels (per
     bench frame: 64-bit entries in shared memory 1.57 ms of emit, 32-bit
     ones 1.47, 16-bit cube-edge ids decoded through a 19-entry table 1.50;
     through L1 emit 1.52 -> 1.54 alone, but the frame 5.53 -> 5.48 ms) */
  using LutT = unsigned long long;
  __shared__ LutT lut_s[RENDER ? 1 : kLutEntries];
  if (!RENDER) {
    for (int q = threadIdx.x; q < kLutEntries; q += blockDim.x) lut_s[q] = lut_g[q];
    __syncthreads();
  }
  const LutT* lut = RENDER ? lut_g : lut_s;
  pdl_wait();
  const long long T_ = (long long)*total_p;
  /* the record region holds the cover and sliver entries (at most the
     triangles) and every warp's unfilled chunk ends */
  const unsigned long long slack = RENDER ? emit_slack_for(gridDim.x) : 0ULL;
  if ((unsigned long long)T_ > tri.cap || (unsigned long long)T_ + slack > tri.rec_cap ||
      (V.pos && total_p[1] > V.cap)) {
    /* more triangles than the arrays hold, or more crossed edges than vertex
       records (sized before the counts were known): nothing is read or
       written, the frame is rendered again */
    if (blockIdx.x == 0 && threadIdx.x == 0)
      atomicOr(tri.ovf, (unsigned long long)T_ + slack > tri.rec_cap || (unsigned long long)T_ > tri.cap
                            ? kOvfTriangles
                            : kOvfVertices);
    return;
  }
  const unsigned lane = threadIdx.x & 31u, below = (1u << lane) - 1u;
  /* the grid works through windows of the slab's triangles, small enough
     that a window's cells and vertex records stay in L2 (blocks with ranges
     of their own measured slower: 1.59 -> 1.82 ms per frame); within a
     window each warp takes kEmitRun consecutive runs of 32, so the entries
     of a list chunk lie close together in the field and on screen, as the
     raster passes like them (a slab's triangles are numbered in 32 bits) */
  const unsigned long long tcount = (unsigned long long)T_;
  const unsigned long long window = (unsigned long long)gridDim.x * blockDim.x * kEmitRun;
  /* this thread's place in a window: its warp's runs, its lane */
  const unsigned toff = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) * kEmitRun + lane;
  /* the warp's current chunk of each list: `size` entries from `base` on,
     `fill` of them taken (size 0: none yet) */
  unsigned long long cbase = 0, sbase = 0, ctaken = 0, staken = 0;
  unsigned cfill = 0, csize = 0, sfill = 0, ssize = 0;
  /* every thread of a block runs the same iterations (warp-wide appends);
     iteration it is run it % kEmitRun of window it / kEmitRun */
  for (unsigned long long it = 0;; it++) {
    const unsigned long long wbase = (it / kEmitRun) * window + (it % kEmitRun) * 32;
    if (wbase + (unsigned long long)blockIdx.x * blockDim.x * kEmitRun >= tcount) break; /* the block's first */
    EmitOut o[kEmitPer];
    const unsigned long long tw = wbase + toff;
#pragma unroll
    for (int u = 0; u < kEmitPer; u++) {
      o[u].route = 0;
      if (tw < tcount) emit_one<T, CHECK, RENDER>(F, S, scene, lut, codes, voff, tri_cell, tri, R, V, checks,
                                                  (long long)tw, o[u]);
    }
    if (RENDER) {
#pragma unroll
      for (int u = 0; u < kEmitPer; u++) {
        const unsigned t = (unsigned)tw;
        const EmitOut& e = o[u];
        /* the tiny list holds a few thousand entries per frame: one atomic each */
        if (e.route == 1) {
          const unsigned long long ti = atomicAdd(R.tiny_count, 1ULL);
          if (ti < R.tiny_cap) R.tiny[ti] = t; /* overflow: the host re-runs the slab */
        }
        const unsigned long long ci =
            warp_append<kCoverChunk>(R.cover_count, e.route == 2, lane, below, cbase, cfill, csize, ctaken);
        const unsigned long long si =
            warp_append<kSliverChunk>(R.sliver_count, e.route == 3, lane, below, sbase, sfill, ssize, staken);
        if (e.route >= 2) {
          float4* rec = e.route == 2 ? tri.rec + 3 * ci : R.sliver_rec - 3 * si;
          rec[0] = make_float4(e.X[0], e.Y[0], e.Z[0], e.X[1]);
          rec[1] = make_float4(e.Y[1], e.Z[1], e.X[2], e.Y[2]);
          rec[2] = make_float4(e.Z[2], e.exy, e.zr, __uint_as_float(t));
        }
      }
    }
  }
  if (RENDER) {
    /* the unfilled ends of the warp's last chunks are marked empty */
    const float4 none = make_float4(0.f, 0.f, 0.f, __uint_as_float(kNoTri));
    for (unsigned q = cfill + lane; q < csize; q += 32) tri.rec[3 * (cbase + q) + 2] = none;
    for (unsigned q = sfill + lane; q < ssize; q += 32) R.sliver_rec[2 - 3 * (long long)(sbase + q)] = none;
    /* the entries themselves, for the statistics */
    if (lane == 0 && ctaken) atomicAdd(R.listed_count, ctaken);
    if (lane == 0 && staken) atomicAdd(R.listed_count + 1, staken);
  }
}

/*
 * A pixel range holding the reference's bounding box (render.c:90-99):
 * [(0.5 + lo) n - 1, (0.5 + hi) n + 1] truncated and clamped to [0, n - 1],
 * for a triangle whose extent lies in [lo, hi].
 */
__device__ __forceinline__ void reference_box(float lo, float hi, long long n, long long& a, long long& b) {
  /* in [-4, n + 4] the FP32 values are within 2u n + u of the exact ones:
     floor / ceil past a margin of 3u n hold the truncated bounds; NaN gives
     the whole axis */
  const float fa = fmaxf(-4.f, fminf((float)n + 4.f, (0.5f + lo) * (float)n - 1.f));
  const float fb = fmaxf(-4.f, fminf((float)n + 4.f, (0.5f + hi) * (float)n + 1.f));
  const float mg = 3.f * kU32 * (float)n + 1e-4f;
  const int ia = __float2int_rd(fa - mg), ib = __float2int_ru(fb + mg);
  a = fa == fa ? max(0LL, (long long)ia) : 0;
  b = fb == fb ? min(n - 1, (long long)ib) : n - 1;
}

/* ------------------------------------------------------------------ */
/* triangles the single-precision filter cannot settle                 */
/* ------------------------------------------------------------------ */
/*
 * Triangles whose culling or bounds are too uncertain for the FP32 filter
 * (a vertex near the camera plane or the edge of the view, or an edge whose
 * value difference is near 1e-8).  The reference's vertices, projection
 * and area are computed once per triangle; when the area is not clamped
 * (|area| >= 1e-16, render.c:108-111) the covered pixel centres lie in the
 * triangle's extent, which holds no pixel centre for most of these
 * triangles; otherwise the reference's whole box is tested.  Fragments go
 * straight to the z-buffer.
 */
template <bool CHECK>
__device__ void tiny_triangle(const Geo& G, const SceneDev& s, long long t, const RasterDev& R,
                              unsigned long long order_base, unsigned* checks) {
  d3 w[3];
  exact_vertices(G, t, w);
  ExactTri x;
  if (!exact_tri(s, w, x)) return;
  long long imin = x.imin, imax = x.imax, jmin = x.jmin, jmax = x.jmax;
  if (fabs(x.area) >= 1.e-16) {
    const double xlo = fmin(x.v0.x, fmin(x.v1.x, x.v2.x)), xhi = fmax(x.v0.x, fmax(x.v1.x, x.v2.x));
    const double ylo = fmin(x.v0.y, fmin(x.v1.y, x.v2.y)), yhi = fmax(x.v0.y, fmax(x.v1.y, x.v2.y));
    const double mb = 1e-6 * ((xhi - xlo) + (yhi - ylo)) + 1e-14;
    const long long W = s.width, H = s.height;
    const double ia = ceil((0.5 + (xlo - mb)) * (double)W - 0.5 - 1e-6);
    const double ib = floor((0.5 + (xhi + mb)) * (double)W - 0.5 + 1e-6);
    const double ja = ceil((0.5 + (ylo - mb)) * (double)H - 0.5 - 1e-6);
    const double jb = floor((0.5 + (yhi + mb)) * (double)H - 0.5 + 1e-6);
    imin = max(imin, (long long)fmax(ia, -1.0));
    imax = min(imax, (long long)fmin(ib, (double)W));
    jmin = max(jmin, (long long)fmax(ja, -1.0));
    jmax = min(jmax, (long long)fmin(jb, (double)H));
  }
  if (CHECK) {
    for (long long j = x.jmin; j <= x.jmax; j++)
      for (long long i = x.imin; i <= x.imax; i++) {
        double w0, w1, w2;
        if (exact_weights(x, i, j, R.xs, R.ys, w0, w1, w2) && (i < imin || i > imax || j < jmin || j > jmax))
          atomicAdd(checks + 2, 1u);
      }
  }
  const unsigned long long order = order_of(G, order_base, t);
  for (long long j = jmin; j <= jmax; j++)
    for (long long i = imin; i <= imax; i++) {
      double w0, w1, w2;
      if (!exact_weights(x, i, j, R.xs, R.ys, w0, w1, w2)) continue;
      const long long p = j * s.width + i;
      if (slot_max(R.canvas + p, depth_key(exact_depth(x, w0, w1, w2)), order << 24, R.zerr))
        keep_weights(R, p, order, w0, w1, w2);
    }
}

/* candidates a k_cover thread keeps before appending */
constexpr unsigned kCandBuf = 8;

/* candidates (t, pix[u]) at slots [b, b + nb); those past the capacity are
   dropped (the host sees the count and re-runs the slab) */
__device__ __forceinline__ void write_candidates(const RasterDev& R, unsigned long long b, unsigned t, float dhi,
                                                 const unsigned* pix, unsigned nb) {
  for (unsigned u = 0; u < nb; u++) {
    if (b + u >= R.cand_cap) break;
    Candidate cd;
    cd.t = t;
    cd.pixel = pix[u];
    cd.dhi = dhi;
    cd.pad = 0;
    R.cand[b + u] = cd;
  }
}

/* one block's 128 entries [base, base + 128) of the cover list (n entries),
   traversed front to back along z (the list is close to emission order,
   which follows z) so that near surfaces raise the floors early.  Every
   thread of the block takes part: a thread keeps up to kCandBuf candidates
   of its triangle and the block appends them at once */
template <bool CHECK>
__device__ __noinline__ void cover_block(const Geo& G, const SceneDev& scene, const TriDev& tri,
                                            const RasterDev& R, unsigned* __restrict__ checks, long long base,
                                            long long n) {
  const long long W = scene.width, H = scene.height;
  {
    const long long q = base + threadIdx.x;
    unsigned pix[kCandBuf];
    unsigned nb = 0, t32 = 0;
    float dhi = 0.f;
    const long long qq = scene.z_descending ? n - 1 - q : q;
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = make_float4(0.f, 0.f, 0.f, __uint_as_float(kNoTri));
    if (q < n) {
      r0 = __ldg(tri.rec + 3 * qq);
      r1 = __ldg(tri.rec + 3 * qq + 1);
      r2 = __ldg(tri.rec + 3 * qq + 2);
    }
    if (__float_as_uint(r2.w) != kNoTri) { /* an entry, not a chunk's empty end */
      const long long t = (long long)__float_as_uint(r2.w);
      const float X[3] = {r0.x, r0.w, r1.z}, Y[3] = {r0.y, r1.x, r1.w}, Z[3] = {r0.z, r1.y, r2.x};
      const float eps = r2.y, zr = r2.z;
      /* inverse area (render.c:102-107) with its bound; k_emit listed only
         triangles whose area is certainly not clamped and whose extent may
         hold a pixel centre.  The per-pixel weight bounds are used when they
         are tight enough to decide anything (rai < 0.5) */
      const EdgeF E0 = edge_f(X[1], Y[1], X[2], Y[2], eps);
      const EdgeF E1 = edge_f(X[2], Y[2], X[0], Y[0], eps);
      const EdgeF E2 = edge_f(X[0], Y[0], X[1], Y[1], eps);
      float errA;
      const float A = edge_eval(E2, X[2], Y[2], eps, eps, errA);
      const float rai = errA / (fabsf(A) - errA) + 1.1f * kU32;
      const bool weights_ok = rai < 0.5f;
      const float ai = 1.f / A;
      const float xlo = fminf(X[0], fminf(X[1], X[2])), xhi = fmaxf(X[0], fmaxf(X[1], X[2]));
      const float ylo = fminf(Y[0], fminf(Y[1], Y[2])), yhi = fmaxf(Y[0], fmaxf(Y[1], Y[2]));
      const float mb = eps + 1e-6f * ((xhi - xlo) + (yhi - ylo)) + 1e-12f;
      long long imin, imax, jmin, jmax;
      centre_range(xlo - mb, xhi + mb, W, imin, imax);
      centre_range(ylo - mb, yhi + mb, H, jmin, jmax);
      /* depth of any covered fragment: the harmonic mean of the vertex depths
         with weights >= -1e-8 summing to 1, so within their range */
      const float zmin = fminf(Z[0], fminf(Z[1], Z[2])), zmax = fmaxf(Z[0], fmaxf(Z[1], Z[2]));
      const float m = zr + 4e-6f;
      const float dlo = zmin - m * fabsf(zmin);
      dhi = zmax + m * fabsf(zmax);
      t32 = (unsigned)t;
      ExactTri ex;
      bool ex_ok = false;
      if (CHECK) {
        d3 wv[3];
        exact_vertices(G, t, wv);
        ex_ok = exact_tri(scene, wv, ex);
        if (ex_ok) {
          /* every covered pixel of the reference's box must lie in the tight range */
          for (long long j = ex.jmin; j <= ex.jmax; j++)
            for (long long i = ex.imin; i <= ex.imax; i++) {
              double w0, w1, w2;
              if (exact_weights(ex, i, j, R.xs, R.ys, w0, w1, w2)) {
                if (i < imin || i > imax || j < jmin || j > jmax) atomicAdd(checks + 2, 1u);
                const double d = exact_depth(ex, w0, w1, w2);
                if (!(d <= (double)dhi && d >= (double)dlo)) atomicAdd(checks + 4, 1u);
              }
            }
        }
      }
      for (long long j = jmin; j <= jmax; j++) {
        const float py = R.ysf[j];
        for (long long i = imin; i <= imax; i++) {
          const float px = R.xsf[i];
          const float ep = 0.5f * kU32;
          float e0, e1, e2;
          const float w0 = ai * edge_eval(E0, px, py, ep, eps, e0);
          const float w1 = ai * edge_eval(E1, px, py, ep, eps, e1);
          const float w2 = ai * edge_eval(E2, px, py, ep, eps, e2);
          const float k = fabsf(ai) * (1.f + rai);
          const float ew0 = __fmaf_rn(1.25f, __fmaf_rn(k, e0, fabsf(w0) * (rai + kU32)), 1e-30f);
          const float ew1 = __fmaf_rn(1.25f, __fmaf_rn(k, e1, fabsf(w1) * (rai + kU32)), 1e-30f);
          const float ew2 = __fmaf_rn(1.25f, __fmaf_rn(k, e2, fabsf(w2) * (rai + kU32)), 1e-30f);
          const bool out = weights_ok && ((w0 + ew0 < kWOut) || (w1 + ew1 < kWOut) || (w2 + ew2 < kWOut));
          const bool inside = weights_ok && !out && (w0 - ew0 > kWIn) && (w1 - ew1 > kWIn) && (w2 - ew2 > kWIn);
          if (CHECK && ex_ok) {
            double x0, x1, x2;
            const bool cov = exact_weights(ex, i, j, R.xs, R.ys, x0, x1, x2);
            if (cov && out) atomicAdd(checks + 2, 1u);     /* dropped a covered pixel */
            if (!cov && inside) atomicAdd(checks + 3, 1u); /* called an uncovered pixel inside */
          }
          if (inside) atomicMax(R.zlo + j * W + i, f_key(dlo));
          if (!out) {
            if (nb == kCandBuf) { /* a large triangle: append the full buffer now */
              write_candidates(R, atomicAdd(R.cand_count, (unsigned long long)kCandBuf), t32, dhi, pix, nb);
              nb = 0;
            }
            pix[nb++] = (unsigned)(j * W + i);
          }
        }
      }
    }
    write_candidates(R, block_reserve<128>(R.cand_count, nb), t32, dhi, pix, nb);
  }
}

/* |a - b| bound of a product of bounded factors, plus its rounding */
__device__ __forceinline__ float prod_err(float a, float ea, float b, float eb) {
  return fabsf(a) * eb + ea * fabsf(b) + ea * eb + kU32 * fabsf(a * b);
}

/*
 * One thread per requested triangle: its area-weighted face normal in FP32.
 * The reference's area * unit normal equals the cross product of two edges
 * up to a few FP64 ulps; the vertices are taken relative to the cell's corner
 * 0 (offsets from the rounded node spacings, interpolation as in vertex_q),
 * so the edge vectors keep their relative accuracy.  w: the largest bound of
 * the three components (infinite when none can be given).
 */
/*
 * The vertices of triangle u (triangulate.c:40-73) relative to its cell's
 * corner 0, in FP32 with a bound on each component's distance to the
 * reference's FP64 vertex minus that corner: corner offsets from the rounded
 * node spacings, the interpolation parameter from interp_param, and an
 * absolute allowance (coord_eps) for the reference's own FP64 rounding.  Edge
 * vectors formed from these keep their relative accuracy however far the
 * cell is from the origin.  False when a vertex cannot be bounded.  Needs
 * the spacing tables (identity converter).
 */
/* one vertex of that kind: on the edge from corner a to corner b at the
   interpolation parameter f (bound e_f), with the rounded node spacings sp of
   the cell */
__device__ __forceinline__ void rel_pos(const FieldDev& F, const float sp[3], unsigned a, unsigned b, float f,
                                        float e_f, float rv[3], float er[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    /* corner offsets from corner 0 along axis d: the rounded spacing or 0 */
    const float oa = ((a >> d) & 1u) ? sp[d] : 0.f, ob = ((b >> d) & 1u) ? sp[d] : 0.f;
    const float dd = ob - oa;
    const float p = oa + f * dd;
    rv[d] = p;
    er[d] = 1.1f * (1.01f * kU32 * (fabsf(oa) + fabsf(f) * (fabsf(oa) + fabsf(ob))) + e_f * fabsf(dd) +
                    kU32 * (2.2f * fabsf(f * dd) + fabsf(p))) +
            F.coord_eps;
  }
}

template <typename T>
__device__ __forceinline__ bool cell_rel_vertices(const Geo& G, unsigned u, float rv[3][3], float er[3][3]) {
  const FieldDev& F = G.F;
  const T* fd = static_cast<const T*>(F.data);
  const ThrF th = thr_f(F.threshold);
  const unsigned tc = G.tri_cell[u];
  const unsigned c = tc & kTcCellMask, r = tc >> kTcRankShift;
  unsigned ui, uj, ukl;
  cell_ijk(F, c, ui, uj, ukl);
  const long long i = ui, j = uj, k = G.S.kfirst + ukl;
  const unsigned long long e = __ldg(G.lut + G.codes[c] * 12 + r);
  const float sp[3] = {__ldg(F.dgx + i), __ldg(F.dgy + j), __ldg(F.dgz + k)};
  const long long base = (k * F.ny + j) * F.nx + i;
  bool ok = true;
#pragma unroll
  for (int v = 0; v < 3; v++) {
    const unsigned a = (unsigned)((e >> (6 * v)) & 7), b = (unsigned)((e >> (6 * v + 3)) & 7);
    const long long ia = base + (a & 1u) + ((a >> 1) & 1u) * F.nx + (long long)(a >> 2) * F.nx * F.ny;
    const long long ib = base + (b & 1u) + ((b >> 1) & 1u) * F.nx + (long long)(b >> 2) * F.nx * F.ny;
    float f = 0.f, e_f = 0.f;
    if (interp_shade(F, th, ShadeVal<T>::load(fd, ia), ShadeVal<T>::load(fd, ib), f, e_f) < 0) ok = false;
    rel_pos(F, sp, a, b, f, e_f, rv[v], er[v]);
  }
  return ok;
}

/*
 * Slivers: triangles whose area may be clamped to +-1e-16 (render.c:108-111).
 * A covered pixel then need not lie in the triangle's extent, so the
 * reference's whole box is tested: with the clamped area a, w_k = e_k / a <
 * -1e-8 holds certainly when s e_k < -tau for the sign s of a (|a| < tau /
 * 1e-8), and the weights need not sum to 1.  A sliver whose pixels are all
 * certainly outside draws nothing; any other goes whole to the exact path
 * (k_tiny).  One thread per sliver, in a list of their own so that a warp's
 * loops over these boxes stay converged.
 */
/*
 * The three screen edge vectors V_b - V_a of triangle t (edge k runs from
 * vertex (k + 1) % 3 to (k + 2) % 3, as the weights of render.c:115-133)
 * from its world edges dv (cell_rel_vertices) in the exact form
 *   dX = b_x ((l_x . dv) - rho_x (n . dv)) / (n . q_a + n . dv),
 *   rho_x = (X_a - a_x) / b_x = (l_x . q_a) / (n . q_a)
 * (and the same for Y), q_a = vertex a - camera, with a bound e on each
 * component.  A point-like triangle keeps the directions of its edges this
 * way, where its FP32 screen vertices (bounds ~1e-7) cannot.  False when no
 * bound can be given.
 */
template <typename T>
__device__ __forceinline__ bool screen_edges(const Geo& G, const SceneDev& s, unsigned t, const float X[3],
                                             const float Y[3], const float Z[3], float eps, float zr, float sdx[3],
                                             float sdy[3], float sde[3]) {
  float rv[3][3], er[3][3];
  if (!G.F.dgx || !cell_rel_vertices<T>(G, t, rv, er)) return false;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int a = (k + 1) % 3, b = (k + 2) % 3;
    float dv[3], edv[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      dv[d] = rv[b][d] - rv[a][d];
      edv[d] = er[a][d] + er[b][d] + kU32 * fabsf(dv[d]);
    }
    float nd = 0.f, ld = 0.f, md = 0.f, e_nd = 0.f, e_ld = 0.f, e_md = 0.f, an = 0.f, al = 0.f, am = 0.f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      nd += s.f_n[d] * dv[d];
      ld += s.f_lx[d] * dv[d];
      md += s.f_ly[d] * dv[d];
      e_nd += fabsf(s.f_n[d]) * edv[d];
      e_ld += fabsf(s.f_lx[d]) * edv[d];
      e_md += fabsf(s.f_ly[d]) * edv[d];
      an += fabsf(s.f_n[d] * dv[d]);
      al += fabsf(s.f_lx[d] * dv[d]);
      am += fabsf(s.f_ly[d] * dv[d]);
    }
    /* the constants' rounding to float (u) and the dot products' (3u) */
    e_nd = 1.01f * (e_nd + 4.f * kU32 * an);
    e_ld = 1.01f * (e_ld + 4.f * kU32 * al);
    e_md = 1.01f * (e_md + 4.f * kU32 * am);
    const float nq = Z[a];
    const float Dn = nq + nd;
    const float e_Dn = 1.01f * (zr * fabsf(nq) + e_nd + kU32 * fabsf(Dn)) + 1e-37f;
    if (!(fabsf(Dn) > 4.f * e_Dn) || !isfinite(Dn)) return false;
    const float rx = (X[a] - s.f_ax) / s.f_bx, ry = (Y[a] - s.f_ay) / s.f_by;
    const float e_rx = 1.01f * (eps + kU32 * (fabsf(s.f_ax) + fabsf(X[a] - s.f_ax))) / fabsf(s.f_bx) + 3.f * kU32 * fabsf(rx);
    const float e_ry = 1.01f * (eps + kU32 * (fabsf(s.f_ay) + fabsf(Y[a] - s.f_ay))) / fabsf(s.f_by) + 3.f * kU32 * fabsf(ry);
    const float Nx = ld - rx * nd, Ny = md - ry * nd;
    const float e_Nx = e_ld + fabsf(rx) * e_nd + e_rx * fabsf(nd) + e_rx * e_nd + kU32 * (fabsf(ld) + 2.f * fabsf(rx * nd));
    const float e_Ny = e_md + fabsf(ry) * e_nd + e_ry * fabsf(nd) + e_ry * e_nd + kU32 * (fabsf(md) + 2.f * fabsf(ry * nd));
    const float iD = 1.f / Dn;
    sdx[k] = s.f_bx * Nx * iD;
    sdy[k] = s.f_by * Ny * iD;
    const float rel = e_Dn / (fabsf(Dn) - e_Dn);
    /* the reference forms V_b - V_a from two FP64 projections, each rounded by up to proj_eps */
    const float ex = 1.01f * fabsf(s.f_bx) * (e_Nx + fabsf(Nx) * rel) * fabsf(iD) + 5.f * kU32 * fabsf(sdx[k]) +
                     2.f * G.F.proj_eps;
    const float ey = 1.01f * fabsf(s.f_by) * (e_Ny + fabsf(Ny) * rel) * fabsf(iD) + 5.f * kU32 * fabsf(sdy[k]) +
                     2.f * G.F.proj_eps;
    sde[k] = fmaxf(ex, ey);
    if (!isfinite(sde[k]) || !isfinite(sdx[k]) || !isfinite(sdy[k])) return false;
  }
  return true;
}

/* one block's 128 entries [base, base + 128) of the sliver list (n entries);
   triangles the bounds cannot settle go to the tiny list (block-wide append) */
template <typename T, bool CHECK>
__device__ __noinline__ void sliver_block(const Geo& G, const SceneDev& scene, const RasterDev& R,
                                             unsigned* __restrict__ checks, long long base, long long n) {
  const long long W = scene.width, H = scene.height;
  {
    const long long q = base + threadIdx.x;
    bool to_tiny = false;
    unsigned t32 = 0;
    const float4* rec = R.sliver_rec - 3 * q;
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = make_float4(0.f, 0.f, 0.f, __uint_as_float(kNoTri));
    if (q < n) {
      r0 = __ldg(rec);
      r1 = __ldg(rec + 1);
      r2 = __ldg(rec + 2);
    }
    if (__float_as_uint(r2.w) != kNoTri) { /* an entry, not a chunk's empty end */
      t32 = __float_as_uint(r2.w);
      const float X[3] = {r0.x, r0.w, r1.z}, Y[3] = {r0.y, r1.x, r1.w}, Z[3] = {r0.z, r1.y, r2.x};
      const float eps = r2.y, zr = r2.z;
      /* the screen edges from the world edges (exact form, tight bounds) */
      float sdx[3], sdy[3], sde[3];
      const bool refined = screen_edges<T>(G, scene, t32, X, Y, Z, eps, zr, sdx, sdy, sde);
      const EdgeF E0 = edge_f(X[1], Y[1], X[2], Y[2], eps);
      const EdgeF E1 = edge_f(X[2], Y[2], X[0], Y[0], eps);
      const EdgeF E2 = edge_f(X[0], Y[0], X[1], Y[1], eps);
      float errA;
      float A = edge_eval(E2, X[2], Y[2], eps, eps, errA);
      if (refined) {
        /* render.c:38-46 area from the refined edges: (V2 - V0) x (V1 - V0) */
        const float ax_ = -sdx[1], ay_ = -sdy[1], bx_ = sdx[2], by_ = sdy[2];
        const float p1 = ax_ * by_, p2 = ay_ * bx_;
        A = p1 - p2;
        errA = 1.1f * ((fabsf(ax_) + fabsf(ay_)) * sde[2] + sde[1] * (fabsf(bx_) + fabsf(by_)) +
                       2.f * sde[1] * sde[2] + kU32 * (fabsf(p1) + fabsf(p2) + fabsf(A))) +
               1e-15f * (fabsf(p1) + fabsf(p2)) + 1e-37f;
      }
      const float xlo = fminf(X[0], fminf(X[1], X[2])), xhi = fmaxf(X[0], fmaxf(X[1], X[2]));
      const float ylo = fminf(Y[0], fminf(Y[1], Y[2])), yhi = fmaxf(Y[0], fmaxf(Y[1], Y[2]));
      long long imin, imax, jmin, jmax;
      /* area certainly not clamped after all: the weights are barycentric up
         to the -1e-8 slack, so every covered pixel centre lies in the
         triangle's extent (as in k_cover) and the per-pixel test runs over
         that box only */
      if (fabsf(A) - errA > 1e-15f) {
        const float mb = eps + 1e-6f * ((xhi - xlo) + (yhi - ylo)) + 1e-12f;
        centre_range(xlo - mb, xhi + mb, W, imin, imax);
        centre_range(ylo - mb, yhi + mb, H, jmin, jmax);
      } else {
        reference_box(xlo - eps, xhi + eps, W, imin, imax);
        reference_box(ylo - eps, yhi + eps, H, jmin, jmax);
      }
      const float tau = 1.001e-8f * (fabsf(A) + errA + 1e-16f) + 1e-37f;
      const bool may_pos = A + errA >= 0.f; /* an area of exactly 0 is clamped to +1e-16 */
      const bool may_neg = A - errA < 0.f;
      ExactTri ex;
      bool ex_ok = false;
      if (CHECK) {
        d3 wv[3];
        exact_vertices(G, (long long)t32, wv);
        ex_ok = exact_tri(scene, wv, ex);
        if (ex_ok)
          for (long long j = ex.jmin; j <= ex.jmax; j++)
            for (long long i = ex.imin; i <= ex.imax; i++) {
              double w0, w1, w2;
              if (exact_weights(ex, i, j, R.xs, R.ys, w0, w1, w2) && (i < imin || i > imax || j < jmin || j > jmax))
                atomicAdd(checks + 2, 1u);
            }
      }
      for (long long j = jmin; j <= jmax && (CHECK || !to_tiny); j++) {
        const float py = R.ysf[j];
        for (long long i = imin; i <= imax && (CHECK || !to_tiny); i++) {
          const float px = R.xsf[i];
          const float ep = 0.5f * kU32;
          bool out;
          if (refined) {
            /* the edge values from the refined edges, for each possible sign of the area */
            bool po = false, no = false;
#pragma unroll
            for (int k = 0; k < 3; k++) {
              const int a = (k + 1) % 3;
              const float ux = px - X[a], uy = py - Y[a];
              const float eux = eps + ep + kU32 * fabsf(ux), euy = eps + ep + kU32 * fabsf(uy);
              const float f = ux * sdy[k] - uy * sdx[k];
              const float ef = 1.1f * (fabsf(ux) * sde[k] + eux * fabsf(sdy[k]) + eux * sde[k] + fabsf(uy) * sde[k] +
                                       euy * fabsf(sdx[k]) + euy * sde[k] +
                                       2.f * kU32 * (fabsf(ux * sdy[k]) + fabsf(uy * sdx[k])) + kU32 * fabsf(f));
              po = po || (f + ef < -tau);
              no = no || (f - ef > tau);
            }
            out = (!may_pos || po) && (!may_neg || no);
          } else {
            float e0, e1, e2;
            const float f0 = edge_eval(E0, px, py, ep, eps, e0);
            const float f1 = edge_eval(E1, px, py, ep, eps, e1);
            const float f2 = edge_eval(E2, px, py, ep, eps, e2);
            const bool pos_out = (f0 + e0 < -tau) || (f1 + e1 < -tau) || (f2 + e2 < -tau);
            const bool neg_out = (f0 - e0 > tau) || (f1 - e1 > tau) || (f2 - e2 > tau);
            out = (!may_pos || pos_out) && (!may_neg || neg_out);
          }
          if (CHECK && ex_ok) {
            double x0, x1, x2;
            if (exact_weights(ex, i, j, R.xs, R.ys, x0, x1, x2) && out) atomicAdd(checks + 2, 1u);
          }
          to_tiny = to_tiny || !out;
        }
      }
    }
    const unsigned long long rt = block_reserve<128>(R.tiny_count, to_tiny);
    if (to_tiny && rt < R.tiny_cap) R.tiny[rt] = t32; /* overflow: the host re-runs the slab */
  }
}

/*
 * k_raster: the cover list and the sliver list in one grid.  Block
 * iterations take the cover list's 128-entry blocks first, then the sliver
 * list's; each iteration is one list's, so the block-wide appends stay
 * uniform.  Blocks of 128 threads: a block-wide append waits for four
 * warps, not eight (256-thread blocks: 0.65 ms per bench frame, 128: 0.63).
 */
template <typename T, bool CHECK>
__global__ void __launch_bounds__(128, 8)
k_raster(Geo G, SceneDev scene, TriDev tri, RasterDev R, unsigned* __restrict__ checks) {
  pdl_enter();
  const long long nc = (long long)*R.cover_count, ns = (long long)*R.sliver_count;
  const long long bc = (nc + 127) / 128, bs = (ns + 127) / 128;
  for (long long b = blockIdx.x; b < bc + bs; b += gridDim.x) {
    if (b < bc) cover_block<CHECK>(G, scene, tri, R, checks, 128 * b, nc);
    else sliver_block<T, CHECK>(G, scene, R, checks, 128 * (b - bc), ns);
  }
}

/* ------------------------------------------------------------------ */
/* k_finish: the reference's arithmetic for the candidates that can win */
/* ------------------------------------------------------------------ */
/* one tiny-list triangle (a call of its own: its registers stay out of the
   candidate loop's allocation) */
template <bool CHECK>
__device__ __noinline__ void finish_tiny(const Geo& G, const SceneDev& scene, unsigned t, const RasterDev& R,
                                         unsigned long long order_base, unsigned* checks) {
  tiny_triangle<CHECK>(G, scene, t, R, order_base, checks);
}

/*
 * k_finish: the candidates that can still win (the reference's fragment
 * test), then the tiny list (the reference's arithmetic for the whole
 * triangle), in one grid; both end in the z-buffer's 128-bit maximum, so
 * their order does not matter.  A block filters kFinChunk candidates at a
 * time against the final depth floors into a shared list and runs the FP64
 * test in whole rounds of its 256 threads once the list holds kFinRun of
 * them, keeping the rest for the next round (an FP64 warp instruction costs
 * the same with one active lane as with 32).
 */
constexpr unsigned kFinChunk = 1024, kFinRun = 512;
template <bool CHECK>
__global__ void __launch_bounds__(256, 4)
k_finish(Geo G, SceneDev scene, RasterDev R, unsigned long long order_base, unsigned* __restrict__ checks) {
  pdl_enter();
  /* before a chunk is filtered the list holds fewer than kFinRun entries */
  __shared__ Candidate s_live[kFinRun + kFinChunk];
  __shared__ unsigned s_n;
  const unsigned long long nc = min(*R.cand_count, R.cand_cap), nt = min(*R.tiny_count, R.tiny_cap);
  const unsigned long long nb = (nc + kFinChunk - 1) / kFinChunk;
  if (threadIdx.x == 0) s_n = 0u;
  __syncthreads();
  unsigned have = 0; /* entries in the list (s_n between the filter passes) */
  for (unsigned long long b = blockIdx.x;; b += gridDim.x) {
    const bool more = b < nb;
    if (more) {
#pragma unroll
      for (unsigned u = 0; u < kFinChunk / 256; u++) {
        const unsigned long long q = b * kFinChunk + u * 256 + threadIdx.x;
        if (q < nc) {
          const Candidate c = R.cand[q];
          /* a certainly drawn fragment of this pixel is nearer than anything this one can reach */
          if (f_key(c.dhi) >= R.zlo[c.pixel]) s_live[atomicAdd(&s_n, 1u)] = c;
        }
      }
    }
    __syncthreads();
    const unsigned n = s_n;
    __syncthreads(); /* every thread has read n before the next filter pass adds to it */
    if (threadIdx.x == 0 && n > have) atomicAdd(R.live_count, (unsigned long long)(n - have));
    have = n;
    if (n >= kFinRun || !more) {
      const unsigned take = more ? n / 256 * 256 : n; /* whole rounds, all at the end */
      for (unsigned e = threadIdx.x; e < take; e += 256) {
        const Candidate c = s_live[e];
        const unsigned pj = c.pixel / (unsigned)scene.width;
        exact_fragment<CHECK>(G, scene, c.t, c.pixel - pj * (unsigned)scene.width, pj, R, order_base, checks);
      }
      __syncthreads();
      /* the rest (fewer than 256, from take >= 256 on) to the front */
      const unsigned rest = n - take;
      Candidate c = {};
      if (threadIdx.x < rest) c = s_live[take + threadIdx.x];
      __syncthreads();
      if (threadIdx.x < rest) s_live[threadIdx.x] = c;
      if (threadIdx.x == 0) s_n = rest;
      __syncthreads();
      have = rest;
    }
    if (!more) break;
  }
  for (unsigned long long q = blockIdx.x * 256ULL + threadIdx.x; q < nt; q += (unsigned long long)gridDim.x * 256ULL)
    finish_tiny<CHECK>(G, scene, R.tiny[q], R, order_base, checks);
}

/* shading (render.c:137-159, normal.c:6-165), once per contour object     */
/* ------------------------------------------------------------------ */
/*
 * After all slabs of an object, every pixel the object won is shaded from the
 * field itself: the winner's drawing order gives its cell and rank (order =
 * base + 12 cell + rank), cell codes are recomputed from the corner values,
 * and each vertex normal is the normalised sum of the area-weighted face
 * normals of the triangles that share the vertex's cube edge, over the
 * neighbour cells in the reference's order.  Four lanes take one pixel: lane
 * m < 3 builds the normal of vertex m, lane 0 then blends them.  The FP32
 * pass settles a pixel when each channel's truncation is certain; the
 * others go to the FP64 pass, which repeats the reference's arithmetic in
 * its order.
 */
struct WinCell {
  long long i, j, k;
  unsigned r;
};

/* the object's triangle that owns a pixel, from the slot's order */
__device__ __forceinline__ bool winner_cell(const FieldDev& F, unsigned long long lo, unsigned long long obase,
                                            WinCell& w) {
  const unsigned long long order = lo >> 24;
  const unsigned long long ncx = (unsigned long long)(F.nx - 1), ncy = (unsigned long long)(F.ny - 1);
  const unsigned long long ncz = (unsigned long long)(F.nz - 1);
  if (order < obase || order - obase >= 12ULL * ncx * ncy * ncz) return false;
  /* rel / 12 by a multiply-high (exact for every 64-bit rel), the rest by
     the 32-bit divisions while the cells fit (no 64-bit division) */
  const unsigned long long rel = order - obase, c = __umul64hi(rel, 0xAAAAAAAAAAAAAAABULL) >> 3;
  w.r = (unsigned)(rel - 12ULL * c);
  if (c < (1ULL << 32)) {
    const unsigned row = fast_div((unsigned)c, F.div_cx);
    w.i = (long long)((unsigned)c - row * (unsigned)ncx);
    const unsigned kk = fast_div(row, F.div_cy);
    w.k = kk;
    w.j = (long long)(row - kk * (unsigned)ncy);
  } else {
    const unsigned long long row = c / ncx;
    w.i = (long long)(c - row * ncx);
    w.k = (long long)(row / ncy);
    w.j = (long long)(row - (unsigned long long)w.k * ncy);
  }
  return true;
}

/* one thread per pixel: the pixels whose owner is one of the object's triangles */
__global__ void __launch_bounds__(256)
k_winners(const Slot* __restrict__ canvas, long long npx, unsigned long long obase, unsigned long long span,
          unsigned* __restrict__ win, unsigned long long* __restrict__ win_count) {
  pdl_enter();
  for (long long base = blockIdx.x * (long long)blockDim.x; base < npx; base += (long long)gridDim.x * blockDim.x) {
    const long long p = base + threadIdx.x;
    bool won = false;
    if (p < npx) {
      const unsigned long long order = canvas[p].lo >> 24;
      won = order >= obase && order - obase < span;
    }
    const unsigned long long w = block_reserve<256>(win_count, won);
    if (won) win[w] = (unsigned)p;
  }
}

/*
 * Area-weighted face normal in FP32: the reference's area * unit normal
 * equals the cross product of two edges up to a few FP64 ulps; with vertices
 * relative to the cell's corner 0 the edge vectors keep their relative
 * accuracy.  eC: the largest bound of the three components, infinite when
 * none can be given.
 */
__device__ __forceinline__ void tri_wn_f(bool ok, const float rv[3][3], const float er[3][3], float C[3],
                                         float& eC) {
  /* edges from vertex 0 and their cross product (triangulate.c:75-93) */
  float x1[3], x2[3], e1[3], e2[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    x1[d] = rv[1][d] - rv[0][d];
    x2[d] = rv[2][d] - rv[0][d];
    e1[d] = er[1][d] + er[0][d] + kU32 * fabsf(x1[d]);
    e2[d] = er[2][d] + er[0][d] + kU32 * fabsf(x2[d]);
  }
  eC = 0.f;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
    const float p1 = x1[d1] * x2[d2], p2 = x1[d2] * x2[d1];
    C[d] = p1 - p2;
    const float ec = prod_err(x1[d1], e1[d1], x2[d2], e2[d2]) + prod_err(x1[d2], e1[d2], x2[d1], e2[d1]) +
                     kU32 * fabsf(C[d]);
    eC = fmaxf(eC, 1.1f * ec + 1e-15f * (fabsf(p1) + fabsf(p2)));
  }
  /* a zero cross product (area exactly 0, also by FP64 underflow) makes the
     reference's weighted normal 0 * (0 * inf) = NaN, which propagates to the
     pixel: unless some component is certainly away from 0, the triangle is
     left to the FP64 pass (a small but nonzero one only adds its small
     absolute bound) */
  const float cmax = fmaxf(fabsf(C[0]), fmaxf(fabsf(C[1]), fabsf(C[2])));
  if (!ok || !isfinite(cmax) || !isfinite(eC) || !(cmax - eC > 1e-30f)) eC = INFINITY;
}

/* 1 / sqrt(x) by the hardware approximation (PTX rsqrt.approx.f32: relative
   error below 2^-22.9 = 4.3u; no FP64 pipe, unlike the correctly rounded
   square root and division of a build without fused multiply-adds) */
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

/*
 * A / |A| in FP32 as A * rsqrt_approx(A . A): the sum of squares is within
 * 3u of its value, the approximation within 4.3u, the products within u,
 * so each component is within 6.9u |component| of the exact unit vector;
 * len = (A . A) * r stands for |A| within 5u.  The bound on the distance to
 * the reference's unit vector B / |B| adds 2 e_E / (|A| - e_E) for a
 * componentwise bound e on |A - B| (e_E = sqrt(3) e, Euclidean); infinite
 * when |A| is too small.
 */
__device__ __forceinline__ float unit_vec(const float A[3], float e, float U[3]) {
  const float ss = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  const float r = rsqrt_approx(ss);
  const float len = ss * r * (1.f - 6.f * kU32);
  const float ee = 1.7321f * e;
#pragma unroll
  for (int d = 0; d < 3; d++) U[d] = A[d] * r;
  if (!(len > 4.f * ee) || !(len > 1e-30f) || !isfinite(r)) return INFINITY;
  return 1.01f * 2.f * ee / (len - ee) + 8.f * kU32;
}

/* code of cell (i, j, k) whose corner 0 is node `base` */
template <typename T>
__device__ __forceinline__ unsigned cell_code_at(const FieldDev& F, long long base);

/* the same, read from the classification's codes when they are kept */
template <typename T>
__device__ __forceinline__ unsigned cell_code_ijk(const FieldDev& F, long long i, long long j, long long k) {
  if (F.codes) return __ldg(F.codes + (k * (F.ny - 1) + j) * (F.nx - 1) + i);
  return cell_code_at<T>(F, (k * F.ny + j) * F.nx + i);
}

template <typename T>
__device__ __forceinline__ unsigned cell_code_at(const FieldDev& F, long long base) {
  const T* f = static_cast<const T*>(F.data);
  unsigned code = 0;
#pragma unroll
  for (int c = 0; c < 8; c++)
    code |= (unsigned)node_above<T>(F, f, base + (c & 1) + ((c >> 1) & 1) * F.nx + (c >> 2) * F.nx * F.ny) << c;
  return code;
}


/* the pixel's colour from the three FP32 vertex normals: false when a
   channel's truncation is not certain */
__device__ __forceinline__ bool blend_f(const SceneDev& scene, const RasterDev& R, long long p, unsigned long long lo,
                                        const float N[3][3], const float en[3], unsigned rgb_in, unsigned& rgb_out) {
  const unsigned long long tag = ((lo >> 24) << 24) | R.epoch;
  const ulonglong2 k0 = R.winfo[3 * p], k1 = R.winfo[3 * p + 1], k2 = R.winfo[3 * p + 2];
  if (!(k0.y == tag && k1.y == tag && k2.y == tag)) return false;
  const ulonglong2 kk[3] = {k0, k1, k2};
  float M[3] = {0.f, 0.f, 0.f}, eM = 0.f, wsum = 0.f;
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const float w = to_f(__longlong_as_double((long long)kk[m].x));
    const float ew = 2.f * kU32 * fabsf(w) + 1e-37f;
#pragma unroll
    for (int d = 0; d < 3; d++) M[d] += w * N[m][d];
    eM += ew * 1.01f + fabsf(w) * en[m];
    wsum += fabsf(w);
  }
  eM += 4.f * kU32 * wsum * 1.01f;
  float U[3];
  const float eN = unit_vec(M, eM, U);
  if (!isfinite(eN)) return false;
  const float* L = scene.f_light;
  const float dotv = U[0] * L[0] + U[1] * L[1] + U[2] * L[2];
  const float l1 = fabsf(L[0]) + fabsf(L[1]) + fabsf(L[2]);
  /* the unit vector's bound, the light's rounding to float, and the dot
     product's rounding (bounded by the sum of |n_i L_i| <= l1 (1 + eN)) */
  const float ed = eN * l1 + 5.f * kU32 * (1.f + eN) * l1 + 1e-30f;
  const float alo = fmaxf(0.f, fabsf(dotv) - ed), ahi = fabsf(dotv) + ed;
  /* factor = max(0.15, |d|): certainly clamped, certainly not, or undecided */
  const bool clamped = ahi < 0.149999f, free = alo > 0.150001f;
  if (clamped) {
    rgb_out = R.clamp_rgb;
    return true;
  }
  if (!free) return false;
  unsigned out = 0;
#pragma unroll
  for (int ch = 0; ch < 3; ch++) {
    const float cc = (float)((rgb_in >> (16 - 8 * ch)) & 255u);
    const float xl = alo * cc * (1.f - 4.f * kU32), xh = ahi * cc * (1.f + 4.f * kU32);
    const float fl = floorf(xl);
    if (floorf(xh) != fl || !(xl >= 0.f)) return false;
    out |= ((unsigned)(int)fl & 255u) << (16 - 8 * ch);
  }
  rgb_out = out;
  return true;
}

constexpr unsigned kFull = 0xFFFFFFFFu;

/* appends each flagged lane's pixel to a list, one atomic per warp */
__device__ __forceinline__ void warp_append(bool flag, unsigned p, unsigned* list, unsigned long long* count) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned bal = __ballot_sync(kFull, flag);
  unsigned long long a0 = 0;
  if (lane == 0 && bal) a0 = atomicAdd(count, (unsigned long long)__popc(bal));
  a0 = __shfl_sync(kFull, a0, 0);
  if (flag) list[a0 + __popc(bal & ((1u << lane) - 1u))] = p;
}

/*
 * FP32 pass over the won pixels, 32 pixels per block and iteration, four
 * threads per pixel (blocks of 128 threads: 0.47 -> 0.46 ms per bench frame
 * against 64 pixels and 256 threads; the block barriers wait for fewer warps).  Neighbouring pixels share most of their vertices'
 * neighbourhoods, so each block first gathers the triangles around its
 * pixels' vertices into a shared hash of (cell, rank) keys, computes each
 * distinct triangle's FP32 weighted normal once, then every (pixel, vertex)
 * thread sums its triangles' normals (the bound covers any summation order)
 * and lane 0 of each pixel blends the three.  A pixel whose neighbourhood
 * does not fit goes to the FP64 pass.  Self-check: every pixel is listed for
 * the FP64 pass, and the FP32 colour, where certain, is kept for it to compare.
 */
constexpr int kShadeHash = 512; /* distinct triangles per block and iteration */
constexpr int kShadeList = 24;    /* triangles around one cube edge (at most 16) */
constexpr unsigned long long kEmptyKey = ~0ULL;

/* (cell, rank) as a hash key: i, j, k below 2^20 each, rank below 12 (never all ones) */
__device__ __forceinline__ unsigned long long tri_key(long long i, long long j, long long k, unsigned r) {
  return ((unsigned long long)k << 44) | ((unsigned long long)j << 24) | ((unsigned long long)i << 4) | r;
}

/* slot of `key` in the block's table (inserted when absent, fresh = true), -1 when full */
__device__ __forceinline__ int hash_slot(unsigned long long* keys, unsigned long long key, bool& fresh) {
  unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ULL) >> 54) & (kShadeHash - 1);
  for (int probe = 0; probe < kShadeHash; probe++) {
    const unsigned long long prev = atomicCAS(keys + h, kEmptyKey, key);
    if (prev == kEmptyKey || prev == key) {
      fresh = prev == kEmptyKey;
      return (int)h;
    }
    h = (h + 1) & (kShadeHash - 1);
  }
  fresh = false;
  return -1;
}

template <typename T, bool CHECK>
__global__ void __launch_bounds__(128)
k_shade_f(FieldDev F, SceneDev scene, RasterDev R, const unsigned long long* __restrict__ lut,
          unsigned long long obase, unsigned rgb_in) {
  pdl_enter();
  __shared__ unsigned long long keys[kShadeHash];
  __shared__ float4 wnf[kShadeHash];
  __shared__ unsigned short lists[kShadeList][128];
  __shared__ unsigned short todo[kShadeHash];
  __shared__ unsigned ntodo;
  for (int q = threadIdx.x; q < kShadeHash; q += blockDim.x) keys[q] = kEmptyKey;
  if (threadIdx.x == 0) ntodo = 0;
  __syncthreads();
  const unsigned long long n = *R.win_count;
  const unsigned tid = threadIdx.x, lane = tid & 31u, m = tid & 3u, g0 = lane & ~3u;
  const ThrF th = thr_f(F.threshold);
  for (unsigned long long base = blockIdx.x * 32ULL; base < n; base += gridDim.x * 32ULL) {
    const unsigned long long q = base + tid / 4;
    /* gather: the (cell, rank) of every triangle around this thread's vertex */
    unsigned p = 0;
    unsigned long long lo = 0;
    WinCell wc;
    bool ok = false, full = false;
    int cnt = 0;
    if (q < n) {
      p = R.win[q];
      lo = R.canvas[p].lo;
      ok = winner_cell(F, lo, obase, wc);
    }
    if (ok && m < 3) {
      const unsigned code = cell_code_ijk<T>(F, wc.i, wc.j, wc.k);
      const int ed = (int)((__ldg(lut + code * 12 + wc.r) >> (18 + 5 * m)) & 31);
      const int nn = c_nb_count[ed];
      for (int s = 0; s < nn; s++) {
        const long long ni = wc.i + c_nb[ed][s][2], nj = wc.j + c_nb[ed][s][1], nk = wc.k + c_nb[ed][s][0];
        const unsigned le = (unsigned)c_nb[ed][s][3];
        const unsigned ncode = cell_code_ijk<T>(F, ni, nj, nk);
        for (unsigned mask = __ldg(g_edge_tris + ncode * 19 + le); mask; mask &= mask - 1) {
          const int r = __ffs(mask) - 1;
          bool fresh;
          const int slot = hash_slot(keys, tri_key(ni, nj, nk, (unsigned)r), fresh);
          if (slot < 0 || cnt >= kShadeList) {
            full = true;
            continue;
          }
          if (fresh) todo[atomicAdd(&ntodo, 1u)] = (unsigned short)slot;
          lists[cnt++][tid] = (unsigned short)slot;
        }
      }
    }
    __syncthreads();
    /* each distinct triangle's FP32 weighted normal, once */
    const unsigned nd = ntodo;
    for (unsigned w = tid; w < nd; w += blockDim.x) {
      const int slot = todo[w];
      const unsigned long long key = keys[slot];
      const long long i = (long long)((key >> 4) & 0xFFFFFu), j = (long long)((key >> 24) & 0xFFFFFu);
      const long long k = (long long)(key >> 44);
      const long long nb = (k * F.ny + j) * F.nx + i;
      const unsigned code = cell_code_ijk<T>(F, i, j, k);
      const unsigned long long e = __ldg(lut + code * 12 + (key & 15u));
      const float sp[3] = {__ldg(F.dgx + i), __ldg(F.dgy + j), __ldg(F.dgz + k)};
      const T* fd = static_cast<const T*>(F.data);
      float rv[3][3], er[3][3];
      bool tok = true;
#pragma unroll
      for (int v = 0; v < 3; v++) {
        const unsigned a = (unsigned)((e >> (6 * v)) & 7), b = (unsigned)((e >> (6 * v + 3)) & 7);
        const typename ShadeVal<T>::type va =
            ShadeVal<T>::load(fd, nb + (a & 1u) + ((a >> 1) & 1u) * F.nx + (long long)(a >> 2) * F.nx * F.ny);
        const typename ShadeVal<T>::type vb =
            ShadeVal<T>::load(fd, nb + (b & 1u) + ((b >> 1) & 1u) * F.nx + (long long)(b >> 2) * F.nx * F.ny);
        float f = 0.f, e_f = 0.f;
        if (interp_shade(F, th, va, vb, f, e_f) < 0) tok = false;
        rel_pos(F, sp, a, b, f, e_f, rv[v], er[v]);
      }
      float C[3], eC;
      tri_wn_f(tok, rv, er, C, eC);
      wnf[slot] = make_float4(C[0], C[1], C[2], eC);
    }
    __syncthreads();
    /* vertex normal: the normalised sum over the triangles around the edge (normal.c:78-158) */
    float N[3] = {0.f, 0.f, 0.f}, en = INFINITY;
    if (ok && m < 3 && !full) {
      float S[3] = {0.f, 0.f, 0.f}, eS = 0.f, asum = 0.f;
      for (int t = 0; t < cnt; t++) {
        const float4 c = wnf[lists[t][tid]];
        S[0] += c.x;
        S[1] += c.y;
        S[2] += c.z;
        eS += c.w;
        asum += fabsf(c.x) + fabsf(c.y) + fabsf(c.z);
      }
      eS += (float)(cnt + 1) * kU32 * asum + 1e-15f * asum; /* FP32 and the reference's FP64 summation */
      en = unit_vec(S, eS, N);
    }
    float Nv[3][3], env[3];
#pragma unroll
    for (int mm = 0; mm < 3; mm++) {
#pragma unroll
      for (int d = 0; d < 3; d++) Nv[mm][d] = __shfl_sync(kFull, N[d], g0 + mm);
      env[mm] = __shfl_sync(kFull, en, g0 + mm);
    }
    bool listed = false;
    if (ok && m == 0) {
      unsigned rgb = 0;
      const bool sure = isfinite(env[0]) && isfinite(env[1]) && isfinite(env[2]) &&
                        blend_f(scene, R, p, lo, Nv, env, rgb_in, rgb);
      if (CHECK) {
        R.shade_check[p] = sure ? (1u << 24) | rgb : 0u;
        listed = true;
      } else if (sure) {
        R.canvas[p].lo = (lo & ~0xFFFFFFULL) | rgb;
      } else {
        listed = true;
      }
    }
    warp_append(listed, p, R.amb, R.amb_count); /* at most the won pixels: fits */
    /* empty the table for the next pixels */
    for (unsigned w = tid; w < nd; w += blockDim.x) keys[todo[w]] = kEmptyKey;
    __syncthreads();
    if (tid == 0) ntodo = 0;
    __syncthreads();
  }
}

/*
 * FP64 pass over the pixels the FP32 pass could not settle, in three steps so
 * that the FP64 work runs on full warps: list every (pixel, vertex)'s
 * neighbour triangles in the reference's order, compute each listed
 * triangle's area-weighted face normal, then sum them in that order and
 * blend.  A list entry is (global cell) * 16 + rank.
 */
__device__ __forceinline__ int vertex_edge(const FieldDev& F, const unsigned long long* lut, const WinCell& wc, int m,
                                           double vals[8], unsigned long long& e) {
  const unsigned code = cell_code_any(F, wc.i, wc.j, wc.k, vals);
  e = lut[code * 12 + wc.r];
  return (int)((e >> (18 + 5 * m)) & 31);
}

/* visits the neighbour triangles around cube edge ed of cell (i, j, k) in the
   reference's order (normal.c:78-158): fn(entry) */
template <typename Fn>
__device__ __forceinline__ void for_edge_triangles(const FieldDev& F, const unsigned long long* lut, long long i,
                                                   long long j, long long k, int ed, Fn fn) {
  const long long ncx = F.nx - 1, ncy = F.ny - 1;
  const int nn = c_nb_count[ed];
  for (int q = 0; q < nn; q++) {
    const long long ni = i + c_nb[ed][q][2], nj = j + c_nb[ed][q][1], nk = k + c_nb[ed][q][0];
    const unsigned le = (unsigned)c_nb[ed][q][3];
    const unsigned long long cell = (unsigned long long)((nk * ncy + nj) * ncx + ni);
    double vals[8];
    const unsigned code = F.codes ? (unsigned)__ldg(F.codes + cell) : cell_code_any(F, ni, nj, nk, vals);
    /* ascending rank: the reference's order within the cell */
    for (unsigned mask = __ldg(g_edge_tris + code * 19 + le); mask; mask &= mask - 1)
      fn(cell * 16ULL + (unsigned long long)(__ffs(mask) - 1));
  }
}

/* step 1: one thread per (pixel, vertex); spans[q] = (first entry, count),
   count 0xFFFFFFFF when the entries did not fit */
__global__ void __launch_bounds__(256)
k_nb_list(FieldDev F, RasterDev R, const unsigned long long* __restrict__ lut_g, const unsigned* __restrict__ pixels,
          const unsigned long long* __restrict__ count, unsigned long long obase, unsigned long long* __restrict__ ent,
          unsigned long long ent_cap, unsigned long long* __restrict__ ent_count, uint2* __restrict__ spans) {
  pdl_trigger();
  /* the table through L1: a copy in each block's shared memory cost every
     block 24 KB of loads and a barrier */
  const unsigned long long* lut = lut_g;
  pdl_wait();
  const unsigned long long n = 3 * *count;
  const unsigned long long iters = (n + blockDim.x - 1) / blockDim.x;
  /* every lane of a warp runs the same iterations (warp-wide reservations) */
  for (unsigned long long it = blockIdx.x; it < iters; it += gridDim.x) {
    const unsigned long long q = it * blockDim.x + threadIdx.x;
    WinCell wc;
    bool ok = false;
    int ed = 0;
    unsigned cnt = 0;
    if (q < n) {
      const unsigned long long pq = q / 3;
      const int m = (int)(q - 3 * pq);
      ok = winner_cell(F, R.canvas[pixels[pq]].lo, obase, wc);
      if (ok) {
        double vals[8];
        unsigned long long e;
        ed = vertex_edge(F, lut, wc, m, vals, e);
        for_edge_triangles(F, lut, wc.i, wc.j, wc.k, ed, [&](unsigned long long) { cnt++; });
      }
    }
    /* warp-aggregated reservation */
    const unsigned lane = threadIdx.x & 31u;
    unsigned incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned y = __shfl_up_sync(kFull, incl, d);
      if ((int)lane >= d) incl += y;
    }
    unsigned long long w0 = 0;
    if (lane == 31 && incl) w0 = atomicAdd(ent_count, (unsigned long long)incl);
    w0 = __shfl_sync(kFull, w0, 31);
    const unsigned long long first = w0 + (incl - cnt);
    if (q < n) {
      const bool fits = first + cnt <= ent_cap;
      spans[q] = make_uint2((unsigned)first, ok && fits ? cnt : 0xFFFFFFFFu);
      if (ok) {
        /* the entries below ent_cap are written even when the span does not
           fit whole: k_nb_wn takes every entry below min(count, ent_cap),
           and one left unwritten would hold a stale (cell, rank) word */
        unsigned long long at = first;
        for_edge_triangles(F, lut, wc.i, wc.j, wc.k, ed, [&](unsigned long long x) {
          if (at < ent_cap) ent[at] = x;
          at++;
        });
      }
    }
  }
}

/* step 2: one thread per listed triangle, its exact area-weighted face normal
   (triangulate.c:40-93, normal.c:39-40) */
__global__ void __launch_bounds__(256)
k_nb_wn(FieldDev F, const unsigned long long* __restrict__ lut, const unsigned long long* __restrict__ ent,
        unsigned long long ent_cap, const unsigned long long* __restrict__ ent_count, double* __restrict__ wn_out) {
  pdl_enter();
  const unsigned long long n = min(*ent_count, ent_cap);
  const unsigned long long ncx = (unsigned long long)(F.nx - 1), ncy = (unsigned long long)(F.ny - 1);
  for (unsigned long long q = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; q < n;
       q += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long x = ent[q], cell = x >> 4, row = cell / ncx;
    const long long i = (long long)(cell - row * ncx), k = (long long)(row / ncy);
    const long long j = (long long)(row - (unsigned long long)k * ncy);
    if (k >= F.nz - 1 || (x & 15) >= 12) continue; /* not a cell of the field: never read past it */
    double vals[8];
    const unsigned code = cell_code_any(F, i, j, k, vals);
    const unsigned long long e = __ldg(lut + code * 12 + (x & 15));
    d3 v[3], fn, wn;
    double area;
#pragma unroll
    for (int qv = 0; qv < 3; qv++) {
      const int a = (int)((e >> (6 * qv)) & 7), b = (int)((e >> (6 * qv + 3)) & 7);
      v[qv] = interpolate(F.threshold, corner_pos(F, i, j, k, a), vals[a], corner_pos(F, i, j, k, b), vals[b]);
    }
    face_normal(v, fn, area, wn);
    wn_out[3 * q + 0] = wn.x;
    wn_out[3 * q + 1] = wn.y;
    wn_out[3 * q + 2] = wn.z;
  }
}

/* step 3: four lanes per pixel; lane m < 3 sums vertex m's normals in the
   reference's order and normalises, lane 0 blends and colours (render.c:137-159) */
template <bool CHECK>
__global__ void __launch_bounds__(256)
k_shade(FieldDev F, SceneDev scene, RasterDev R, const unsigned long long* __restrict__ lut,
        const unsigned* __restrict__ pixels, const unsigned long long* __restrict__ count, unsigned long long obase,
        const uint2* __restrict__ spans, const double* __restrict__ wn_in, unsigned rgb_in,
        unsigned* __restrict__ checks) {
  pdl_enter();
  const unsigned long long n = *count;
  const unsigned lane = threadIdx.x & 31u, m = lane & 3u, g0 = lane & ~3u;
  const long long W = scene.width;
  const double cr = (double)((rgb_in >> 16) & 255), cg = (double)((rgb_in >> 8) & 255),
               cb = (double)(rgb_in & 255);
  const unsigned long long step = (unsigned long long)gridDim.x * (blockDim.x / 4);
  for (unsigned long long base = ((unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) / 4; base < n;
       base += step) {
    const unsigned long long q = base + lane / 4;
    d3 nm = {0., 0., 0.};
    int good = 1;
    if (q < n && m < 3) {
      const uint2 sp = spans[3 * q + m];
      if (sp.y == 0xFFFFFFFFu) {
        good = 0;
      } else {
        d3 sum = {0., 0., 0.};
        for (unsigned t = 0; t < sp.y; t++) {
          const double* w = wn_in + 3 * ((unsigned long long)sp.x + t);
          sum = v_add(sum, d3{w[0], w[1], w[2]});
        }
        nm = v_normalise(sum);
      }
    }
    d3 n3[3];
#pragma unroll
    for (int mm = 0; mm < 3; mm++)
      n3[mm] = {__shfl_sync(kFull, nm.x, g0 + mm), __shfl_sync(kFull, nm.y, g0 + mm),
                __shfl_sync(kFull, nm.z, g0 + mm)};
    good = __shfl_sync(kFull, good, g0) & __shfl_sync(kFull, good, g0 + 1) & __shfl_sync(kFull, good, g0 + 2);
    if (q >= n || m != 0 || !good) continue;
    const unsigned p = pixels[q];
    const unsigned long long lo = R.canvas[p].lo;
    WinCell wc;
    if (!winner_cell(F, lo, obase, wc)) continue;
    const unsigned long long tag = ((lo >> 24) << 24) | R.epoch;
    const ulonglong2 k0 = R.winfo[3 * p], k1 = R.winfo[3 * p + 1], k2 = R.winfo[3 * p + 2];
    double w0, w1, w2;
    if (k0.y == tag && k1.y == tag && k2.y == tag) {
      /* the weights the winning fragment was drawn with */
      w0 = __longlong_as_double((long long)k0.x);
      w1 = __longlong_as_double((long long)k1.x);
      w2 = __longlong_as_double((long long)k2.x);
    } else {
      /* a stale or mixed record: the same arithmetic again (render.c:102-133) */
      double vals[8];
      unsigned long long e;
      vertex_edge(F, lut, wc, 0, vals, e);
      d3 v[3];
#pragma unroll
      for (int qv = 0; qv < 3; qv++) {
        const int a = (int)((e >> (6 * qv)) & 7), b = (int)((e >> (6 * qv + 3)) & 7);
        v[qv] = interpolate(F.threshold, corner_pos(F, wc.i, wc.j, wc.k, a), vals[a],
                            corner_pos(F, wc.i, wc.j, wc.k, b), vals[b]);
      }
      ExactTri x;
      const long long pj = (long long)(p / (unsigned long long)W), pi = (long long)p - pj * W;
      if (!exact_tri(scene, v, x) || !exact_weights(x, pi, pj, R.xs, R.ys, w0, w1, w2)) continue;
    }
    const d3 nrm = v_normalise(v_add(v_mul(w0, n3[0]), v_add(v_mul(w1, n3[1]), v_mul(w2, n3[2]))));
    const double factor = fmax(0.15, fabs(v_dot(nrm, scene.light)));
    const unsigned r8 = (unsigned)(unsigned char)(int)dmul(factor, cr);
    const unsigned g8 = (unsigned)(unsigned char)(int)dmul(factor, cg);
    const unsigned b8 = (unsigned)(unsigned char)(int)dmul(factor, cb);
    const unsigned rgb = (r8 << 16) | (g8 << 8) | b8;
    if (CHECK) {
      /* the FP32 colour, where it was certain, must be this one */
      const unsigned f = R.shade_check[p];
      if ((f >> 24) && (f & 0xFFFFFFu) != rgb) atomicAdd(checks + 5, 1u);
    }
    R.canvas[p].lo = (lo & ~0xFFFFFFULL) | rgb;
  }
}

/* ------------------------------------------------------------------ */
/* lines (line.c:26-119), canvas init, resolve                          */
/* ------------------------------------------------------------------ */
__global__ void k_lines(const LineSegDev* __restrict__ segs, int nseg, long long W, long long H,
                        Slot* __restrict__ canvas, unsigned long long order_base, unsigned* zerr) {
  pdl_enter();
  const int sidx = blockIdx.x;
  if (sidx >= nseg) return;
  const LineSegDev L = segs[sidx];
  if (!L.valid) return;
  const double p0x = L.p0x, p0y = L.p0y, p0z = L.p0z, p1x = L.p1x, p1y = L.p1y, p1z = L.p1z;
  const long long xmin = (long long)dsub(fmin(p0x, p1x), 1.), xmax = (long long)dadd(fmax(p0x, p1x), 1.);
  const long long ymin = (long long)dsub(fmin(p0y, p1y), 1.), ymax = (long long)dadd(fmax(p0y, p1y), 1.);
  const long long imin = min(W - 1, max(0LL, xmin)), imax = min(W - 1, max(0LL, xmax));
  const long long jmin = min(H - 1, max(0LL, ymin)), jmax = min(H - 1, max(0LL, ymax));
  const double a = dsub(p1y, p0y);
  const double b = dadd(-p1x, p0x);
  const double c = dsub(dmul(dsub(p1x, p0x), p0y), dmul(dsub(p1y, p0y), p0x));
  const double h = dmul(0.5, L.width);
  const double thr = dmul(h, h);
  const double ab2 = dadd(dmul(a, a), dmul(b, b));
  const double dx = dsub(p1x, p0x), dy = dsub(p1y, p0y);
  const double dd = dadd(dmul(dx, dx), dmul(dy, dy));
  const long long nx = imax - imin + 1, ny = jmax - jmin + 1;
  const unsigned long long order = order_base + (unsigned long long)sidx;
  for (long long q = threadIdx.x; q < nx * ny; q += blockDim.x) {
    const long long i = imin + q % nx, j = jmin + q / nx;
    const double di = (double)i, dj = (double)j;
    const double num = dadd(dadd(dmul(a, di), dmul(b, dj)), c);
    const double distance = ddiv(dmul(num, num), ab2);
    if (thr < distance) continue;
    const double param = ddiv(dmul(-1., dadd(dmul(dsub(p1x, p0x), dsub(p0x, di)), dmul(dsub(p1y, p0y), dsub(p0y, dj)))), dd);
    const double dist0 = drcp(dadd(ddiv(param, p1z), ddiv(dsub(1., param), p0z)));
    const unsigned long long key = depth_key(dist0);
    Slot* s = canvas + j * W + i;
    slot_max(s, key, (order << 24) | L.rgb, zerr);
  }
}

__global__ void k_canvas_init(Slot* canvas, unsigned* zlo, long long n, unsigned long long hi, unsigned long long lo) {
  pdl_enter();
  const unsigned floor_key = f_key(-__int_as_float(0x7f800000));
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    canvas[p].hi = hi;
    canvas[p].lo = lo;
    zlo[p] = floor_key;
  }
}

/* ppm body: rows flipped (output.c:113-123); optional canvas-order depth */
__global__ void k_resolve(const Slot* __restrict__ canvas, long long W, long long H, unsigned char* __restrict__ rgb,
                          double* __restrict__ depth) {
  pdl_enter();
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < W * H; p += (long long)gridDim.x * blockDim.x) {
    const long long r = p / W, i = p % W;
    const Slot s = canvas[(H - 1 - r) * W + i];
    rgb[3 * p + 0] = (unsigned char)(s.lo >> 16);
    rgb[3 * p + 1] = (unsigned char)(s.lo >> 8);
    rgb[3 * p + 2] = (unsigned char)(s.lo);
    if (depth) {
      const Slot sc = canvas[p];
      depth[p] = depth_from_key(sc.hi);
    }
  }
}

/* ------------------------------------------------------------------ */
/* launchers                                                           */
/* ------------------------------------------------------------------ */
/* SMs of the first device the library runs on (thread-safe one-time query) */
static int num_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      v = 1;
    }
    return v;
  }();
  return n;
}

static std::atomic<int> g_cls_z{kClsZ}, g_emit_per_sm{8}, g_raster_per_sm{8};
static std::atomic<int> g_pdl{0};

void set_dependent_launch(int on) { g_pdl = on ? 1 : 0; }
int dependent_launch() { return g_pdl.load(); }

int set_launch_shape(const LaunchShape& s) {
  if (s.cls_z < 1 || s.cls_z > 1024 || s.emit_per_sm < 1 || s.emit_per_sm > 32 || s.raster_per_sm < 1 ||
      s.raster_per_sm > 32)
    return 1;
  g_cls_z = s.cls_z;
  g_emit_per_sm = s.emit_per_sm;
  g_raster_per_sm = s.raster_per_sm;
  return 0;
}

LaunchShape launch_shape() { return LaunchShape{g_cls_z.load(), g_emit_per_sm.load(), g_raster_per_sm.load()}; }

/* every kernel launch of the library: programmatic dependent launch (the
   kernels call pdl_wait() before they touch what earlier work produced) */
/* C3D_LAUNCH_CHECK=1 in the environment: every launch is followed by a
   synchronisation of its stream and an error check that names the kernel
   (debugging; changes timing) */
static bool launch_check() {
  static const bool on = [] {
    const char* e = getenv("C3D_LAUNCH_CHECK");
    return e && e[0] == '1';
  }();
  return on;
}

template <typename... KArgs, typename... Args>
static void launch_k(void (*kernel)(KArgs...), const char* name, dim3 grid, dim3 block, size_t smem,
                     cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = g_pdl.load() ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
  if (launch_check()) {
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
      fprintf(stderr, "[CONTOUR3D ERROR] %s (grid %u x %u x %u): %s\n", name, grid.x, grid.y, grid.z,
              cudaGetErrorString(e));
  }
}

static int grid_for(long long n, int threads, int per_sm) {
  const int g_num_sms = num_sms();
  long long b = (n + threads - 1) / threads;
  const long long cap = (long long)g_num_sms * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

int upload_tables(const unsigned char code_count[256], const signed char nb[19][4][4],
                  const unsigned char nb_count[19], const unsigned short edge_tris[256 * 19]) {
  if (cudaMemcpyToSymbol(c_code_count, code_count, 256) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(g_edge_tris, edge_tris, sizeof(unsigned short) * 256 * 19) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_nb, nb, sizeof(signed char) * 19 * 16) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_nb_count, nb_count, 19) != cudaSuccess) return 1;
  /* beyond the default 48 KB of dynamic shared memory: set once per device */
  if (cudaFuncSetAttribute(k_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScanWriteSmem) !=
      cudaSuccess)
    return 1;
  return 0;
}

/* cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda
   link); looked up once, thread-safely (a function-local static) */
static PFN_cuTensorMapEncodeTiled_v12000 lookup_tensor_map_encoder() {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  cudaGetLastError();
  return nullptr;
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = lookup_tensor_map_encoder();
  return fn;
}

/* the field as a 3-D tensor map with one node plane of a classify tile per box,
   or false when TMA cannot address it (row or plane pitch not a multiple of 16
   bytes, base not 16-byte aligned, more than 2^31 nodes along an axis) */
static bool classify_tensor_map(const FieldDev& F, CUtensorMap* map) {
  const size_t es = F.is_f32 ? 4 : 8;
  if (((uintptr_t)F.data & 15) || (F.nx * es) % 16 || F.nx >= (1LL << 31) || F.ny >= (1LL << 31) ||
      F.nz >= (1LL << 31))
    return false;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)F.nx, (cuuint64_t)F.ny, (cuuint64_t)F.nz};
  const cuuint64_t strides[2] = {(cuuint64_t)(F.nx * es), (cuuint64_t)(F.nx * F.ny * es)};
  const cuuint32_t box[3] = {(cuuint32_t)(F.is_f32 ? TmaBox<float>::kX : TmaBox<double>::kX), kClsY + 1, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(map, F.is_f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                         const_cast<void*>(F.data), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

/* ThrSet's range form of a field's threshold.  thr_key is the key with -0
   taken as +0, so lo = thr_key + 1 and the keys above run up to key(+inf);
   thr_f_key is the unsigned float key of the least float above the
   threshold, turned back into the float's bits (a zero of either sign
   admits both zeros: lo = key(-0) = -1). */
static void thr_range(const FieldDev& F, ThrSet& ts, int t) {
  const long long kInfKey = 0x7FF0000000000000LL;
  ts.lo[t] = (unsigned long long)F.thr_key + 1;
  ts.cnt[t] = F.thr_nan ? 0ULL : (unsigned long long)kInfKey - (unsigned long long)F.thr_key;
  const int kInfKeyF = 0x7F800000;
  const unsigned K = F.thr_f_key;
  const unsigned u = (K & 0x80000000u) ? (K & 0x7FFFFFFFu) : ~K; /* the float's bits */
  int flo;
  if ((u << 1) == 0) flo = -1;
  else flo = (u & 0x80000000u) ? (int)(u ^ 0x7FFFFFFFu) : (int)u;
  ts.flo[t] = (unsigned)flo;
  ts.fcnt[t] = F.thr_f_ok ? (unsigned)((long long)kInfKeyF - flo + 1) : 0u;
}

template <typename T>
static void launch_classify_tma(const CUtensorMap& map, const FieldDev& F, const SlabDev& S, const ThrSet& ts,
                                const CodeOut& out, unsigned* err, const dim3& grid, cudaStream_t st) {
  switch (ts.n) {
    case 1: launch_k(k_classify_tma<T, 1>, "k_classify_tma", grid, kClsX, 0, st, map, F, S, ts, out, err); break;
    case 2: launch_k(k_classify_tma<T, 2>, "k_classify_tma", grid, kClsX, 0, st, map, F, S, ts, out, err); break;
    case 3: launch_k(k_classify_tma<T, 3>, "k_classify_tma", grid, kClsX, 0, st, map, F, S, ts, out, err); break;
    default: launch_k(k_classify_tma<T, 4>, "k_classify_tma", grid, kClsX, 0, st, map, F, S, ts, out, err); break;
  }
}

int launch_classify(const FieldDev* Fs, int nf, const SlabDev& S0, unsigned char* const* codes, unsigned* err,
                    cudaStream_t st) {
  /* codes[q] receives the cell codes of threshold q; the scan turns them into counts */
  const FieldDev& F = Fs[0];
  SlabDev S = S0;
  /* bricks of the launch shape's depth, or shallower when the slab is thin:
     at least 16 bricks per SM, so that every SM has copies in flight (the
     deeper the brick, the fewer node planes are read twice) */
  const long long bxy = ((F.nx - 1 + kClsX - 1) / kClsX) * ((F.ny - 1 + kClsY - 1) / kClsY);
  const long long want_z = ((long long)num_sms() * 16 + bxy - 1) / bxy;
  S.cls_z = (int)std::max(std::min<long long>(launch_shape().cls_z, (S.nslices + want_z - 1) / want_z),
                          (long long)std::min(8, launch_shape().cls_z));
  const dim3 grid((unsigned)((F.nx - 1 + kClsX - 1) / kClsX), (unsigned)((F.ny - 1 + kClsY - 1) / kClsY),
                  (unsigned)((S.nslices + S.cls_z - 1) / S.cls_z));
  CUtensorMap map;
  if (classify_tensor_map(F, &map)) {
    /* one pass over the field for up to kMaxThr thresholds */
    for (int q0 = 0; q0 < nf; q0 += kMaxThr) {
      ThrSet ts;
      CodeOut out;
      ts.n = min(kMaxThr, nf - q0);
      for (int t = 0; t < ts.n; t++) {
        thr_range(Fs[q0 + t], ts, t);
        out.codes[t] = codes[q0 + t];
      }
      if (F.is_f32) launch_classify_tma<float>(map, F, S, ts, out, err, grid, st);
      else launch_classify_tma<double>(map, F, S, ts, out, err, grid, st);
    }
    return (nf + kMaxThr - 1) / kMaxThr;
  }
  /* rows TMA cannot address: plain loads, still one pass per kMaxThr objects */
  for (int q0 = 0; q0 < nf; q0 += kMaxThr) {
    ThrSet ts;
    CodeOut out;
    ts.n = min(kMaxThr, nf - q0);
    for (int t = 0; t < ts.n; t++) {
      thr_range(Fs[q0 + t], ts, t);
      out.codes[t] = codes[q0 + t];
    }
    for (int t = ts.n; t < kMaxThr; t++) out.codes[t] = nullptr;
    if (F.is_f32)
      launch_k(k_classify_multi<float>, "k_classify_multi", grid, kClsX, 0, st, F.data, F.nx, F.ny, S, ts, out);
    else
      launch_k(k_classify_multi<double>, "k_classify_multi", grid, kClsX, 0, st, F.data, F.nx, F.ny, S, ts, out);
  }
  return (nf + kMaxThr - 1) / kMaxThr;
}

void make_cls_item(const FieldDev* Fs, int nf, const SlabDev& S, unsigned char* const* codes, ClsItem* it) {
  const FieldDev& F = Fs[0];
  memset(it, 0, sizeof *it);
  it->data = F.data;
  it->is_f32 = F.is_f32;
  it->nx = F.nx;
  it->ny = F.ny;
  it->S = S;
  it->ts.n = min(nf, kMaxThr);
  for (int t = 0; t < it->ts.n; t++) {
    thr_range(Fs[t], it->ts, t);
    it->out.codes[t] = codes[t];
  }
  it->nbx = (unsigned)((F.nx - 1 + kClsX - 1) / kClsX);
  it->nby = (unsigned)((F.ny - 1 + kClsY - 1) / kClsY);
  it->nbz = (unsigned)((S.nslices + S.cls_z - 1) / S.cls_z);
}

void launch_classify_queue(const ClsItem* items, int nitems, unsigned long long nunits, unsigned long long* next,
                           cudaStream_t st) {
  if (nitems < 1 || nunits == 0) return;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_classify_queue, kClsX, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 8;
  const unsigned long long cap = (unsigned long long)num_sms() * (unsigned long long)per_sm;
  const unsigned grid = (unsigned)(nunits < cap ? nunits : cap);
  launch_k(k_classify_queue, "k_classify_queue", grid, kClsX, 0, st, items, nitems, nunits, next);
}

long long scan_state_words(long long n) { return std::max((n + kScanTile - 1) / kScanTile, 1LL) + 1; }

size_t voff_bytes(long long n) {
  return ((size_t)(n + 1) * sizeof(unsigned short) + 255) / 256 * 256 + sizeof(unsigned) * (size_t)scan_state_words(n);
}

VOffDev voff_layout(void* base, long long n) {
  const size_t rel_bytes = ((size_t)(n + 1) * sizeof(unsigned short) + 255) / 256 * 256;
  VOffDev o;
  o.rel = static_cast<unsigned short*>(base);
  o.seg = reinterpret_cast<unsigned*>(static_cast<char*>(base) + rel_bytes);
  return o;
}

cudaError_t launch_scan(const unsigned char* codes, long long n, unsigned long long* state, unsigned* offsets,
                        const VOffDev& voff, unsigned long long* totals, unsigned* tri_cell,
                        unsigned long long tri_cap, bool want_offsets, unsigned* ovf, unsigned* err,
                        cudaStream_t st) {
  const long long nseg = scan_state_words(n) - 1;
  const cudaError_t e = cudaMemsetAsync(state, 0, sizeof(unsigned long long) * (size_t)(nseg + 1), st);
  if (e != cudaSuccess) return e;
  launch_k(k_scan, "k_scan", (unsigned)nseg, kScanThreads, kScanWriteSmem, st, codes, n, nseg, state, offsets,
           voff, totals, tri_cell, tri_cap, want_offsets ? 1 : 0, ovf, err);
  return cudaSuccess;
}

void launch_vertices(const FieldDev& F, const SlabDev& S, const SceneDev& scene, const unsigned char* codes,
                     const VOffDev& voff, long long n, const VertDev& V, cudaStream_t st) {
  const unsigned blocks = (unsigned)((n + kVTile - 1) / kVTile);
  if (F.is_f32) launch_k(k_vertices<float>, "k_vertices", blocks, kVThreads, 0, st, F, S, scene, codes, voff, n, V);
  else launch_k(k_vertices<double>, "k_vertices", blocks, kVThreads, 0, st, F, S, scene, codes, voff, n, V);
}

void launch_emit(const FieldDev& F, const SlabDev& S, const SceneDev& scene, const unsigned long long* lut,
                 const unsigned char* codes, const unsigned* offsets,
                 const VOffDev& voff, const unsigned* tri_cell, const unsigned long long* total,
                 long long tri_bound, const TriDev& tri, const RasterDev& R, const VertDev& V, unsigned* checks,
                 cudaStream_t st) {
  const int g = grid_for(tri_bound, 256, g_emit_per_sm);
  if (!R.cover_count) {
    /* inspection: edge ids and flags only */
    launch_k(k_emit<double, false, false>, "k_emit", g, 256, 0, st, F, S, scene, lut, codes, offsets, voff,
             tri_cell, total, tri, R, V, checks);
  } else if (checks) {
    if (F.is_f32)
      launch_k(k_emit<float, true, true>, "k_emit", g, 256, 0, st, F, S, scene, lut, codes, offsets, voff,
               tri_cell, total, tri, R, V, checks);
    else
      launch_k(k_emit<double, true, true>, "k_emit", g, 256, 0, st, F, S, scene, lut, codes, offsets, voff,
               tri_cell, total, tri, R, V, checks);
  } else {
    if (F.is_f32)
      launch_k(k_emit<float, false, true>, "k_emit", g, 256, 0, st, F, S, scene, lut, codes, offsets, voff,
               tri_cell, total, tri, R, V, checks);
    else
      launch_k(k_emit<double, false, true>, "k_emit", g, 256, 0, st, F, S, scene, lut, codes, offsets, voff,
               tri_cell, total, tri, R, V, checks);
  }
}

unsigned long long emit_list_slack(long long tri_bound) {
  return emit_slack_for((unsigned long long)grid_for(tri_bound, 256, g_emit_per_sm));
}

void launch_exact_all(const Geo& G, const unsigned long long* total, long long tri_bound, const TriDev& tri,
                      cudaStream_t st) {
  launch_k(k_exact_all, "k_exact_all", grid_for(tri_bound, 256, 8), 256, 0, st, G, total, tri);
}

void launch_normals(const FieldDev& F, const SlabDev& S, const unsigned* offsets, const unsigned* tri_cell,
                    const unsigned long long* total, long long tri_bound, const TriDev& tri, cudaStream_t st) {
  const int g = grid_for(tri_bound, 256, 8);
  launch_k(k_normals, "k_normals", g, 256, 0, st, F, S, offsets, tri_cell, total, tri);
}

void launch_raster(const Geo& G, const SceneDev& scene, long long tri_bound, const TriDev& tri,
                   const RasterDev& R, unsigned* checks, cudaStream_t st) {
  /* cover and sliver entries together number at most the slab's triangles */
  const int g = grid_for(tri_bound, 128, 2 * g_raster_per_sm);
  if (G.F.is_f32) {
    if (checks) launch_k(k_raster<float, true>, "k_raster", g, 128, 0, st, G, scene, tri, R, checks);
    else launch_k(k_raster<float, false>, "k_raster", g, 128, 0, st, G, scene, tri, R, checks);
  } else {
    if (checks) launch_k(k_raster<double, true>, "k_raster", g, 128, 0, st, G, scene, tri, R, checks);
    else launch_k(k_raster<double, false>, "k_raster", g, 128, 0, st, G, scene, tri, R, checks);
  }
}

void launch_finish(const Geo& G, const SceneDev& scene, long long bound, const RasterDev& R,
                   unsigned long long order_base, unsigned* checks, cudaStream_t st) {
  const int g = grid_for(bound, 256, g_raster_per_sm);
  if (checks) launch_k(k_finish<true>, "k_finish", g, 256, 0, st, G, scene, R, order_base, checks);
  else launch_k(k_finish<false>, "k_finish", g, 256, 0, st, G, scene, R, order_base, checks);
}

void launch_shade_f(const FieldDev& F, const SceneDev& scene, const RasterDev& R, const unsigned long long* lut,
                    unsigned long long obase, unsigned rgb, cudaStream_t st) {
  const long long npx = scene.width * scene.height;
  const unsigned long long span = 12ULL * (unsigned long long)((F.nx - 1) * (F.ny - 1) * (F.nz - 1));
  launch_k(k_winners, "k_winners", grid_for(npx, 256, 8), 256, 0, st, R.canvas, npx, obase, span, R.win, R.win_count);
  /* no single-precision shading without node spacings (a converter) or for
     axes of 2^20 nodes and more (hash keys): every pixel to the FP64 pass */
  if (!F.dgx || F.nx > (1 << 20) || F.ny > (1 << 20) || F.nz > (1 << 20)) return;
  const int gs = grid_for(4 * npx, 128, 16); /* four threads per pixel */
  if (F.is_f32) {
    if (R.shade_check) launch_k(k_shade_f<float, true>, "k_shade_f", gs, 128, 0, st, F, scene, R, lut, obase, rgb);
    else launch_k(k_shade_f<float, false>, "k_shade_f", gs, 128, 0, st, F, scene, R, lut, obase, rgb);
  } else {
    if (R.shade_check) launch_k(k_shade_f<double, true>, "k_shade_f", gs, 128, 0, st, F, scene, R, lut, obase, rgb);
    else launch_k(k_shade_f<double, false>, "k_shade_f", gs, 128, 0, st, F, scene, R, lut, obase, rgb);
  }
}

void launch_shade_exact(const FieldDev& F, const SceneDev& scene, const RasterDev& R, const unsigned long long* lut,
                        const unsigned* pixels, const unsigned long long* count, long long npix,
                        unsigned long long obase, unsigned long long* ent, unsigned long long ent_cap,
                        unsigned long long* ent_count, uint2* spans, double* wn, unsigned rgb, unsigned* checks,
                        cudaStream_t st) {
  if (npix <= 0) return;
  launch_k(k_nb_list, "k_nb_list", grid_for(3 * npix, 256, 8), 256, 0, st, F, R, lut, pixels, count, obase, ent,
           ent_cap, ent_count, spans);
  launch_k(k_nb_wn, "k_nb_wn", grid_for((long long)ent_cap, 256, 8), 256, 0, st, F, lut, ent, ent_cap, ent_count, wn);
  const int gs = grid_for(4 * npix, 256, 8);
  if (checks && R.shade_check)
    launch_k(k_shade<true>, "k_shade", gs, 256, 0, st, F, scene, R, lut, pixels, count, obase, spans, wn, rgb, checks);
  else
    launch_k(k_shade<false>, "k_shade", gs, 256, 0, st, F, scene, R, lut, pixels, count, obase, spans, wn, rgb, checks);
}

void launch_lines(const LineSegDev* segs, int nseg, long long W, long long H, Slot* canvas,
                  unsigned long long order_base, unsigned* zerr, cudaStream_t st) {
  if (nseg > 0) launch_k(k_lines, "k_lines", nseg, 128, 0, st, segs, nseg, W, H, canvas, order_base, zerr);
}

void launch_canvas_init(Slot* canvas, unsigned* zlo, long long n, unsigned long long hi, unsigned long long lo,
                        cudaStream_t st) {
  launch_k(k_canvas_init, "k_canvas_init", grid_for(n, 256, 8), 256, 0, st, canvas, zlo, n, hi, lo);
}

void launch_resolve(const Slot* canvas, long long W, long long H, unsigned char* rgb, double* depth,
                    cudaStream_t st) {
  launch_k(k_resolve, "k_resolve", grid_for(W * H, 256, 8), 256, 0, st, canvas, W, H, rgb, depth);
}

}  // namespace c3d
