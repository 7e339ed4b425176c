/*
 * kernels.cu -- sm_103a kernels of the isosurface-to-image path.
 *
 * One contour object is processed in z-slabs of cells.  Per slab:
 *   k_classify   cell codes -> triangle count per cell          (HBM: field read)
 *   k_scan       decoupled-look-back exclusive scan of the counts, writing
 *                per-cell offsets and the triangle -> cell map
 *   k_emit       one thread per triangle: vertices, face normal, weighted
 *                normal, cube-edge ids, screen projection      (FP64)
 *   k_normals    one thread per rendered triangle: area-weighted vertex
 *                normals gathered over the cells sharing each cube edge
 *   k_raster     one thread per rendered triangle: bounding-box walk,
 *                barycentric test, harmonic depth, shading, 128-bit
 *                (depth, order) max into the z-buffer
 * and once per frame k_canvas_init, k_lines and k_resolve.
 *
 * The FP64 stages run one triangle per thread on compacted triangle lists so
 * that warps stay converged: on GB300 an FP64 warp instruction costs the same
 * whether 2 or 32 lanes are active.
 *
 * Reference correspondence (file:line of the reference tree):
 *   k_classify/k_emit  src/contour3d/contour/triangulate.c:95-342
 *   k_normals          src/contour3d/contour/normal.c:6-165
 *   k_raster           src/contour3d/contour/render.c:48-163, project.c:9-67
 *   k_lines            src/contour3d/line.c:26-119
 *   k_resolve          src/contour3d/output.c:10-30, 113-123
 *   slab / interior    src/contour3d/contour/main.c:38-112
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <cuda/atomic>
#include "c3d_common.cuh"
#include "c3d_kernels.h"

namespace c3d {

__constant__ unsigned char c_code_count[256];
/* normal.c:78-158: per cube edge, the (dk, dj, di, local edge id) of the
   cells sharing it, in the reference's accumulation order */
__constant__ signed char c_nb[19][4][4];
__constant__ unsigned char c_nb_count[19];

/* ------------------------------------------------------------------ */
/* field access                                                        */
/* ------------------------------------------------------------------ */
template <typename T>
__device__ __forceinline__ double load_value(const T* f, long long idx) {
  return (double)__ldg(f + idx);
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

/* ------------------------------------------------------------------ */
/* k_classify                                                          */
/* ------------------------------------------------------------------ */
template <typename T>
__global__ void __launch_bounds__(256) k_classify(FieldDev F, SlabDev S, unsigned char* __restrict__ counts) {
  const long long ncx = F.nx - 1, ncy = F.ny - 1;
  const long long ncell = S.nslices * ncx * ncy;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const long long i = c % ncx;
    const long long j = (c / ncx) % ncy;
    const long long k = S.kfirst + c / (ncx * ncy);
    double v[8];
    const unsigned code = cell_code<T>(F, i, j, k, v);
    counts[c] = c_code_count[code];
  }
}

/* ------------------------------------------------------------------ */
/* k_scan: single-pass decoupled look-back exclusive scan              */
/* ------------------------------------------------------------------ */
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;  /* cells per thread */
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr unsigned long long kFlagAgg = 1ULL << 62;
constexpr unsigned long long kFlagPrefix = 2ULL << 62;
constexpr unsigned long long kValueMask = (1ULL << 62) - 1;

__global__ void __launch_bounds__(kScanThreads)
k_scan(const unsigned char* __restrict__ counts, long long n, unsigned* __restrict__ offsets,
       unsigned long long* __restrict__ tile_state,
       unsigned* __restrict__ tile_counter, unsigned long long* __restrict__ total,
       unsigned* __restrict__ err) {
  __shared__ unsigned s_tile;
  __shared__ unsigned long long s_warp[kScanThreads / 32];
  __shared__ unsigned long long s_excl;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const unsigned tile = s_tile;
  const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;

  unsigned char cnt[kScanItems];
  unsigned sum = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    const long long c = base + q;
    cnt[q] = c < n ? counts[c] : 0;
    sum += cnt[q];
  }
  /* block-wide exclusive scan of the per-thread sums */
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
    unsigned long long w = lane < kScanThreads / 32 ? s_warp[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, d);
      if (lane >= d) w += y;
    }
    if (lane < kScanThreads / 32) s_warp[lane] = w;  /* inclusive per warp */
  }
  __syncthreads();
  const unsigned long long block_agg = s_warp[kScanThreads / 32 - 1];
  const unsigned long long thread_excl = (warp ? s_warp[warp - 1] : 0) + incl - sum;

  /* publish and look back (warp 0) */
  if (warp == 0) {
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> my(tile_state[tile]);
    if (lane == 0)
      my.store((tile == 0 ? kFlagPrefix : kFlagAgg) | block_agg, cuda::memory_order_release);
    unsigned long long excl = 0;
    if (tile > 0) {
      long long pred = (long long)tile - 1;
      int spins = 0;
      bool done = false;
      while (!done) {
        /* each lane inspects one predecessor, nearest first */
        const long long p = pred - lane;
        unsigned long long st = kFlagPrefix;  /* beyond tile 0: neutral */
        if (p >= 0) {
          cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> ps(tile_state[p]);
          st = ps.load(cuda::memory_order_acquire);
        }
        const unsigned invalid = __ballot_sync(0xFFFFFFFFu, p >= 0 && (st >> 62) == 0);
        const unsigned prefix = __ballot_sync(0xFFFFFFFFu, p >= 0 && (st >> 62) == 2);
        /* lanes up to (excluding) the first invalid one are usable; stop at the first prefix */
        const unsigned first_invalid = invalid ? __ffs(invalid) - 1 : 32;
        const unsigned first_prefix = prefix ? __ffs(prefix) - 1 : 32;
        if (first_prefix < first_invalid) {
          unsigned long long v = (lane <= (int)first_prefix && p >= 0) ? (st & kValueMask) : 0;
#pragma unroll
          for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
          excl += v;
          done = true;
        } else if (first_invalid == 32) {
          /* 32 aggregates and no prefix yet: consume them and move on */
          unsigned long long v = p >= 0 ? (st & kValueMask) : 0;
#pragma unroll
          for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
          excl += v;
          pred -= 32;
          if (pred < 0) done = true;
        } else if (first_invalid > 0) {
          /* consume the aggregates before the first invalid predecessor */
          unsigned long long v = (lane < (int)first_invalid && p >= 0) ? (st & kValueMask) : 0;
#pragma unroll
          for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
          excl += v;
          pred -= first_invalid;
        } else {
          if (++spins > (1 << 22)) {
            if (lane == 0) atomicOr(err, kErrScanTimeout);
            done = true;
          } else {
            __nanosleep(64);
          }
        }
      }
      if (lane == 0) my.store(kFlagPrefix | ((excl + block_agg) & kValueMask), cuda::memory_order_release);
    }
    if (lane == 0) s_excl = excl;
  }
  __syncthreads();
  unsigned long long run = s_excl + thread_excl;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    const long long c = base + q;
    if (c <= n) offsets[c] = (unsigned)run;  /* offsets[n] = total */
    if (c == n) *total = run;
    run += cnt[q];
  }
}

/* triangle -> cell map from the offsets: tri_cell[offsets[c] + r] = c */
__global__ void __launch_bounds__(256)
k_fill_tri_cell(const unsigned* __restrict__ offsets, long long n, unsigned* __restrict__ tri_cell) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    const unsigned a = offsets[c], b = offsets[c + 1];
    for (unsigned u = a; u < b; u++) tri_cell[u] = (unsigned)c;
  }
}

/* ------------------------------------------------------------------ */
/* k_emit                                                              */
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

template <typename T>
__global__ void __launch_bounds__(256)
k_emit(FieldDev F, SlabDev S, SceneDev scene, const unsigned long long* __restrict__ lut_g,
       const unsigned* __restrict__ offsets, const unsigned* __restrict__ tri_cell,
       const unsigned long long* __restrict__ total_p, TriDev tri) {
  __shared__ unsigned long long lut[kLutEntries];
  for (int q = threadIdx.x; q < kLutEntries; q += blockDim.x) lut[q] = lut_g[q];
  __syncthreads();
  const long long T_ = (long long)*total_p;
  const long long ncx = F.nx - 1, ncy = F.ny - 1;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T_;
       t += (long long)gridDim.x * blockDim.x) {
    const unsigned c = tri_cell[t];
    const unsigned r = (unsigned)(t - offsets[c]);
    const long long i = c % ncx;
    const long long j = (c / ncx) % ncy;
    const long long kl = c / (ncx * ncy);
    const long long k = S.kfirst + kl;
    double val[8];
    const unsigned code = cell_code<T>(F, i, j, k, val);
    const unsigned long long e = lut[code * 12 + r];
    d3 v[3];
    unsigned edges = 0;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const int a = (int)((e >> (6 * q)) & 7), b = (int)((e >> (6 * q + 3)) & 7);
      v[q] = interpolate(F.threshold, corner_pos(F, i, j, k, a), val[a], corner_pos(F, i, j, k, b), val[b]);
      edges |= (unsigned)((e >> (18 + 5 * q)) & 31) << (5 * q);
    }
    /* triangulate.c:75-93 */
    d3 fn = v_cross(v_sub(v[1], v[0]), v_sub(v[2], v[0]));
    const double area = dsqrt(v_dot(fn, fn));
    fn = v_mul(ddiv(1., area), fn);
    const d3 wn = v_mul(area, fn); /* normal.c:39-40 */
    tri.wn[0][t] = wn.x;
    tri.wn[1][t] = wn.y;
    tri.wn[2][t] = wn.z;
    /* rendered set: interior cells of the slab's own slices (contour/main.c:70-112) */
    const bool rendered = i >= 1 && i <= ncx - 2 && j >= 1 && j <= ncy - 2 &&
                          k >= S.krender0 && k < S.krender1;
    unsigned meta = edges | (rendered ? kMetaRendered : 0u);
    if (rendered) {
      bool ok = true;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        d3 p;
        ok = project(scene, v[q], p) && ok;
        tri.proj[3 * q + 0][t] = p.x;
        tri.proj[3 * q + 1][t] = p.y;
        tri.proj[3 * q + 2][t] = p.z;
      }
      if (!ok) meta |= kMetaCulled;
    }
    tri.meta[t] = meta;
    if (tri.dbg_vert) {
#pragma unroll
      for (int q = 0; q < 3; q++) {
        tri.dbg_vert[(9 * t) + 3 * q + 0] = v[q].x;
        tri.dbg_vert[(9 * t) + 3 * q + 1] = v[q].y;
        tri.dbg_vert[(9 * t) + 3 * q + 2] = v[q].z;
      }
      tri.dbg_fn[3 * t + 0] = fn.x;
      tri.dbg_fn[3 * t + 1] = fn.y;
      tri.dbg_fn[3 * t + 2] = fn.z;
      tri.dbg_area[t] = area;
    }
  }
}

/* ------------------------------------------------------------------ */
/* k_normals                                                           */
/* ------------------------------------------------------------------ */
__global__ void __launch_bounds__(256)
k_normals(FieldDev F, SlabDev S, const unsigned* __restrict__ offsets, const unsigned* __restrict__ tri_cell,
          const unsigned long long* __restrict__ total_p, TriDev tri) {
  const long long T_ = (long long)*total_p;
  const long long ncx = F.nx - 1, ncy = F.ny - 1;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T_;
       t += (long long)gridDim.x * blockDim.x) {
    const unsigned meta = tri.meta[t];
    if (!(meta & kMetaRendered)) continue;
    const long long c = tri_cell[t];
#pragma unroll 1
    for (int m = 0; m < 3; m++) {
      const int e = (meta >> (5 * m)) & 31;
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
      const d3 n = v_normalise(sum);
      tri.vn[3 * m + 0][t] = n.x;
      tri.vn[3 * m + 1][t] = n.y;
      tri.vn[3 * m + 2][t] = n.z;
    }
  }
}

/* ------------------------------------------------------------------ */
/* k_raster                                                            */
/* ------------------------------------------------------------------ */
__global__ void __launch_bounds__(256)
k_raster(SceneDev scene, const unsigned long long* __restrict__ total_p, TriDev tri,
         const double* __restrict__ xs, const double* __restrict__ ys, Slot* __restrict__ canvas,
         unsigned long long order_base, unsigned rgb_in) {
  const long long T_ = (long long)*total_p;
  const long long W = scene.width, H = scene.height;
  const double cr = (double)((rgb_in >> 16) & 255), cg = (double)((rgb_in >> 8) & 255),
               cb = (double)(rgb_in & 255);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T_;
       t += (long long)gridDim.x * blockDim.x) {
    const unsigned meta = tri.meta[t];
    if (!(meta & kMetaRendered) || (meta & kMetaCulled)) continue;
    d3 v0 = {tri.proj[0][t], tri.proj[1][t], tri.proj[2][t]};
    d3 v1 = {tri.proj[3][t], tri.proj[4][t], tri.proj[5][t]};
    d3 v2 = {tri.proj[6][t], tri.proj[7][t], tri.proj[8][t]};
    /* render.c:81-89 */
    const long long xmin = (long long)dsub(dmul(dadd(0.5, fmin(v0.x, fmin(v1.x, v2.x))), (double)W), 1.);
    const long long xmax = (long long)dadd(dmul(dadd(0.5, fmax(v0.x, fmax(v1.x, v2.x))), (double)W), 1.);
    const long long ymin = (long long)dsub(dmul(dadd(0.5, fmin(v0.y, fmin(v1.y, v2.y))), (double)H), 1.);
    const long long ymax = (long long)dadd(dmul(dadd(0.5, fmax(v0.y, fmax(v1.y, v2.y))), (double)H), 1.);
    const long long imin = min(W - 1, max(0LL, xmin)), imax = min(W - 1, max(0LL, xmax));
    const long long jmin = min(H - 1, max(0LL, ymin)), jmax = min(H - 1, max(0LL, ymax));
    const double area = edge_fn(v0, v1, v2);
    const double area_inv = ddiv(1., area < 0. ? fmin(area, -1.e-16) : fmax(area, +1.e-16));
    const d3 n0 = {tri.vn[0][t], tri.vn[1][t], tri.vn[2][t]};
    const d3 n1 = {tri.vn[3][t], tri.vn[4][t], tri.vn[5][t]};
    const d3 n2 = {tri.vn[6][t], tri.vn[7][t], tri.vn[8][t]};
    const unsigned long long order = order_base + (unsigned long long)t;
    for (long long j = jmin; j <= jmax; j++) {
      for (long long i = imin; i <= imax; i++) {
        const d3 v3 = {xs[i], ys[j], 0.};
        const double w0 = dmul(area_inv, edge_fn(v1, v2, v3));
        const double w1 = dmul(area_inv, edge_fn(v2, v0, v3));
        const double w2 = dmul(area_inv, edge_fn(v0, v1, v3));
        if (w0 < -1.e-8 || w1 < -1.e-8 || w2 < -1.e-8) continue;
        const double dist0 = ddiv(1., dadd(dadd(ddiv(w0, v0.z), ddiv(w1, v1.z)), ddiv(w2, v2.z)));
        const unsigned long long key = depth_key(dist0);
        Slot* s = canvas + j * W + i;
        const unsigned long long seen = *(volatile unsigned long long*)&s->hi;
        if (key < seen) continue;
        const d3 n = v_normalise(v_add(v_mul(w0, n0), v_add(v_mul(w1, n1), v_mul(w2, n2))));
        const double factor = fmax(0.15, fabs(v_dot(n, scene.light)));
        const unsigned r8 = (unsigned)(unsigned char)(int)dmul(factor, cr);
        const unsigned g8 = (unsigned)(unsigned char)(int)dmul(factor, cg);
        const unsigned b8 = (unsigned)(unsigned char)(int)dmul(factor, cb);
        slot_max(s, key, (order << 24) | (r8 << 16) | (g8 << 8) | b8);
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* lines (line.c:26-119), canvas init, resolve                          */
/* ------------------------------------------------------------------ */
__global__ void k_lines(const LineSegDev* __restrict__ segs, int nseg, long long W, long long H,
                        Slot* __restrict__ canvas, unsigned long long order_base) {
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
    const double dist0 = ddiv(1., dadd(ddiv(param, p1z), ddiv(dsub(1., param), p0z)));
    const unsigned long long key = depth_key(dist0);
    Slot* s = canvas + j * W + i;
    slot_max(s, key, (order << 24) | L.rgb);
  }
}

__global__ void k_canvas_init(Slot* canvas, long long n, unsigned long long hi, unsigned long long lo) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    canvas[p].hi = hi;
    canvas[p].lo = lo;
  }
}

/* ppm body: rows flipped (output.c:113-123); optional canvas-order depth */
__global__ void k_resolve(const Slot* __restrict__ canvas, long long W, long long H, unsigned char* __restrict__ rgb,
                          double* __restrict__ depth) {
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
static int g_num_sms = 0;
static int grid_for(long long n, int threads, int per_sm) {
  if (!g_num_sms) cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, 0);
  long long b = (n + threads - 1) / threads;
  const long long cap = (long long)g_num_sms * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

int upload_tables(const unsigned char code_count[256], const signed char nb[19][4][4],
                  const unsigned char nb_count[19]) {
  if (cudaMemcpyToSymbol(c_code_count, code_count, 256) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_nb, nb, sizeof(signed char) * 19 * 16) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_nb_count, nb_count, 19) != cudaSuccess) return 1;
  return 0;
}

void launch_classify(const FieldDev& F, const SlabDev& S, unsigned char* counts, cudaStream_t st) {
  const long long n = S.nslices * (F.nx - 1) * (F.ny - 1);
  const int g = grid_for(n, 256, 16);
  if (F.is_f32) k_classify<float><<<g, 256, 0, st>>>(F, S, counts);
  else k_classify<double><<<g, 256, 0, st>>>(F, S, counts);
}

void launch_scan(const unsigned char* counts, long long n, unsigned* offsets,
                 unsigned long long* tile_state, unsigned* tile_counter, unsigned long long* total,
                 unsigned* err, cudaStream_t st) {
  const long long tiles = (n + kScanTile) / kScanTile; /* covers position n too */
  cudaMemsetAsync(tile_state, 0, sizeof(unsigned long long) * tiles, st);
  cudaMemsetAsync(tile_counter, 0, sizeof(unsigned), st);
  k_scan<<<(unsigned)tiles, kScanThreads, 0, st>>>(counts, n, offsets, tile_state, tile_counter, total, err);
}

void launch_fill_tri_cell(const unsigned* offsets, long long n, unsigned* tri_cell, cudaStream_t st) {
  k_fill_tri_cell<<<grid_for(n, 256, 16), 256, 0, st>>>(offsets, n, tri_cell);
}

long long scan_tiles(long long n) { return (n + kScanTile) / kScanTile; }

void launch_emit(const FieldDev& F, const SlabDev& S, const SceneDev& scene, const unsigned long long* lut,
                 const unsigned* offsets, const unsigned* tri_cell, const unsigned long long* total,
                 long long tri_bound, const TriDev& tri, cudaStream_t st) {
  const int g = grid_for(tri_bound, 256, 8);
  if (F.is_f32) k_emit<float><<<g, 256, 0, st>>>(F, S, scene, lut, offsets, tri_cell, total, tri);
  else k_emit<double><<<g, 256, 0, st>>>(F, S, scene, lut, offsets, tri_cell, total, tri);
}

void launch_normals(const FieldDev& F, const SlabDev& S, const unsigned* offsets, const unsigned* tri_cell,
                    const unsigned long long* total, long long tri_bound, const TriDev& tri, cudaStream_t st) {
  const int g = grid_for(tri_bound, 256, 8);
  k_normals<<<g, 256, 0, st>>>(F, S, offsets, tri_cell, total, tri);
}

void launch_raster(const SceneDev& scene, const unsigned long long* total, long long tri_bound, const TriDev& tri,
                   const double* xs, const double* ys, Slot* canvas, unsigned long long order_base, unsigned rgb,
                   cudaStream_t st) {
  const int g = grid_for(tri_bound, 256, 8);
  k_raster<<<g, 256, 0, st>>>(scene, total, tri, xs, ys, canvas, order_base, rgb);
}

void launch_lines(const LineSegDev* segs, int nseg, long long W, long long H, Slot* canvas,
                  unsigned long long order_base, cudaStream_t st) {
  if (nseg > 0) k_lines<<<nseg, 128, 0, st>>>(segs, nseg, W, H, canvas, order_base);
}

void launch_canvas_init(Slot* canvas, long long n, unsigned long long hi, unsigned long long lo, cudaStream_t st) {
  k_canvas_init<<<grid_for(n, 256, 8), 256, 0, st>>>(canvas, n, hi, lo);
}

void launch_resolve(const Slot* canvas, long long W, long long H, unsigned char* rgb, double* depth,
                    cudaStream_t st) {
  k_resolve<<<grid_for(W * H, 256, 8), 256, 0, st>>>(canvas, W, H, rgb, depth);
}

}  // namespace c3d
