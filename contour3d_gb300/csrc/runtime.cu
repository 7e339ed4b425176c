/*
 * runtime.cu -- host runtime of the GB300 isosurface path: the drop-in
 * contour3d_execute (reference src/contour3d/main.c:68-146) and the
 * extension entry points of contour3d_gb300.h.
 *
 * Per call: scene constants on the host (same operations as main.c:25-63 and
 * project.c:9-67, compiled without contraction), one device z-buffer of
 * 16-byte slots, then the contour objects field by field: a host field is
 * copied to the device once (in chunks on a copy stream, overlapped with the
 * slabs, when it is large), the objects of one field are classified together
 * per z-slab and take the slab pipeline of kernels.cu in turn, and each
 * object is shaded once after its slabs; then the lines, one resolve pass and
 * one device->host copy of the image.  Device buffers are kept between calls
 * (grow-only) so that repeated frames do not pay for cudaMalloc;
 * contour3d_gb300_release() frees them.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include "contour3d.h"
#include "contour3d_gb300.h"
#include "c3d_common.cuh"
#include "c3d_host.h"
#include "c3d_kernels.h"

namespace c3d {

#define C3D_CUDA(call)                                                           \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      log_error("%s failed: %s", #call, cudaGetErrorString(e_));                 \
      return 1;                                                                  \
    }                                                                            \
  } while (0)

typedef contour3d_vector_t V;

/* ---------------- host vector algebra (vector.c:5-76) ---------------- */
static inline V h_add(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V h_sub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V h_mul(double w, V a) { return {w * a.x, w * a.y, w * a.z}; }
static inline double h_dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V h_cross(V a, V b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline V h_normalise(V a) {
  const double inv = 1. / sqrt(h_dot(a, a));
  return {a.x * inv, a.y * inv, a.z * inv};
}
static inline d3 to_d3(V v) { return {v.x, v.y, v.z}; }

/* host copy of the scene (main.c:13-63) */
struct HostScene {
  V cam, center, lx, ly, normal, light;
  size_t W, H;
};

static HostScene make_scene(const V *cam, const V *light, const size_t sizes[2], const V *center, const V local[2]) {
  HostScene s;
  s.cam = *cam;
  s.light = h_normalise(*light);
  s.center = *center;
  s.lx = local[0];
  s.ly = local[1];
  s.normal = h_normalise(h_cross(s.lx, s.ly));
  s.W = sizes[0];
  s.H = sizes[1];
  return s;
}

static SceneDev scene_dev(const HostScene &s) {
  SceneDev d;
  d.cam = to_d3(s.cam);
  d.center = to_d3(s.center);
  d.lx = to_d3(s.lx);
  d.ly = to_d3(s.ly);
  d.normal = to_d3(s.normal);
  d.light = to_d3(s.light);
  d.nc = h_dot(s.normal, s.cam);
  d.d = h_dot(s.normal, s.center);
  d.lxx = h_dot(s.lx, s.lx);
  d.lyy = h_dot(s.ly, s.ly);
  d.width = (long long)s.W;
  d.height = (long long)s.H;
  /* single-precision projection constants (see project_f in kernels.cu) */
  const V cam = s.cam, n = s.normal, lx = s.lx, ly = s.ly;
  const double cm[3] = {cam.x, cam.y, cam.z}, nn[3] = {n.x, n.y, n.z}, ax[3] = {lx.x, lx.y, lx.z},
               ay[3] = {ly.x, ly.y, ly.z};
  d.f_cam_max = 0.f;
  d.f_n1 = d.f_lx1 = d.f_lxm = d.f_ly1 = d.f_lym = 0.f;
  for (int q = 0; q < 3; q++) {
    d.f_cam[q] = (float)cm[q];
    d.f_n[q] = (float)nn[q];
    d.f_lx[q] = (float)ax[q];
    d.f_ly[q] = (float)ay[q];
    d.f_cam_max = std::max(d.f_cam_max, (float)fabs(cm[q]));
    d.f_n1 += (float)fabs(nn[q]);
    d.f_lx1 += (float)fabs(ax[q]);
    d.f_ly1 += (float)fabs(ay[q]);
    d.f_lxm = std::max(d.f_lxm, (float)fabs(ax[q]));
    d.f_lym = std::max(d.f_lym, (float)fabs(ay[q]));
  }
  /* widen the norms by a few ulps so the bounds built from them stay upper bounds */
  d.f_n1 *= 1.0001f;
  d.f_lx1 *= 1.0001f;
  d.f_ly1 *= 1.0001f;
  d.f_lxm *= 1.0001f;
  d.f_lym *= 1.0001f;
  d.f_cam_max *= 1.0001f;
  const V cc = h_sub(s.cam, s.center);
  const double dq = d.d - d.nc;
  d.f_ax = (float)(h_dot(cc, lx) / d.lxx);
  d.f_bx = (float)(dq / d.lxx);
  d.f_ay = (float)(h_dot(cc, ly) / d.lyy);
  d.f_by = (float)(dq / d.lyy);
  d.f_dq = (float)dq;
  d.f_light[0] = (float)s.light.x;
  d.f_light[1] = (float)s.light.y;
  d.f_light[2] = (float)s.light.z;
  /* emission order is z-major: when the view points down z, high slices are near */
  d.z_descending = (s.center.z - s.cam.z) < 0. ? 1 : 0;
  return d;
}

/*
 * A bound on the FP64 rounding of one screen coordinate in project.c:26-66,
 * for points p with |p_i| <= pmax.  The projection forms ray = p - cam,
 * nr = n . ray, t = (d - nc) / nr, delta = cam + t ray - center and
 * x = delta . lx / lxx.  With u = 2^-53 and P = cam + t ray the screen point,
 * which lies between cam and p (0 < t < 1), so |P_i| <= max(|cam_i|, pmax):
 *   nr has relative error <= 4.01 u (sum |n_i| |ray_i|) / |nr|, and |nr| > |d - nc|
 *     because t < 1, so t has relative error <= u kappa - 2u with
 *     kappa = 4.01 sum |n_i| (pmax + |cam_i|) / |d - nc| + 3;
 *   t ray_i is off by <= u kappa (|P_i| + |cam_i|), the two sums by
 *     u |P_i| + u |delta_i| with |delta_i| <= |P_i| + |center_i|;
 *   the dot product with lx adds 3.01 u sum |delta_i lx_i|, the quotient u |x|,
 *     and |x| <= sum |delta_i lx_i| / lxx.
 * The common constants (d - nc, lxx) scale every point's x by the same factor
 * and change a difference of two points only relatively; that relative
 * error has to stay far below single precision for the bound to be used,
 * else the bound is infinite (every single-precision decision defers).
 */
static float projection_rounding(const SceneDev &sd, double pmax) {
  const double u = std::ldexp(1.0, -53);
  const double cam[3] = {sd.cam.x, sd.cam.y, sd.cam.z}, ctr[3] = {sd.center.x, sd.center.y, sd.center.z};
  const double n[3] = {sd.normal.x, sd.normal.y, sd.normal.z};
  const double lx[3] = {sd.lx.x, sd.lx.y, sd.lx.z}, ly[3] = {sd.ly.x, sd.ly.y, sd.ly.z};
  const double D = std::fabs(sd.d - sd.nc);
  double g = 0., rel = 0.;
  for (int i = 0; i < 3; i++) {
    g += std::fabs(n[i]) * (pmax + std::fabs(cam[i]));
    rel += 3. * std::fabs(n[i]) * (std::fabs(cam[i]) + std::fabs(ctr[i]));
  }
  rel = u * (3. + (std::fabs(sd.d) + std::fabs(sd.nc) + rel) / D);
  const double kappa = 4.01 * g / D + 3.;
  double sx = 0., sy = 0.;
  for (int i = 0; i < 3; i++) {
    const double P = std::max(std::fabs(cam[i]), pmax), dl = P + std::fabs(ctr[i]);
    const double term = kappa * (P + std::fabs(cam[i])) + P + 5.02 * dl;
    sx += std::fabs(lx[i]) * term;
    sy += std::fabs(ly[i]) * term;
  }
  const double e = 1.2 * u * std::max(sx / sd.lxx, sy / sd.lyy);
  if (!(D > 0.) || !(rel < 1e-9) || !std::isfinite(e) || e > 1e30) return INFINITY;
  return (float)(e * (1. + 1e-6)) + 1e-37f;
}

/* project.c:9-67 on the host (line end points) */
static int h_project(const HostScene &s, V p0, V *p1) {
  const V ray = h_sub(p0, s.cam);
  const double nc = h_dot(s.normal, s.cam);
  const double nr = h_dot(s.normal, ray);
  const double d = h_dot(s.normal, s.center);
  const double small = 1.e-8;
  if (-small < nr && nr < small) return 1;
  const double t = (d - nc) / nr;
  if (t <= 0. || 1. <= t) return 1;
  const V delta = {s.cam.x + t * ray.x - s.center.x, s.cam.y + t * ray.y - s.center.y,
                   s.cam.z + t * ray.z - s.center.z};
  p1->x = h_dot(delta, s.lx) / h_dot(s.lx, s.lx);
  p1->y = h_dot(delta, s.ly) / h_dot(s.ly, s.ly);
  p1->z = nr;
  return 0;
}

static long long h_key(double x) {
  long long b;
  memcpy(&b, &x, sizeof b);
  if ((b << 1) == 0) b = 0;
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}
static unsigned long long h_depth_key(double x) { return (unsigned long long)h_key(x) ^ 0x8000000000000000ULL; }

static unsigned h_fkey(float x) {
  unsigned u;
  memcpy(&u, &x, sizeof u);
  if ((u << 1) == 0) u = 0;
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* the least float strictly above the threshold: for a float v,
   threshold < (double)v  <=>  v >= that float (no such float: never above) */
static void set_float_threshold(FieldDev &F) {
  const double t = F.threshold;
  F.thr_f_ok = 0;
  F.thr_f_key = 0;
  if (std::isnan(t) || t == (double)INFINITY) return;
  /* beyond FLT_MAX only +inf is above; (float) of such t rounds to +inf or FLT_MAX */
  float f = (float)t;
  if (!((double)f > t)) f = nextafterf(f, INFINITY);
  F.thr_f_key = h_fkey(f);
  F.thr_f_ok = 1;
}

/* ---------------- marching-tetrahedra tables (triangulate.c) ---------------- */
/* cube corners of the six tetrahedra sharing the 0-7 diagonal */
static const int kTet[6][4] = {{0, 7, 3, 1}, {0, 7, 1, 5}, {0, 7, 5, 4}, {0, 7, 4, 6}, {0, 7, 6, 2}, {0, 7, 2, 3}};
/* triangles of each folded mask as (tail, head) pairs of tetrahedron vertices */
static const int kNtri[8] = {0, 1, 1, 2, 1, 2, 2, 1};
static const int kTriPairs[8][2][3][2] = {
    {{{0}}},
    {{{0, 1}, {0, 3}, {0, 2}}},
    {{{1, 0}, {1, 2}, {1, 3}}},
    {{{0, 2}, {1, 3}, {0, 3}}, {{0, 2}, {1, 2}, {1, 3}}},
    {{{2, 0}, {2, 3}, {2, 1}}},
    {{{2, 1}, {0, 3}, {2, 3}}, {{2, 1}, {0, 1}, {0, 3}}},
    {{{0, 2}, {2, 3}, {1, 3}}, {{0, 2}, {1, 3}, {0, 1}}},
    {{{3, 0}, {3, 2}, {3, 1}}},
};

/* cube-edge id of two corners: 0-3 x, 4-7 y, 8-11 z, 12-17 face diagonals, 18 body diagonal */
static int edge_id(int a, int b) {
  if (a > b) std::swap(a, b);
  switch (a ^ b) {
    case 1: return a >> 1;
    case 2: return 4 + ((a & 1) | ((a >> 2) << 1));
    case 4: return 8 + (a & 3);
    case 6: return 12 + (a & 1);
    case 5: return 14 + ((a >> 1) & 1);
    case 3: return 16 + (a >> 2);
    case 7: return 18;
    default: return 31;
  }
}

/* normal.c:78-158 in table form: (dk, dj, di, local edge id) per cube edge */
static const signed char kNb[19][4][4] = {
    {{-1, -1, 0, 3}, {-1, 0, 0, 2}, {0, -1, 0, 1}, {0, 0, 0, 0}},
    {{-1, 0, 0, 3}, {-1, 1, 0, 2}, {0, 0, 0, 1}, {0, 1, 0, 0}},
    {{0, -1, 0, 3}, {0, 0, 0, 2}, {1, -1, 0, 1}, {1, 0, 0, 0}},
    {{0, 0, 0, 3}, {0, 1, 0, 2}, {1, 0, 0, 1}, {1, 1, 0, 0}},
    {{-1, 0, -1, 7}, {-1, 0, 0, 6}, {0, 0, -1, 5}, {0, 0, 0, 4}},
    {{-1, 0, 0, 7}, {-1, 0, 1, 6}, {0, 0, 0, 5}, {0, 0, 1, 4}},
    {{0, 0, -1, 7}, {0, 0, 0, 6}, {1, 0, -1, 5}, {1, 0, 0, 4}},
    {{0, 0, 0, 7}, {0, 0, 1, 6}, {1, 0, 0, 5}, {1, 0, 1, 4}},
    {{0, -1, -1, 11}, {0, -1, 0, 10}, {0, 0, -1, 9}, {0, 0, 0, 8}},
    {{0, -1, 0, 11}, {0, -1, 1, 10}, {0, 0, 0, 9}, {0, 0, 1, 8}},
    {{0, 0, -1, 11}, {0, 0, 0, 10}, {0, 1, -1, 9}, {0, 1, 0, 8}},
    {{0, 0, 0, 11}, {0, 0, 1, 10}, {0, 1, 0, 9}, {0, 1, 1, 8}},
    {{0, 0, -1, 13}, {0, 0, 0, 12}},
    {{0, 0, 0, 13}, {0, 0, 1, 12}},
    {{0, -1, 0, 15}, {0, 0, 0, 14}},
    {{0, 0, 0, 15}, {0, 1, 0, 14}},
    {{-1, 0, 0, 17}, {0, 0, 0, 16}},
    {{0, 0, 0, 17}, {1, 0, 0, 16}},
    {{0, 0, 0, 18}},
};
static const unsigned char kNbCount[19] = {4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 2, 2, 2, 2, 2, 2, 1};

static void build_tables(std::vector<unsigned long long> &lut, unsigned char count[256]) {
  lut.assign(kLutEntries, 0ULL);
  for (int code = 0; code < 256; code++) {
    int n = 0;
    for (int t = 0; t < 6; t++) {
      int mask = 0;
      for (int m = 0; m < 4; m++) mask |= ((code >> kTet[t][m]) & 1) << m;
      const bool rev = mask >= 8;
      if (rev) mask = 15 - mask;
      for (int s = 0; s < kNtri[mask]; s++) {
        unsigned long long e = 0;
        for (int q = 0; q < 3; q++) {
          const int src = rev ? 2 - q : q;
          const int a = kTet[t][kTriPairs[mask][s][src][0]];
          const int b = kTet[t][kTriPairs[mask][s][src][1]];
          e |= (unsigned long long)a << (6 * q);
          e |= (unsigned long long)b << (6 * q + 3);
          e |= (unsigned long long)edge_id(a, b) << (18 + 5 * q);
        }
        lut[code * 12 + n++] = e;
      }
    }
    count[code] = (unsigned char)n;
  }
}

/* ---------------- device context ---------------- */
/* device bytes held by every library buffer of the process */
static std::atomic<unsigned long long> g_device_bytes{0};

/*
 * Device buffers come from one stream-ordered memory pool per device that
 * keeps freed blocks (release threshold = all), so a buffer that grows while
 * other contexts render costs no device-wide synchronisation, and a new
 * context reuses the blocks of released ones.
 */
static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[64];

static cudaMemPool_t device_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    unsigned long long keep = ~0ULL;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pool[dev] = pool;
  }
  return g_pool[dev];
}

/*
 * Device-memory accounting of one context of a server: every growth of one
 * of the context's buffers is charged before it is allocated (charge may
 * wait until the server's HBM budget has room) and every release is
 * credited.  Contexts outside a server have none.
 */
/* set when a buffer had to grow while its stream was being captured */
static thread_local bool t_capture_needs_growth = false;

struct MemHook {
  virtual int charge(size_t bytes) = 0;
  virtual void credit(size_t bytes) = 0;
  virtual ~MemHook() {}
};

struct Buf {
  void *p = nullptr;
  size_t cap = 0;
  MemHook *hook = nullptr;
  /* grow to at least `bytes`; the old contents are not kept.  Allocation and
     release are ordered on `st`, the stream every use of the buffer is on
     (or whose previous uses have completed) */
  int ensure(size_t bytes, cudaStream_t st) {
    if (bytes <= cap) return 0;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (st && cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      /* a frame being recorded into a graph must not allocate: the caller
         abandons the recording and renders the frame without it */
      t_capture_needs_growth = true;
      return 1;
    }
    release(st);
    const size_t want = bytes + bytes / 4 + 256;
    if (hook && hook->charge(want)) return 1;
    cudaMemPool_t pool = device_pool();
    if (!pool || cudaMallocFromPoolAsync(&p, want, pool, st) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      if (hook) hook->credit(want);
      log_error("device allocation of %zu bytes failed", want);
      return 1;
    }
    cap = want;
    g_device_bytes += want;
    return 0;
  }
  void release(cudaStream_t st) {
    if (p) {
      cudaFreeAsync(p, st);
      g_device_bytes -= cap;
      if (hook) hook->credit(cap);
    }
    p = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return 0;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      log_error("pinned host allocation of %zu bytes failed", bytes);
      return 1;
    }
    cap = bytes;
    return 0;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

struct Ctx {
  int device = -1;
  bool ready = false;
  cudaStream_t own_stream = nullptr;
  Buf lut, counts, scratch, dbg, field, nodes, canvas, rgb;
  Buf zlo, checks, winfo, shade_check;
  /* the per-slab arrays of one contour object's pass.  Unsynchronised frames
     run the objects of a slab on two lanes (the frame's stream and
     lane_stream), each with its own arrays; the passes of different objects
     meet only in the z-buffer, the depth floors and the winner weights,
     whose updates are order-independent maxima and tagged stores */
  struct Lane {
    Buf offsets, voffsets, tile_state, tri_cell, tri, verts, cand, tiny;
    /* one object's shading: its won pixels, those left to FP64, and the
       FP64 pass's neighbour lists (unsynchronised frames shade the objects
       of a field on both lanes; the passes meet only in the colour bits of
       disjoint pixels) */
    Buf win, amb, nb_ent, nb_wn, nb_span;
    /* the vertex offsets of a slab of n cells (in voffsets) */
    VOffDev voff(long long n) const { return voff_layout(voffsets.p, n); }
  };
  Lane lanes[2];
  cudaStream_t lane_stream = nullptr;
  cudaEvent_t ev_lane_fork = nullptr, ev_lane_join = nullptr;
  unsigned long long epoch = 0; /* frame counter for the winner-weight tags (1 .. 2^24 - 1) */
  Buf consts;                  /* the frame constants (pixel centres, grid blocks, line segments) */
  HostBuf h_consts;            /* their pinned staging block */
  cudaEvent_t ev_staged = nullptr; /* the staging block may be rewritten once this completed */
  bool filter_check = false;
  HostBuf h_small, h_rgb, h_slots;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evs[11] = {};
  bool stage_timing = false;
  unsigned long long slab_cells = kMaxSlabCells; /* the most the scan's 32-bit packed sums allow */
  contour3d_gb300_stats_t stats = {};
  const void *field_src = nullptr; /* host array currently in `field` (valid within one call) */
  size_t field_bytes = 0;
  uint64_t stats_h2d = 0;
  /* frames without host synchronisation: buffers sized from the largest
     counts seen so far (caps), the counts of every pass kept in a device
     status block read once at the frame's end; a frame whose counts exceed
     the sizes is rendered again with synchronisation, which learns them */
  bool async_enabled = true;
  bool frame_async = false;     /* the current frame runs without host synchronisation */
  struct Caps {
    unsigned long long T = 0, V = 0, cand = 0, tiny = 0, ent = 0;
  } caps;
  bool caps_known = false;      /* a frame completed with synchronisation on this context */
  Buf status;                   /* device status block of the current frame */
  HostBuf h_status;             /* its pinned copy */
  int status_next = 0, status_obj_next = 0;
  unsigned long long async_cand_cap = 0, async_tiny_cap = 0, async_ent_cap = 0;
  std::vector<char> async_obj_fp32; /* per object status record: the FP32 shading pass ran */
  /* the last unsynchronised device frame as a CUDA graph: recorded the second
     time a frame with the same description (frame_key) comes, launched
     instead of the individual calls from the third time on */
  bool graphs_enabled = true;
  bool capturing = false;
  uint64_t graph_key = 0;
  bool graph_key_seen = false;
  cudaGraphExec_t graph_exec = nullptr;
  struct GraphFrame {
    int status_next = 0, status_obj_next = 0;
    unsigned long long cand_cap = 0, tiny_cap = 0, ent_cap = 0;
    std::vector<char> obj_fp32;
    uint64_t kernel_launches = 0, slabs = 0, cells = 0;
  } graph_frame;
  cudaStream_t copy_stream = nullptr;  /* host field uploads, overlapped with the slabs */
  cudaEvent_t ev_field = nullptr;      /* the field buffer may be overwritten once this completed */
  std::vector<cudaEvent_t> chunk_ev;   /* upload chunk s has arrived */
  size_t chunks_used = 0;              /* of them, this frame's */
  /* C3D_TRACE=1: timing events of the frame's passes, with their labels */
  std::vector<cudaEvent_t> trace_ev;
  std::vector<std::string> trace_label;
  size_t trace_used = 0;
};

static Ctx g_ctx;
static std::mutex g_mu;
/* the unsynchronised-frame and graph settings new contexts (server slots)
   start with: off, so worker contexts synchronise after every slab pass
   (see contour3d_gb300_set_async) */
static std::atomic<bool> g_async_default{false}, g_graphs_default{false};

static int ctx_init(Ctx &c) {
  int dev = 0;
  C3D_CUDA(cudaGetDevice(&dev));
  if (c.ready && c.device == dev) return 0;
  if (c.ready) {
    log_error("the library context is bound to device %d; call contour3d_gb300_release() first", c.device);
    return 1;
  }
  if (&c != &g_ctx) {
    c.async_enabled = g_async_default.load();
    c.graphs_enabled = g_graphs_default.load();
  }
  C3D_CUDA(cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking));
  C3D_CUDA(cudaEventCreate(&c.ev0));
  C3D_CUDA(cudaEventCreate(&c.ev1));
  C3D_CUDA(cudaEventCreateWithFlags(&c.ev_staged, cudaEventDisableTiming));
  C3D_CUDA(cudaEventRecord(c.ev_staged, c.own_stream));
  for (auto &e : c.evs) C3D_CUDA(cudaEventCreate(&e));
  C3D_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
  C3D_CUDA(cudaEventCreateWithFlags(&c.ev_field, cudaEventDisableTiming));
  C3D_CUDA(cudaStreamCreateWithFlags(&c.lane_stream, cudaStreamNonBlocking));
  C3D_CUDA(cudaEventCreateWithFlags(&c.ev_lane_fork, cudaEventDisableTiming));
  C3D_CUDA(cudaEventCreateWithFlags(&c.ev_lane_join, cudaEventDisableTiming));
  std::vector<unsigned long long> lut;
  unsigned char count[256];
  build_tables(lut, count);
  {
    /* constant tables: once per device for every context of the process */
    static std::mutex tables_mu;
    static bool uploaded[64] = {false};
    std::lock_guard<std::mutex> lk(tables_mu);
    if (dev < 0 || dev >= 64) return 1;
    if (!uploaded[dev]) {
      /* per code and cube edge, the ranks of the triangles with a vertex on it */
      std::vector<unsigned short> edge_tris(256 * 19, 0);
      for (int code = 0; code < 256; code++)
        for (int r = 0; r < count[code]; r++) {
          const unsigned long long e = lut[code * 12 + r];
          for (int q = 0; q < 3; q++) {
            const unsigned id = (unsigned)((e >> (18 + 5 * q)) & 31);
            if (id < 19) edge_tris[code * 19 + id] |= (unsigned short)(1u << r);
          }
        }
      if (upload_tables(count, kNb, kNbCount, edge_tris.data())) {
        log_error("constant table upload failed");
        return 1;
      }
      uploaded[dev] = true;
    }
  }
  if (c.lut.ensure(sizeof(unsigned long long) * kLutEntries, c.own_stream)) return 1;
  C3D_CUDA(cudaMemcpyAsync(c.lut.p, lut.data(), sizeof(unsigned long long) * kLutEntries, cudaMemcpyHostToDevice,
                           c.own_stream));
  C3D_CUDA(cudaStreamSynchronize(c.own_stream));
  if (c.h_small.ensure(256)) return 1;
  c.device = dev;
  c.ready = true;
  return 0;
}

/* ---------------- identity converters ---------------- */
typedef V (*conv_fn)(const V);
static conv_fn g_identity[16];
static int g_nidentity = 0;

static bool is_identity(conv_fn f);

/* ---------------- frame description ---------------- */
struct ContourIn {
  const void *data = nullptr;  /* field: host or device */
  bool on_device = false;
  bool f32 = false;
  size_t sz[3] = {0, 0, 0};    /* extended block sizes */
  size_t off[3] = {0, 0, 0};   /* global offset of the block */
  const double *grid[3] = {nullptr, nullptr, nullptr}; /* host node coordinates of the block */
  conv_fn converter = nullptr;
  double threshold = 0.;
  contour3d_color_t color = {0, 0, 0};
  /* the object's cell codes of the whole field, already classified (the
     batched form classifies every frame in one launch), or null */
  unsigned char *pre_codes = nullptr;
};

struct FrameIn {
  HostScene scene;
  contour3d_color_t bg;
  std::vector<ContourIn> contours;
  const contour3d_line_obj_t *lines = nullptr;
  size_t nlines = 0;
  cudaStream_t stream = nullptr;
};

/* host sink of rendered-triangle records (contour3d_gb300_debug_triangles) */
struct TriRecord {
  double vertices[9];
  double vertex_normals[9];
  double face_normal[3];
  double area;
  int64_t cell[3];
  int64_t edge_ids[3];
};
static_assert(sizeof(TriRecord) == 224, "triangle record is 224 bytes");

struct DebugSink {
  TriRecord *out = nullptr;
  long capacity = 0;
  long count = 0;
  long triangulated = 0;
  bool triangulated_only = false; /* only count, do not render */
};

struct FrameOut {
  uint8_t *rgb_host = nullptr;  /* ppm body */
  bool rgb_pinned = false;      /* leave the ppm body in the context's pinned buffer h_rgb */
  uint8_t *rgb_dev = nullptr;   /* ppm body on the device */
  double *depth_host = nullptr; /* canvas order */
  PixelRec *pixels_host = nullptr; /* canvas order, for the multi-rank reduction */
  DebugSink *sink = nullptr;
};

/* words of the 64-byte check buffer: 0-5 self-check counters, then the
   z-buffer error flags, the overflow flags (kOvf*) and, in frames without
   host synchronisation, the classification's error flags */
static const int kZbufErrWord = 8;
static const int kOvfWord = 9;
static const int kClsErrWord = 10;

/* a field group's block of the frame constants: node coordinates (doubles),
   their float roundings, the float node spacings, and the largest |coordinate| */
struct GroupGrid {
  const double *dev = nullptr;
  double coord_max = 0.;
};

static size_t grid_block_bytes(const ContourIn &ci) {
  const size_t ng = ci.sz[0] + ci.sz[1] + ci.sz[2];
  return sizeof(double) * ng + sizeof(float) * (2 * ng - 3);
}

/* the grid block of one field (x, y, z nodes in turn) into hg; returns the largest |coordinate| */
static double fill_grid_block(const ContourIn &ci, double *hg) {
  const long long n3[3] = {(long long)ci.sz[0], (long long)ci.sz[1], (long long)ci.sz[2]};
  const size_t ng = (size_t)(n3[0] + n3[1] + n3[2]);
  float *hgf = reinterpret_cast<float *>(hg + ng);
  float *hgd = hgf + ng;
  memcpy(hg, ci.grid[0], sizeof(double) * n3[0]);
  memcpy(hg + n3[0], ci.grid[1], sizeof(double) * n3[1]);
  memcpy(hg + n3[0] + n3[1], ci.grid[2], sizeof(double) * n3[2]);
  for (size_t q = 0; q < ng; q++) hgf[q] = (float)hg[q];
  double coord_max = 0.;
  size_t at = 0, out = 0;
  for (int d = 0; d < 3; d++) {
    for (long long q = 0; q + 1 < n3[d]; q++) hgd[out++] = (float)(hg[at + q + 1] - hg[at + q]);
    for (long long q = 0; q < n3[d]; q++) coord_max = std::max(coord_max, std::fabs(hg[at + q]));
    at += (size_t)n3[d];
  }
  return coord_max;
}

/* line.c:121-170 on the host: every segment's end points projected to pixel
   units (render.c's convention); 1 on a line object with fewer than two items */
static int build_line_segs(const FrameIn &f, std::vector<LineSegDev> &segs) {
  const HostScene &s = f.scene;
  for (size_t n = 0; n < f.nlines; n++) {
    const contour3d_line_obj_t *l = f.lines + n;
    const size_t np = l->nitems;
    if (np < 2) {
      log_error("give more than two points to draw a line, received %zu", np);
      log_error("line processing failed");
      return 1;
    }
    const conv_fn conv = l->converter ? l->converter : contour3d_gb300_identity;
    const V *heads = l->edges + 0, *tails = l->edges + 1;
    const V deltas = h_mul(1. / (np - 1), h_sub(*tails, *heads));
    const unsigned rgb = ((unsigned)l->color.r << 16) | ((unsigned)l->color.g << 8) | l->color.b;
    for (size_t q = 0; q < np - 1; q++) {
      const V a = h_add(*heads, h_mul(q + 0, deltas));
      const V b = h_add(*heads, h_mul(q + 1, deltas));
      const V pa = conv(a), pb = conv(b);
      V p0 = {0., 0., 0.}, p1 = {0., 0., 0.};
      LineSegDev sg = {};
      sg.valid = !h_project(s, pa, &p0) && !h_project(s, pb, &p1);
      if (sg.valid) {
        sg.p0x = (0.5 + p0.x) * s.W;
        sg.p0y = (0.5 + p0.y) * s.H;
        sg.p1x = (0.5 + p1.x) * s.W;
        sg.p1y = (0.5 + p1.y) * s.H;
        sg.p0z = p0.z;
        sg.p1z = p1.z;
      }
      sg.width = l->width;
      sg.rgb = rgb;
      segs.push_back(sg);
    }
  }
  return 0;
}

/*
 * The frame's constant inputs, staged in one pinned block and copied to the
 * device with one copy: the pixel centres (render.c:100-104) in double and
 * float, every field group's grid block, and the line segments.  Each region
 * starts on 256 bytes.
 */
struct FrameConsts {
  const double *xy = nullptr;
  const float *xyf = nullptr;
  std::vector<GroupGrid> groups;
  const LineSegDev *segs = nullptr;
  int nseg = 0;
};

static int stage_frame_consts(Ctx &c, const FrameIn &f, const std::vector<std::pair<size_t, size_t>> &groups,
                              const std::vector<LineSegDev> &segs, FrameConsts &fc) {
  const size_t W = f.scene.W, H = f.scene.H;
  size_t at = 0;
  auto take = [&](size_t bytes) {
    const size_t a = at;
    at = (at + bytes + 255) & ~(size_t)255;
    return a;
  };
  const size_t o_xy = take(sizeof(double) * (W + H)), o_xyf = take(sizeof(float) * (W + H));
  std::vector<size_t> o_grid(groups.size());
  for (size_t g = 0; g < groups.size(); g++) o_grid[g] = take(grid_block_bytes(f.contours[groups[g].first]));
  const size_t o_segs = take(sizeof(LineSegDev) * segs.size());
  /* the previous frame's copy from the staging block must have left it (a
     frame being recorded synchronised before the recording began) */
  if (!c.capturing) C3D_CUDA(cudaEventSynchronize(c.ev_staged));
  if (c.h_consts.ensure(at) || c.consts.ensure(at, f.stream)) return 1;
  char *h = c.h_consts.as<char>();
  char *d = c.consts.as<char>();
  double *xy = reinterpret_cast<double *>(h + o_xy);
  float *xyf = reinterpret_cast<float *>(h + o_xyf);
  for (size_t i = 0; i < W; i++) xy[i] = 1. * (i + 0.5) / W - 0.5;
  for (size_t j = 0; j < H; j++) xy[W + j] = 1. * (j + 0.5) / H - 0.5;
  for (size_t q = 0; q < W + H; q++) xyf[q] = (float)xy[q];
  fc.xy = reinterpret_cast<const double *>(d + o_xy);
  fc.xyf = reinterpret_cast<const float *>(d + o_xyf);
  fc.groups.assign(groups.size(), GroupGrid());
  for (size_t g = 0; g < groups.size(); g++) {
    fc.groups[g].coord_max = fill_grid_block(f.contours[groups[g].first], reinterpret_cast<double *>(h + o_grid[g]));
    fc.groups[g].dev = reinterpret_cast<const double *>(d + o_grid[g]);
  }
  if (!segs.empty()) memcpy(h + o_segs, segs.data(), sizeof(LineSegDev) * segs.size());
  fc.segs = reinterpret_cast<const LineSegDev *>(d + o_segs);
  fc.nseg = (int)segs.size();
  C3D_CUDA(cudaMemcpyAsync(d, h, at, cudaMemcpyHostToDevice, f.stream));
  if (!c.capturing) C3D_CUDA(cudaEventRecord(c.ev_staged, f.stream));
  return 0;
}

/* the status block of a frame rendered without host synchronisation, in
   64-bit words: kStatusHead words, then per (slab, object) pass kSlabRec
   words (triangles, vertices, the kCounters raster counters), then per
   object three words (won pixels, ambiguous pixels, neighbour entries) */
static const int kStatusHead = 2;
static const int kStatusSlabs = 1024;
static const int kStatusObjs = 256;

/* device counters of one slab's raster passes: candidates, tiny triangles,
   cover and sliver triangles, the cover list's entries (with the empty ends
   of k_emit's chunks), surviving candidates, the sliver list's entries, two
   unused */
static const int kCounters = 9;
static const int kSlabRec = 2 + kCounters;
static const size_t kStatusWords = kStatusHead + (size_t)kSlabRec * kStatusSlabs + 3 * (size_t)kStatusObjs;

/* bytes per triangle of the slab arrays (see TriDev): inspection keeps
   weighted normals, records and flags; the render path the raster records */
static const size_t kTriBytes = 3 * sizeof(double) + 48 + sizeof(unsigned);
static const size_t kRecBytes = 48;
static size_t tri_bytes(bool inspect) { return inspect ? kTriBytes : kRecBytes; }
/* doubles per triangle of the inspection arrays: vertices, vertex normals, face normal, area */
static const size_t kDbgDoubles = 22;

static TriDev tri_layout(void *base, size_t cap, double *dbg, bool inspect) {
  TriDev t;
  double *d = static_cast<double *>(base);
  for (int q = 0; q < 3; q++) t.wn[q] = inspect ? d + q * cap : nullptr;
  t.rec = reinterpret_cast<float4 *>(inspect ? d + 3 * cap : d);
  t.meta = inspect ? reinterpret_cast<unsigned *>(t.rec + 3 * cap) : nullptr;
  for (int q = 0; q < 9; q++) t.vert[q] = dbg ? dbg + q * cap : nullptr;
  for (int q = 0; q < 9; q++) t.vn[q] = dbg ? dbg + (9 + q) * cap : nullptr;
  t.dbg_fn = dbg ? dbg + 18 * cap : nullptr;
  t.dbg_area = dbg ? dbg + 21 * cap : nullptr;
  return t;
}

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

/*
 * The upload of one host field in z-chunks on the context's copy stream.  A
 * copy from pageable memory returns only once the driver has staged it, so a
 * helper thread issues the chunks in the order the slabs need them and
 * records one event per chunk; the slab loop waits for chunk s to be issued,
 * then makes its stream wait on the chunk's event, and the slabs compute
 * while later chunks are still crossing the host link.
 */
struct FieldUpload {
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  int issued = 0;
  bool failed = false;
  char what[160] = {0};
  ~FieldUpload() {
    if (th.joinable()) th.join();
  }
  void start(int device, cudaStream_t cs, std::vector<cudaEvent_t> evs, char *dst, const char *src,
             std::vector<std::pair<size_t, size_t>> ranges) {
    th = std::thread([this, device, cs, evs, dst, src, ranges]() {
      cudaError_t e = cudaSetDevice(device);
      for (size_t q = 0; q < ranges.size(); q++) {
        const size_t a = ranges[q].first, b = ranges[q].second;
        if (e == cudaSuccess && b > a) e = cudaMemcpyAsync(dst + a, src + a, b - a, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaEventRecord(evs[q], cs);
        {
          std::lock_guard<std::mutex> lk(mu);
          if (e != cudaSuccess) {
            failed = true;
            snprintf(what, sizeof what, "field upload chunk %zu: %s", q, cudaGetErrorString(e));
          } else {
            issued = (int)q + 1;
          }
        }
        cv.notify_all();
        if (e != cudaSuccess) return;
      }
    });
  }
  /* chunk s is issued (its event recorded); false when the upload failed */
  bool wait(int s) {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return issued > s || failed; });
    return !failed || issued > s;
  }
};

/* fields at least this large are uploaded in chunks overlapped with the slabs */
constexpr size_t kPipelineBytes = 64ull << 20;
constexpr long long kPipelineMinSlices = 16;
/* the upload model (GB300, host field in pinned memory; set with
   contour3d_gb300_set_upload_model): the link moves about 211 GB/s however
   the copy is issued (one or four copy streams, or SMs reading mapped host
   memory); a slab pass costs about 18.9 ps per cell and object (a 512^3 f64
   field, two objects on two lanes, 1920 x 1080) plus about 0.04 ms per
   object and slab of fixed cost (the kernels' ramp-up and tails, the slab's
   halo slices) */
struct UploadModel {
  double link_bytes_per_s = 211e9;
  double slab_s_per_cell = 18.9e-12;
  double slab_fixed_s = 0.04e-3;
};
static std::mutex g_upload_mu;
static UploadModel g_upload_model;
static UploadModel upload_model() {
  std::lock_guard<std::mutex> lk(g_upload_mu);
  return g_upload_model;
}
constexpr int kMaxUploadSlabs = 24;

/*
 * Slab sizes (rendered slices, in visiting order) for L slices of a field
 * that arrives while it is processed.  In units of the whole copy's time:
 * chunk s has landed at C_s (its slices and every earlier chunk's), and slab
 * s runs from max(E_{s-1}, C_s) for r per slice's copy time plus o.  A plan
 * starts with a first slab of L / m slices and makes each next slab as large
 * as still lands before the slab before it ends, so that the compute does
 * not wait; the plan with the earliest modelled end over m = 2 .. 24 is
 * taken.  An empty plan: one slab after the whole copy is modelled faster.
 */
static std::vector<long long> upload_plan(long long L, long long max_slab, double r, double o) {
  std::vector<long long> best;
  double best_end = 1.0 + r + o; /* the whole copy, then one pass */
  for (int m = 2; m <= kMaxUploadSlabs; m++) {
    const long long first = std::max(1LL, L / m);
    if (first > max_slab) continue;
    std::vector<long long> plan{first};
    long long S = first;
    double E = (double)first / (double)L * (1.0 + r) + o;
    bool ok = true;
    while (S < L) {
      if ((int)plan.size() >= kMaxUploadSlabs) {
        ok = false;
        break;
      }
      long long z = (long long)(E * (double)L) - S; /* lands before slab s - 1 ends */
      z = std::max(z, std::max(1LL, first / 2));
      z = std::min(std::min(z, max_slab), L - S);
      S += z;
      E = std::max(E, (double)S / (double)L) + r * (double)z / (double)L + o;
      plan.push_back(z);
    }
    if (ok && E < best_end) {
      best_end = E;
      best = plan;
    }
  }
  return best;
}

/* objects that read one field with one geometry: they share the upload, the
   node tables and the slabs */
static bool same_field(const ContourIn &a, const ContourIn &b) {
  return a.data == b.data && a.on_device == b.on_device && a.f32 == b.f32 && a.converter == b.converter &&
         a.sz[0] == b.sz[0] && a.sz[1] == b.sz[1] && a.sz[2] == b.sz[2] && a.grid[0] == b.grid[0] &&
         a.grid[1] == b.grid[1] && a.grid[2] == b.grid[2];
}

/*
 * A group of contour objects of one field (same_field) through all of the
 * field's slabs.  The objects take their slabs in turn (slab 0 of every
 * object, then slab 1, ...), so that while a host field is still arriving
 * every object works on the slices that are already there; the result does
 * not depend on this order (fragments carry their drawing order).
 */
/* C3D_TRACE=1 in the environment: every frame prints to stderr when each
   upload chunk landed and each slab pass and shading pass ended, relative
   to the frame's start (a debugging aid; off by default) */
static bool trace_on() {
  static const bool on = [] {
    const char *v = getenv("C3D_TRACE");
    return v && v[0] == '1';
  }();
  return on;
}

static void trace_mark(Ctx &c, cudaStream_t st, const std::string &label) {
  if (!trace_on() || c.capturing) return;
  if (c.trace_used == c.trace_ev.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    c.trace_ev.push_back(e);
    c.trace_label.emplace_back();
  }
  c.trace_label[c.trace_used] = label;
  if (cudaEventRecord(c.trace_ev[c.trace_used], st) == cudaSuccess) c.trace_used++;
  else cudaGetLastError();
}

/* after the frame's final synchronisation */
static void trace_print(Ctx &c) {
  if (!trace_on()) return;
  for (size_t q = 0; q < c.chunks_used && q < c.chunk_ev.size(); q++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c.ev0, c.chunk_ev[q]) == cudaSuccess)
      fprintf(stderr, "[c3d trace] %8.3f ms  upload chunk %zu landed\n", ms, q);
    else
      cudaGetLastError();
  }
  for (size_t q = 0; q < c.trace_used; q++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c.ev0, c.trace_ev[q]) == cudaSuccess)
      fprintf(stderr, "[c3d trace] %8.3f ms  %s\n", ms, c.trace_label[q].c_str());
    else
      cudaGetLastError();
  }
  c.trace_used = 0;
  c.chunks_used = 0;
}

static int render_contour(Ctx &c, const FrameIn &f, const SceneDev &sd, const ContourIn *objs, size_t nobj,
                          unsigned long long &order_base, const RasterDev &R, DebugSink *sink,
                          const GroupGrid &gg) {
  const ContourIn &ci = objs[0];
  cudaStream_t st = f.stream;
  const long long nx = (long long)ci.sz[0], ny = (long long)ci.sz[1], nz = (long long)ci.sz[2];
  if (nx < 2 || ny < 2 || nz < 2) return 0;
  const long long ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
  const size_t elem = ci.f32 ? 4 : 8;
  const size_t nnodes = (size_t)(nx * ny * nz);
  /* field */
  const void *dfield = ci.data;
  bool pipelined = false; /* the field arrives in chunks while the slabs run */
  if (!ci.on_device) {
    /* objects of one call that share a host array (the reference's example
       draws two levels of one field) upload it once */
    if (!(c.field_src == ci.data && c.field_bytes == nnodes * elem && c.field.p)) {
      if (c.field.ensure(nnodes * elem, st)) return 1;
      pipelined = sink == nullptr && nnodes * elem >= kPipelineBytes && ncz >= kPipelineMinSlices;
      if (!pipelined)
        C3D_CUDA(cudaMemcpyAsync(c.field.p, ci.data, nnodes * elem, cudaMemcpyHostToDevice, st));
      c.field_src = ci.data;
      c.field_bytes = nnodes * elem;
      c.stats_h2d += nnodes * elem;
    }
    dfield = c.field.p;
  }
  /* node coordinates, their float roundings and spacings: this group's
     block of the frame constants */
  const size_t ng = (size_t)(nx + ny + nz);
  const double *g = gg.dev;
  const float *gf = reinterpret_cast<const float *>(g + ng);
  const float *gd = gf + ng;
  const double coord_max = gg.coord_max;
  const double *dnodes = nullptr;
  std::vector<double> nodes;
  if (!is_identity(ci.converter)) {
    /* tabulate the converter once per node (triangulate.c:165-170 calls it per tetrahedron corner) */
    nodes.resize(3 * nnodes);
    size_t q = 0;
    for (long long k = 0; k < nz; k++)
      for (long long j = 0; j < ny; j++)
        for (long long i = 0; i < nx; i++) {
          const V p = ci.converter(V{ci.grid[0][i], ci.grid[1][j], ci.grid[2][k]});
          nodes[q++] = p.x;
          nodes[q++] = p.y;
          nodes[q++] = p.z;
        }
    if (c.nodes.ensure(sizeof(double) * 3 * nnodes, st)) return 1;
    C3D_CUDA(cudaMemcpyAsync(c.nodes.p, nodes.data(), sizeof(double) * 3 * nnodes, cudaMemcpyHostToDevice, st));
    dnodes = c.nodes.as<double>();
  }
  FieldDev F;
  F.data = dfield;
  F.codes = nullptr;
  F.is_f32 = ci.f32 ? 1 : 0;
  F.nx = nx;
  F.ny = ny;
  F.nz = nz;
  F.gx = g;
  F.gy = g + nx;
  F.gz = g + nx + ny;
  F.gxf = gf;
  F.gyf = gf + nx;
  F.gzf = gf + nx + ny;
  F.nodes = dnodes;
  F.div_cx = make_fast_div((unsigned)(nx - 1));
  F.div_cy = make_fast_div((unsigned)(ny - 1));
  /* single-precision shading needs Cartesian nodes and finite coordinates */
  const bool fp32_shading = dnodes == nullptr && std::isfinite(coord_max) && coord_max < 1e30;
  F.dgx = fp32_shading ? gd : nullptr;
  F.dgy = fp32_shading ? gd + (nx - 1) : nullptr;
  F.dgz = fp32_shading ? gd + (nx - 1) + (ny - 1) : nullptr;
  /* the reference's vertex p0 + f (p1 - p0) and its differences carry FP64
     rounding of a few 2^-53 |coordinate|: 1e-15 covers it */
  F.coord_eps = (float)(1e-15 * coord_max) + 1e-37f;
  double pos_max = coord_max;
  for (const double v : nodes) pos_max = std::max(pos_max, std::fabs(v));
  F.proj_eps = projection_rounding(sd, pos_max);
  std::vector<FieldDev> Fo(nobj, F);
  for (size_t q = 0; q < nobj; q++) {
    Fo[q].threshold = objs[q].threshold;
    Fo[q].thr_key = h_key(objs[q].threshold);
    Fo[q].thr_nan = std::isnan(objs[q].threshold) ? 1 : 0;
    set_float_threshold(Fo[q]);
  }
  c.stats.cells += (uint64_t)(ncx * ncy * ncz) * nobj;

  /* rendered cell slices are [1, ncz - 2] (contour/main.c:49-112); each slab
     also classifies and scans the slice above it, whose cells own vertices of
     the slab's top triangles, and the slice below it, whose codes the
     per-object shading reads when one slab covers the field (the neighbour
     triangles of slice k lie in slices k - 1 .. k + 1); the scan and vertex
     work on the slice below is not used.
     Slabs are visited front to back (the z-buffer result does not depend on
     the order: fragments carry their position in the reference's drawing
     sequence), except for inspection, which reports triangles in order. */
  const long long per_slice = ncx * ncy;
  const unsigned long long slab_cells = std::min<unsigned long long>(c.slab_cells, (unsigned long long)kMaxSlabCells);
  long long slab_slices = (long long)(slab_cells / (unsigned long long)per_slice) - 2;
  if (slab_slices < 1) slab_slices = 1;
  if (3 * per_slice > kMaxSlabCells) {
    log_error("z-slices of %lld cells are too large (a slab of three slices must hold at most %lld cells)",
              per_slice, kMaxSlabCells);
    return 1;
  }
  const bool want_all = sink != nullptr;
  const bool async = c.frame_async && !sink;
  const long long kr0 = want_all ? 0 : 1, kr1 = want_all ? ncz : ncz - 1;
  /* the slabs [k0, k1) of rendered slices, in the order they are visited */
  std::vector<std::pair<long long, long long>> slabs;
  const bool descending = sd.z_descending && !want_all;
  if (pipelined) {
    /* while the field arrives: the modelled plan (upload_plan) */
    const UploadModel um = upload_model();
    const double copy_s = (double)(nnodes * elem) / um.link_bytes_per_s;
    const double r = um.slab_s_per_cell * (double)(per_slice * ncz) * (double)nobj / copy_s;
    const double o = um.slab_fixed_s * (double)nobj / copy_s;
    const std::vector<long long> sizes = upload_plan(kr1 - kr0, slab_slices, r, o);
    if (sizes.empty()) {
      pipelined = false;
      C3D_CUDA(cudaMemcpyAsync(c.field.p, ci.data, nnodes * elem, cudaMemcpyHostToDevice, st));
    }
    long long k = descending ? kr1 : kr0;
    for (const long long z : sizes) {
      slabs.push_back(descending ? std::make_pair(k - z, k) : std::make_pair(k, k + z));
      k += descending ? -z : z;
    }
  }
  if (slabs.empty()) {
    for (long long k0 = kr0; k0 < kr1; k0 += slab_slices) slabs.push_back({k0, std::min(k0 + slab_slices, kr1)});
    if (descending) std::reverse(slabs.begin(), slabs.end());
  }
  FieldUpload up;
  if (pipelined) {
    /* chunk s: the node slices slab s reads that earlier slabs did not; the
       first chunk also takes the slices below (above) the first slab and the
       last one those beyond the last slab */
    const size_t slice = (size_t)(nx * ny) * elem;
    std::vector<std::pair<size_t, size_t>> ranges;
    long long done_lo = nz, done_hi = 0; /* node slices issued: [done_lo, done_hi) */
    for (size_t q = 0; q < slabs.size(); q++) {
      const long long k0 = slabs[q].first, k1 = slabs[q].second;
      long long a = std::max(k0 - 1, 0LL), b = std::min(k1, ncz - 1) + 2; /* node slices [a, b) */
      if (q == 0) {
        if (sd.z_descending) b = nz; else a = 0;
      }
      if (q + 1 == slabs.size()) {
        if (sd.z_descending) a = 0; else b = nz;
      }
      long long ca = a, cb = b;
      if (q > 0) {
        if (sd.z_descending) { cb = std::min(b, done_lo); ca = std::min(a, cb); }
        else { ca = std::max(a, done_hi); cb = std::max(b, ca); }
      }
      done_lo = std::min(done_lo, ca);
      done_hi = std::max(done_hi, cb);
      ranges.push_back({(size_t)ca * slice, (size_t)cb * slice});
    }
    while (c.chunk_ev.size() < ranges.size()) {
      cudaEvent_t e; /* with timing: the trace reports when each chunk landed */
      C3D_CUDA(cudaEventCreate(&e));
      c.chunk_ev.push_back(e);
    }
    c.chunks_used = ranges.size();
    /* the copies follow the buffer's allocation and every earlier reader */
    C3D_CUDA(cudaEventRecord(c.ev_field, st));
    C3D_CUDA(cudaStreamWaitEvent(c.copy_stream, c.ev_field, 0));
    up.start(c.device, c.copy_stream,
             std::vector<cudaEvent_t>(c.chunk_ev.begin(), c.chunk_ev.begin() + (long)ranges.size()),
             static_cast<char *>(c.field.p), static_cast<const char *>(ci.data), ranges);
  }
  int slab_index = 0;
  /* the last slab's code arrays: the whole field's when that slab covers it */
  std::vector<unsigned char *> last_codes(nobj, nullptr);
  bool codes_whole = false;
  unsigned *h_small = c.h_small.as<unsigned>();
  unsigned long long *h_total = reinterpret_cast<unsigned long long *>(h_small + 4);
  for (const auto &slab : slabs) {
    const long long k0 = slab.first, k1 = slab.second;
    SlabDev S;
    S.kfirst = std::max(k0 - 1, 0LL);
    const long long klast = std::min(k1, ncz - 1); /* inclusive */
    S.nslices = klast - S.kfirst + 1;
    S.krender0 = std::max(k0, 1LL);
    S.krender1 = std::min(k1, ncz - 1);
    const long long ncell = S.nslices * per_slice;
    /* one code array per object, each starting on 256 bytes (the scan and the
       vertex pass read codes with 16-byte loads) */
    const size_t code_stride = ((size_t)ncell + 255) & ~(size_t)255;
    if (c.counts.ensure(code_stride * nobj, st) || c.scratch.ensure(128, st)) return 1;
    unsigned *d_counter = c.scratch.as<unsigned>();
    unsigned *d_err = async ? c.checks.as<unsigned>() + kClsErrWord : d_counter + 1;
    unsigned *d_ovf = c.checks.as<unsigned>() + kOvfWord;
    if (pipelined) {
      if (!up.wait(slab_index)) {
        log_error("%s", up.what);
        return 1;
      }
      C3D_CUDA(cudaStreamWaitEvent(st, c.chunk_ev[slab_index], 0));
    }
    slab_index++;
    /* the cell codes of every object of the slab, one pass over the field
       for up to four objects -- or the codes the batch classified already,
       when the slab is the whole field */
    codes_whole = S.kfirst == 0 && S.nslices == ncz;
    bool pre = codes_whole && slabs.size() == 1;
    for (size_t q = 0; q < nobj; q++) pre = pre && objs[q].pre_codes != nullptr;
    std::vector<unsigned char *> obj_codes(nobj);
    for (size_t q = 0; q < nobj; q++)
      obj_codes[q] = pre ? objs[q].pre_codes : c.counts.as<unsigned char>() + code_stride * q;
    last_codes = obj_codes;
    if (!async) C3D_CUDA(cudaMemsetAsync(d_err, 0, sizeof(unsigned), st));
    if (c.stage_timing) cudaEventRecord(c.evs[0], st);
    if (!pre)
      c.stats.kernel_launches += (uint64_t)launch_classify(Fo.data(), (int)nobj, S, obj_codes.data(), d_err, st);
    if (c.stage_timing) cudaEventRecord(c.evs[1], st);
    /* unsynchronised frames: odd objects on the second lane, after the
       classification; joined again before the next slab's classification */
    const int nlanes = async && !sink && !c.stage_timing && nobj > 1 ? 2 : 1;
    const cudaStream_t st_main = st;
    if (nlanes > 1) {
      C3D_CUDA(cudaEventRecord(c.ev_lane_fork, st_main));
      C3D_CUDA(cudaStreamWaitEvent(c.lane_stream, c.ev_lane_fork, 0));
    }
    for (size_t ob = 0; ob < nobj; ob++) {
      const FieldDev &F = Fo[ob];
      unsigned char *codes = obj_codes[ob];
      const bool odd_lane = nlanes > 1 && (ob & 1);
      Ctx::Lane &L = c.lanes[odd_lane ? 1 : 0];
      const cudaStream_t st = odd_lane ? c.lane_stream : st_main; /* this object's pass */
      if (L.offsets.ensure(sizeof(unsigned) * (size_t)(ncell + 1), st) ||
          L.voffsets.ensure(voff_bytes(ncell), st) ||
          L.tile_state.ensure(sizeof(unsigned long long) * (size_t)scan_state_words(ncell), st))
        return 1;
      /* the triangle -> cell map is written by the scan when the slab's
         triangles fit: the buffer keeps the size of the largest slab so far,
         at least one triangle per two cells */
      if (L.tri_cell.ensure(sizeof(unsigned) * (size_t)(ncell / 2 + 1024), st)) return 1;
      unsigned long long *scan_state = L.tile_state.as<unsigned long long>();
      const unsigned long long obase = order_base + 12ULL * (unsigned long long)(ncx * ncy * ncz) * ob;
      /* this slab and object's record of the frame status: the scan's totals
         (triangles, vertices), then the raster counters */
      unsigned long long *srec = nullptr;
      if (async) {
        if (c.status_next >= kStatusSlabs) {
          log_error("internal: more slab passes than status records");
          return 1;
        }
        srec = c.status.as<unsigned long long>() + kStatusHead + kSlabRec * c.status_next++;
      }
      unsigned long long *d_total = async ? srec : reinterpret_cast<unsigned long long *>(d_counter + 2);
      if (async) {
        /* sized before the count is known, from the largest slab seen so
           far; kernels that find more record an overflow and the frame is
           rendered again */
        if (L.tri_cell.ensure(sizeof(unsigned) * c.caps.T, st) ||
            L.tri.ensure(kRecBytes * (c.caps.T + 64 + emit_list_slack((long long)c.caps.T)), st))
          return 1;
      }
      /* read per object: an earlier object of the slab may have grown the buffer */
      const unsigned long long tri_cap = L.tri_cell.cap / sizeof(unsigned);
      if (c.stage_timing && ob > 0) cudaEventRecord(c.evs[1], st);
      C3D_CUDA(launch_scan(codes, ncell, scan_state, L.offsets.as<unsigned>(), L.voff(ncell), d_total,
                           L.tri_cell.as<unsigned>(), tri_cap, sink != nullptr, async ? d_ovf : nullptr, d_err, st));
      if (c.stage_timing) cudaEventRecord(c.evs[2], st);
      c.stats.kernel_launches += 1;
      unsigned long long T = 0, NV = 0;
      if (async) {
        T = c.caps.T;
        NV = c.caps.V;
        c.stats.slabs += 1;
      } else {
        C3D_CUDA(cudaMemcpyAsync(h_small, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        C3D_CUDA(cudaMemcpyAsync(h_total, d_total, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        C3D_CUDA(cudaStreamSynchronize(st));
        if (c.stage_timing) {
          if (ob == 0) c.stats.ms_classify += elapsed(c.evs[0], c.evs[1]);
          c.stats.ms_scan += elapsed(c.evs[1], c.evs[2]);
        }
        if (h_small[0]) {
          log_error("device classification or scan did not complete (error flags 0x%x)", h_small[0]);
          return 1;
        }
        T = h_total[0];
        NV = h_total[1];
        c.stats.triangles += T;
        c.stats.slabs += 1;
        c.caps.T = std::max(c.caps.T, T);
        c.caps.V = std::max(c.caps.V, NV);
        if (T == 0) continue;
      }
      /* the float4 records start at byte 24 * cap: keep cap a multiple of 32 so
         every sub-array stays aligned (and over-allocate so that cap >= T) */
      /* the record region also holds the empty ends of k_emit's list chunks */
      const unsigned long long slack = sink ? 0ULL : emit_list_slack((long long)T);
      if (L.tri_cell.ensure(sizeof(unsigned) * T, st) || L.tri.ensure(tri_bytes(sink) * (T + 64 + slack), st))
        return 1;
      const size_t cap = (L.tri.cap / tri_bytes(sink)) & ~(size_t)31;
      if (cap < T + slack) {
        log_error("internal: triangle buffer capacity %zu below %llu", cap, T + slack);
        return 1;
      }
      double *dbg = nullptr;
      if (sink) {
        if (c.dbg.ensure(sizeof(double) * kDbgDoubles * cap, st)) return 1;
        dbg = c.dbg.as<double>();
      }
      TriDev tri = tri_layout(L.tri.p, cap, dbg, sink != nullptr);
      tri.rec_cap = cap;
      tri.cap = std::min<unsigned long long>(cap, L.tri_cell.cap / sizeof(unsigned));
      tri.ovf = d_ovf;
      unsigned *checks = c.filter_check ? c.checks.as<unsigned>() : nullptr;
      /* the vertex stage: triangle -> cell map, screen vertices */
      if (c.stage_timing) cudaEventRecord(c.evs[3], st);
      if (!async && T > tri_cap) {
        /* the map did not fit: the scan again, with the grown map */
        C3D_CUDA(launch_scan(codes, ncell, scan_state, L.offsets.as<unsigned>(), L.voff(ncell), d_total,
                             L.tri_cell.as<unsigned>(), L.tri_cell.cap / sizeof(unsigned), sink != nullptr, nullptr,
                             d_err, st));
        c.stats.kernel_launches += 1;
      }
      VertDev VD = {};
      if (!sink) {
        /* the screen vertices of the slab's crossed edges, 16 bytes each */
        if (L.verts.ensure(16 * (size_t)NV + 64, st)) return 1;
        VD.pos = L.verts.as<float4>();
        VD.cap = L.verts.cap / 16;
        VD.ovf = d_ovf;
        launch_vertices(F, S, sd, codes, L.voff(ncell), ncell, VD, st);
        c.stats.kernel_launches += 1;
        if (!async) c.stats.vertices += NV;
      }
      if (c.stage_timing) cudaEventRecord(c.evs[8], st);
      const unsigned long long slab_order = obase + 12ULL * (unsigned long long)(S.kfirst * per_slice);
      Geo G;
      G.F = F;
      G.S = S;
      G.lut = c.lut.as<unsigned long long>();
      G.codes = codes;
      G.tri_cell = L.tri_cell.as<unsigned>();
      G.offsets = L.offsets.as<unsigned>();
      if (sink) {
        RasterDev none = {};
        launch_emit(F, S, sd, c.lut.as<unsigned long long>(), codes, L.offsets.as<unsigned>(),
                    L.voff(ncell), L.tri_cell.as<unsigned>(), d_total, (long long)T, tri, none, VD, checks,
                    st);
        launch_exact_all(G, d_total, (long long)T, tri, st);
        launch_normals(F, S, L.offsets.as<unsigned>(), L.tri_cell.as<unsigned>(), d_total, (long long)T, tri, st);
        c.stats.kernel_launches += 3;
      } else {
        /* candidate and tiny lists: about one entry per covered pixel and a few
           percent of the triangles; when one overflows, the slab's emission and
           raster passes run again with larger lists (every z-buffer update is
           an idempotent maximum, so repeating them is harmless).  The cover
           list holds at most one entry per triangle and cannot overflow. */
        unsigned long long cand_want = std::max<unsigned long long>(T / 2, 1ULL << 20);
        unsigned long long tiny_want = std::max<unsigned long long>(T / 16, 1ULL << 16);
        if (async) {
          cand_want = std::max(cand_want, c.caps.cand);
          tiny_want = std::max(tiny_want, c.caps.tiny);
        }
        RasterDev RS = R;
        /* without host synchronisation the counters stay in the frame status */
        unsigned long long *counters = async ? srec + 2 : reinterpret_cast<unsigned long long *>(d_counter + 6);
        unsigned long long *h_cnt = h_total + 2;
        RS.cover_count = counters + 4;
        RS.live_count = counters + 5;
        RS.sliver_count = counters + 6;
        RS.listed_count = counters + 2;
        RS.sliver_rec = tri.rec + 3 * (cap - 1);
        for (int attempt = 0;; attempt++) {
          if (L.cand.ensure(sizeof(Candidate) * cand_want, st) ||
              L.tiny.ensure(sizeof(unsigned) * tiny_want, st))
            return 1;
          RS.cand = L.cand.as<Candidate>();
          RS.cand_cap = L.cand.cap / sizeof(Candidate);
          RS.cand_count = counters + 0;
          RS.tiny = L.tiny.as<unsigned>();
          RS.tiny_cap = L.tiny.cap / sizeof(unsigned);
          RS.tiny_count = counters + 1;
          if (!async) C3D_CUDA(cudaMemsetAsync(counters, 0, kCounters * sizeof(unsigned long long), st));
          if (c.stage_timing) cudaEventRecord(c.evs[9], st);
          launch_emit(F, S, sd, c.lut.as<unsigned long long>(), codes, L.offsets.as<unsigned>(),
                      L.voff(ncell), L.tri_cell.as<unsigned>(), d_total, (long long)T, tri, RS, VD, checks,
                      st);
          if (c.stage_timing) cudaEventRecord(c.evs[4], st);
          launch_raster(G, sd, (long long)T, tri, RS, checks, st);
          if (c.stage_timing) cudaEventRecord(c.evs[5], st);
          launch_finish(G, sd, (long long)(RS.cand_cap + RS.tiny_cap), RS, slab_order, checks, st);
          if (c.stage_timing) cudaEventRecord(c.evs[6], st);
          trace_mark(c, st, "slab " + std::to_string(slab_index - 1) + " object " + std::to_string(ob) + " (" +
                                std::to_string(S.nslices) + " slices) raster done");
          c.stats.kernel_launches += 3;
          if (async) {
            /* list capacities of this pass, compared with the counts at the frame's end */
            c.async_cand_cap = std::min(c.async_cand_cap, RS.cand_cap);
            c.async_tiny_cap = std::min(c.async_tiny_cap, RS.tiny_cap);
            break;
          }
          C3D_CUDA(cudaMemcpyAsync(h_cnt, counters, kCounters * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
          C3D_CUDA(cudaStreamSynchronize(st));
          if (h_cnt[0] <= RS.cand_cap && h_cnt[1] <= RS.tiny_cap) break;
          if (attempt > 4) {
            log_error("raster candidate lists keep overflowing (%llu, %llu)", h_cnt[0], h_cnt[1]);
            return 1;
          }
          c.stats.candidate_overflows += 1;
          cand_want = std::max<unsigned long long>(cand_want, h_cnt[0] + h_cnt[0] / 4);
          tiny_want = std::max<unsigned long long>(tiny_want, h_cnt[1] + h_cnt[1] / 4);
        }
        if (!async) {
          c.stats.candidates += h_cnt[0];
          c.stats.tiny += h_cnt[1];
          c.stats.cover_triangles += h_cnt[2];
          c.stats.exact_fragments += h_cnt[5];
          c.stats.slivers += h_cnt[3];
          c.caps.cand = std::max(c.caps.cand, h_cnt[0] + h_cnt[0] / 4);
          c.caps.tiny = std::max(c.caps.tiny, h_cnt[1] + h_cnt[1] / 4);
        }
        if (c.stage_timing) {
          c.stats.ms_vertices += elapsed(c.evs[3], c.evs[8]);
          c.stats.ms_emit += elapsed(c.evs[9], c.evs[4]);
          c.stats.ms_cover += elapsed(c.evs[4], c.evs[5]);
          c.stats.ms_exact += elapsed(c.evs[5], c.evs[6]);
        }
      }
      if (sink) {
        /* copy this slab's triangles back and keep the rendered ones in order */
        std::vector<unsigned> meta(T), cellv(T);
        /* the slab's T entries of each inspection array (the buffers have
           the capacity of the largest slab so far): vertices and vertex
           normals as 18 rows of pitch cap, face normals (3 per triangle),
           areas; nothing when only counts are wanted */
        const bool want_records = sink->out && sink->count < sink->capacity;
        std::vector<double> dv(want_records ? kDbgDoubles * T : 0);
        C3D_CUDA(cudaMemcpyAsync(meta.data(), tri.meta, sizeof(unsigned) * T, cudaMemcpyDeviceToHost, st));
        C3D_CUDA(cudaMemcpyAsync(cellv.data(), L.tri_cell.p, sizeof(unsigned) * T, cudaMemcpyDeviceToHost, st));
        if (want_records) {
          C3D_CUDA(cudaMemcpy2DAsync(dv.data(), sizeof(double) * T, dbg, sizeof(double) * cap, sizeof(double) * T, 18,
                                     cudaMemcpyDeviceToHost, st));
          C3D_CUDA(cudaMemcpyAsync(dv.data() + 18 * T, dbg + 18 * cap, sizeof(double) * 3 * T, cudaMemcpyDeviceToHost,
                                   st));
          C3D_CUDA(cudaMemcpyAsync(dv.data() + 21 * T, dbg + 21 * cap, sizeof(double) * T, cudaMemcpyDeviceToHost,
                                   st));
        }
        C3D_CUDA(cudaStreamSynchronize(st));
        for (unsigned long long t = 0; t < T; t++) {
          const long long cl = cellv[t] & kTcCellMask;
          const long long i = cl % ncx, j = (cl / ncx) % ncy, k = S.kfirst + cl / (ncx * ncy);
          if (k >= k0 && k < k1) sink->triangulated++;
          if (!(meta[t] & kMetaRendered)) continue;
          if (sink->out && sink->count < sink->capacity) {
            TriRecord &r = sink->out[sink->count];
            for (int q = 0; q < 9; q++) r.vertices[q] = dv[q * T + t];
            for (int q = 0; q < 9; q++) r.vertex_normals[q] = dv[(9 + q) * T + t];
            for (int q = 0; q < 3; q++) r.face_normal[q] = dv[18 * T + 3 * t + q];
            r.area = dv[21 * T + t];
            r.cell[0] = i + (long long)ci.off[0];
            r.cell[1] = j + (long long)ci.off[1];
            r.cell[2] = k + (long long)ci.off[2];
            for (int q = 0; q < 3; q++) r.edge_ids[q] = (meta[t] >> (5 * q)) & 31;
          }
          sink->count++;
        }
      }
    }
    if (nlanes > 1) {
      C3D_CUDA(cudaEventRecord(c.ev_lane_join, c.lane_stream));
      C3D_CUDA(cudaStreamWaitEvent(st_main, c.ev_lane_join, 0));
    }
  }
  if (!sink) {
    /* every object's won pixels, shaded once after all of its slabs */
    const size_t npx = (size_t)(sd.width * sd.height);
    if (c.scratch.ensure(128, st)) return 1;
    if (c.filter_check && c.shade_check.ensure(sizeof(unsigned) * npx, st)) return 1;
    unsigned long long *counters = reinterpret_cast<unsigned long long *>(c.scratch.as<unsigned>() + 6);
    unsigned long long *h_cnt = h_total + 2;
    unsigned *checks = c.filter_check ? c.checks.as<unsigned>() : nullptr;
    /* unsynchronised frames: odd objects' shading on the second lane */
    const int slanes = async && !c.stage_timing && nobj > 1 ? 2 : 1;
    const cudaStream_t st_main = st;
    if (slanes > 1) {
      C3D_CUDA(cudaEventRecord(c.ev_lane_fork, st_main));
      C3D_CUDA(cudaStreamWaitEvent(c.lane_stream, c.ev_lane_fork, 0));
    }
    for (size_t ob = 0; ob < nobj; ob++) {
      const contour3d_color_t &col = objs[ob].color;
      const bool odd_lane = slanes > 1 && (ob & 1);
      Ctx::Lane &L = c.lanes[odd_lane ? 1 : 0];
      const cudaStream_t st = odd_lane ? c.lane_stream : st_main; /* this object's shading */
      if (L.win.ensure(sizeof(unsigned) * npx, st) || L.amb.ensure(sizeof(unsigned) * npx, st)) return 1;
      if (async) {
        /* the object's record of the frame status: won, ambiguous, neighbour entries */
        if (c.status_obj_next >= kStatusObjs) {
          log_error("internal: more contour objects than status records");
          return 1;
        }
        counters = c.status.as<unsigned long long>() + kStatusHead + kSlabRec * kStatusSlabs + 3 * c.status_obj_next++;
      }
      RasterDev RS = R;
      RS.win = L.win.as<unsigned>();
      RS.win_count = counters + 0;
      RS.amb = L.amb.as<unsigned>();
      RS.amb_count = counters + 1;
      /* render.c:150-159 at the clamped factor: (unsigned char)(int)(0.15 * c) in FP64 */
      const int r8 = (int)(0.15 * (double)col.r), g8 = (int)(0.15 * (double)col.g), b8 = (int)(0.15 * (double)col.b);
      RS.clamp_rgb = ((unsigned)(unsigned char)r8 << 16) | ((unsigned)(unsigned char)g8 << 8) |
                     (unsigned)(unsigned char)b8;
      RS.shade_check = c.filter_check ? c.shade_check.as<unsigned>() : nullptr;
      const unsigned rgb = ((unsigned)col.r << 16) | ((unsigned)col.g << 8) | col.b;
      const unsigned long long obase = order_base + 12ULL * (unsigned long long)(ncx * ncy * ncz) * ob;
      if (!async) C3D_CUDA(cudaMemsetAsync(counters, 0, 3 * sizeof(unsigned long long), st));
      if (c.stage_timing) cudaEventRecord(c.evs[6], st);
      /* the classification's codes, when the slab loop left the whole field's */
      FieldDev Fs = Fo[ob];
      Fs.codes = codes_whole ? last_codes[ob] : nullptr;
      launch_shade_f(Fs, sd, RS, c.lut.as<unsigned long long>(), obase, rgb, st);
      if (c.stage_timing) cudaEventRecord(c.evs[10], st);
      trace_mark(c, st, "object " + std::to_string(ob) + " FP32 shading done");
      /* without node spacings (a converter) every won pixel takes the FP64 pass */
      const bool fp32 = Fo[ob].dgx != nullptr && nx <= (1 << 20) && ny <= (1 << 20) && nz <= (1 << 20);
      const unsigned *list = fp32 ? RS.amb : RS.win;
      const unsigned long long *lcount = fp32 ? RS.amb_count : RS.win_count;
      if (async) {
        /* the FP64 pass over at most every pixel, its neighbour entries
           sized from the largest count seen; overflow shows in the status */
        const unsigned long long want = std::max<unsigned long long>(c.caps.ent, 1ULL << 16);
        if (L.nb_ent.ensure(sizeof(unsigned long long) * want, st) || L.nb_wn.ensure(3 * sizeof(double) * want, st) ||
            L.nb_span.ensure(sizeof(uint2) * 3 * npx, st))
          return 1;
        const unsigned long long cap =
            std::min(L.nb_ent.cap / sizeof(unsigned long long), L.nb_wn.cap / (3 * sizeof(double)));
        c.async_ent_cap = std::min(c.async_ent_cap, cap);
        c.async_obj_fp32.push_back(fp32 ? 1 : 0);
        launch_shade_exact(Fs, sd, RS, c.lut.as<unsigned long long>(), list, lcount, (long long)npx, obase,
                           L.nb_ent.as<unsigned long long>(), cap, counters + 2, L.nb_span.as<uint2>(),
                           L.nb_wn.as<double>(), rgb, fp32 ? checks : nullptr, st);
        c.stats.kernel_launches += 3 + (fp32 ? 2 : 1);
        continue;
      }
      C3D_CUDA(cudaMemcpyAsync(h_cnt, counters, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
      C3D_CUDA(cudaStreamSynchronize(st));
      const unsigned long long nwin = h_cnt[0], namb = fp32 ? h_cnt[1] : nwin;
      unsigned long long entries = 0;
      if (namb) {
        /* about six neighbour triangles per vertex; more are listed again */
        unsigned long long want = 24 * namb + 1024;
        for (int attempt = 0;; attempt++) {
          if (L.nb_ent.ensure(sizeof(unsigned long long) * want, st) || L.nb_wn.ensure(3 * sizeof(double) * want, st) ||
              L.nb_span.ensure(sizeof(uint2) * 3 * namb, st))
            return 1;
          const unsigned long long cap =
              std::min(L.nb_ent.cap / sizeof(unsigned long long), L.nb_wn.cap / (3 * sizeof(double)));
          C3D_CUDA(cudaMemsetAsync(counters + 2, 0, sizeof(unsigned long long), st));
          launch_shade_exact(Fs, sd, RS, c.lut.as<unsigned long long>(), list, lcount, (long long)namb, obase,
                             L.nb_ent.as<unsigned long long>(), cap, counters + 2, L.nb_span.as<uint2>(),
                             L.nb_wn.as<double>(), rgb, fp32 ? checks : nullptr, st);
          c.stats.kernel_launches += 3;
          C3D_CUDA(cudaMemcpyAsync(h_cnt + 2, counters + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
          C3D_CUDA(cudaStreamSynchronize(st));
          entries = h_cnt[2];
          if (entries <= cap) break;
          if (attempt > 3) {
            log_error("shading neighbour lists keep overflowing (%llu)", entries);
            return 1;
          }
          want = entries + entries / 4;
        }
      }
      if (c.stage_timing) cudaEventRecord(c.evs[7], st);
      c.stats.kernel_launches += fp32 ? 2 : 1;
      c.stats.winners += nwin;
      c.stats.shade_exact += namb;
      c.stats.normals += entries;
      c.caps.ent = std::max(c.caps.ent, entries + entries / 4);
      if (c.stage_timing) {
        cudaEventSynchronize(c.evs[7]);
        c.stats.ms_normals += elapsed(c.evs[6], c.evs[10]);
        c.stats.ms_shade += elapsed(c.evs[10], c.evs[7]);
      }
    }
    if (slanes > 1) {
      C3D_CUDA(cudaEventRecord(c.ev_lane_join, c.lane_stream));
      C3D_CUDA(cudaStreamWaitEvent(st_main, c.ev_lane_join, 0));
    }
  }
  order_base += 12ULL * (unsigned long long)(ncx * ncy * ncz) * nobj;
  return 0;
}

/* the field groups of a frame: objects that read one field with one
   geometry share its upload, node tables and slabs (inspection takes one
   object at a time) */
static std::vector<std::pair<size_t, size_t>> field_groups(const FrameIn &f, bool one_each) {
  std::vector<std::pair<size_t, size_t>> groups;
  for (size_t n = 0; n < f.contours.size();) {
    size_t m = n + 1;
    if (!one_each)
      while (m < f.contours.size() && same_field(f.contours[n], f.contours[m])) m++;
    groups.push_back({n, m});
    n = m;
  }
  return groups;
}

/* a frame rendered without host synchronisation found more work than its
   buffers were sized for: render it again with synchronisation */
static const int kFrameRedo = 2;

static int render_frame_pass(Ctx &c, const FrameIn &f, const FrameOut &o, bool async);
static int frame_status(Ctx &c, bool async);

/* FNV-1a over everything a frame's recorded work depends on besides the
   field values: the scene, each field's address, type, sizes, node
   coordinates, converter, level and colour, the lines, the output and the
   stream */
struct KeyHash {
  uint64_t h = 1469598103934665603ULL;
  void add(const void *p, size_t n) {
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t q = 0; q < n; q++) h = (h ^ b[q]) * 1099511628211ULL;
  }
  template <typename T> void add(const T &v) { add(&v, sizeof v); }
};

static uint64_t frame_key(const Ctx &c, const FrameIn &f, const FrameOut &o) {
  KeyHash k;
  const HostScene &s = f.scene;
  k.add(s.cam);
  k.add(s.center);
  k.add(s.lx);
  k.add(s.ly);
  k.add(s.light);
  k.add(s.W);
  k.add(s.H);
  k.add(f.bg);
  for (const ContourIn &ci : f.contours) {
    k.add(ci.data);
    k.add(ci.f32);
    k.add(ci.sz);
    k.add(ci.converter);
    k.add(ci.threshold);
    k.add(ci.color);
    for (int d = 0; d < 3; d++) k.add(ci.grid[d], sizeof(double) * ci.sz[d]);
  }
  if (f.nlines) k.add(f.lines, sizeof(contour3d_line_obj_t) * f.nlines);
  k.add(o.rgb_dev);
  k.add(f.stream);
  /* a recorded graph keeps the launch shapes, launch attributes and slab
     sizes it was recorded with: another setting is another frame */
  const LaunchShape ls = launch_shape();
  k.add(ls.cls_z);
  k.add(ls.emit_per_sm);
  k.add(ls.raster_per_sm);
  k.add(dependent_launch());
  k.add(c.slab_cells);
  return k.h;
}

/* device-resident identity-grid fields drawn into a device image on a
   stream of the caller's or the context's (the legacy default stream cannot
   be recorded) */
static bool graph_eligible(const Ctx &c, const FrameIn &f, const FrameOut &o) {
  if (!c.graphs_enabled || !f.stream || o.sink || o.rgb_host || o.rgb_pinned || o.depth_host || o.pixels_host ||
      !o.rgb_dev || c.filter_check || c.stage_timing)
    return false;
  for (const ContourIn &ci : f.contours)
    if (!ci.on_device || !is_identity(ci.converter) || ci.pre_codes) return false; /* codes of one batch */
  return true;
}

static void drop_graph(Ctx &c) {
  if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
  c.graph_exec = nullptr;
}

/* end the recording of the current frame, keep it as the context's graph and
   run it on `st` (between the frame's timing events) */
static int end_capture_and_launch(Ctx &c, cudaStream_t st) {
  cudaGraph_t g = nullptr;
  c.capturing = false;
  cudaError_t e = cudaStreamEndCapture(st, &g);
  drop_graph(c);
  if (e == cudaSuccess && g) e = cudaGraphInstantiate(&c.graph_exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess || !c.graph_exec) {
    log_error("recording the frame as a graph failed: %s", cudaGetErrorString(e));
    c.graph_exec = nullptr;
    return 1;
  }
  Ctx::GraphFrame &gf = c.graph_frame;
  gf.status_next = c.status_next;
  gf.status_obj_next = c.status_obj_next;
  gf.cand_cap = c.async_cand_cap;
  gf.tiny_cap = c.async_tiny_cap;
  gf.ent_cap = c.async_ent_cap;
  gf.obj_fp32 = c.async_obj_fp32;
  gf.kernel_launches = c.stats.kernel_launches;
  gf.slabs = c.stats.slabs;
  gf.cells = c.stats.cells;
  C3D_CUDA(cudaEventRecord(c.ev0, st));
  C3D_CUDA(cudaGraphLaunch(c.graph_exec, st));
  C3D_CUDA(cudaEventRecord(c.ev1, st));
  return 0;
}

/* the context's graph run again: the frame's work with its final copies of
   the status words, then the one synchronisation */
static int replay_graph(Ctx &c, cudaStream_t st) {
  const Ctx::GraphFrame &gf = c.graph_frame;
  c.stats = contour3d_gb300_stats_t{};
  c.stats.kernel_launches = gf.kernel_launches;
  c.stats.slabs = gf.slabs;
  c.stats.cells = gf.cells;
  c.frame_async = true;
  c.status_next = gf.status_next;
  c.status_obj_next = gf.status_obj_next;
  c.async_cand_cap = gf.cand_cap;
  c.async_tiny_cap = gf.tiny_cap;
  c.async_ent_cap = gf.ent_cap;
  c.async_obj_fp32 = gf.obj_fp32;
  C3D_CUDA(cudaEventRecord(c.ev0, st));
  C3D_CUDA(cudaGraphLaunch(c.graph_exec, st));
  C3D_CUDA(cudaEventRecord(c.ev1, st));
  C3D_CUDA(cudaStreamSynchronize(st));
  C3D_CUDA(cudaGetLastError());
  return frame_status(c, true);
}

/*
 * One frame.  The first frame of a context synchronises after every slab
 * pass and learns the counts; later frames run unsynchronised, sized from
 * them, and are rendered again with synchronisation if they find more work.
 * An unsynchronised device frame whose description repeats is recorded as a
 * CUDA graph the second time and launched as one from the third on (an
 * in-situ solver's time steps: the same fields, levels and camera, new field
 * values).
 */
static int render_frame(Ctx &c, const FrameIn &f, const FrameOut &o) {
  const bool async = c.async_enabled && c.caps_known && !o.sink && !c.stage_timing;
  int rc = -1;
  bool redone = false, replayed = false, recorded = false;
  if (async && graph_eligible(c, f, o)) {
    const uint64_t key = frame_key(c, f, o);
    if (c.graph_exec && c.graph_key == key) {
      rc = replay_graph(c, f.stream);
      replayed = true;
    } else if (c.graph_key_seen && c.graph_key == key) {
      C3D_CUDA(cudaEventSynchronize(c.ev_staged));
      if (cudaStreamBeginCapture(f.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        c.capturing = true;
        t_capture_needs_growth = false;
        rc = render_frame_pass(c, f, o, true);
        if (c.capturing) {
          /* the recording stopped short (a buffer had to grow, or an error):
             abandon it and render the frame without it */
          c.capturing = false;
          cudaGraph_t g = nullptr;
          cudaStreamEndCapture(f.stream, &g);
          if (g) cudaGraphDestroy(g);
          cudaGetLastError();
          drop_graph(c);
          rc = -1;
        } else {
          recorded = rc != 1;
        }
      } else {
        cudaGetLastError();
      }
    } else {
      drop_graph(c);
      c.graph_key = key;
      c.graph_key_seen = true;
    }
  }
  if (rc == -1) rc = render_frame_pass(c, f, o, async);
  if (rc == 0) trace_print(c);
  if (rc == kFrameRedo) {
    /* the graph (if any) was sized for less work than this frame has */
    drop_graph(c);
    c.graph_key_seen = false;
    rc = render_frame_pass(c, f, o, false);
    redone = true;
  }
  if (rc == 0 && !o.sink) c.caps_known = true;
  c.stats.unsynchronised = async && !redone ? 1 : 0;
  c.stats.redone = redone ? 1 : 0;
  c.stats.graph = replayed && !redone ? 2 : (recorded && !redone ? 1 : 0);
  return rc;
}

/* after a frame's final synchronisation: its error words, and for an
   unsynchronised frame the counts of every pass (statistics, the sizes later
   frames use, and whether the frame must be rendered again) */
static int frame_status(Ctx &c, bool async) {
  const unsigned *h_checks = c.h_small.as<unsigned>() + 32;
  const unsigned long long *hs = c.h_status.as<unsigned long long>();
  const size_t obj0 = kStatusHead + (size_t)kSlabRec * kStatusSlabs;
  if (h_checks[kZbufErrWord]) {
    log_error("a z-buffer update gave up after its retry bound (error flags 0x%x)", h_checks[kZbufErrWord]);
    return 1;
  }
  if (async) {
    if (h_checks[kClsErrWord]) {
      log_error("device classification or scan did not complete (error flags 0x%x)", h_checks[kClsErrWord]);
      return 1;
    }
    /* the counts of every pass: statistics, and the sizes the next frames use */
    bool over = h_checks[kOvfWord] != 0;
    for (int q = 0; q < c.status_next; q++) {
      const unsigned long long *r = hs + kStatusHead + (size_t)kSlabRec * q, *cnt = r + 2;
      c.stats.triangles += r[0];
      c.stats.vertices += r[1];
      c.stats.candidates += cnt[0];
      c.stats.tiny += cnt[1];
      c.stats.cover_triangles += cnt[2];
      c.stats.exact_fragments += cnt[5];
      c.stats.slivers += cnt[3];
      over = over || cnt[0] > c.async_cand_cap || cnt[1] > c.async_tiny_cap;
      c.caps.T = std::max(c.caps.T, r[0]);
      c.caps.V = std::max(c.caps.V, r[1]);
      c.caps.cand = std::max(c.caps.cand, cnt[0] + cnt[0] / 4);
      c.caps.tiny = std::max(c.caps.tiny, cnt[1] + cnt[1] / 4);
    }
    for (int q = 0; q < c.status_obj_next; q++) {
      const unsigned long long *r = hs + obj0 + 3 * (size_t)q;
      c.stats.winners += r[0];
      c.stats.shade_exact += c.async_obj_fp32[(size_t)q] ? r[1] : r[0];
      c.stats.normals += r[2];
      over = over || r[2] > c.async_ent_cap;
      c.caps.ent = std::max(c.caps.ent, r[2] + r[2] / 4);
    }
    if (over) return kFrameRedo;
  }
  c.stats.ms_total = elapsed(c.ev0, c.ev1);
  for (int q = 0; q < 5; q++) c.stats.filter_violations[q] = h_checks[q];
  c.stats.shade_violations = h_checks[5];
  return 0;
}

static int render_frame_pass(Ctx &c, const FrameIn &f, const FrameOut &o, bool async) {
  const HostScene &s = f.scene;
  const size_t W = s.W, H = s.H, npx = W * H;
  if (W == 0 || H == 0) {
    log_error("screen size must be positive (%zu x %zu)", W, H);
    return 1;
  }
  c.stats = contour3d_gb300_stats_t{};
  c.frame_async = async;
  c.trace_used = 0;
  c.chunks_used = 0;
  c.status_next = c.status_obj_next = 0;
  c.async_cand_cap = c.async_tiny_cap = c.async_ent_cap = ~0ULL;
  c.async_obj_fp32.clear();
  c.field_src = nullptr;
  c.field_bytes = 0;
  c.stats_h2d = 0;
  cudaStream_t st = f.stream;
  const std::vector<std::pair<size_t, size_t>> groups = field_groups(f, o.sink != nullptr);
  std::vector<LineSegDev> segs;
  if (build_line_segs(f, segs)) return 1;
  if (!c.capturing) C3D_CUDA(cudaEventRecord(c.ev0, st));
  const SceneDev sd = scene_dev(s);
  FrameConsts fc;
  if (stage_frame_consts(c, f, groups, segs, fc)) return 1;
  if (c.canvas.ensure(sizeof(Slot) * npx, st) || c.zlo.ensure(sizeof(unsigned) * npx, st) || c.checks.ensure(64, st))
    return 1;
  /* per-pixel winner weights: tags carry a frame epoch, so the buffer is
     cleared only when it is new or the epoch wraps */
  const void *winfo_before = c.winfo.p;
  if (c.winfo.ensure(3 * sizeof(ulonglong2) * npx, st)) return 1;
  if (c.winfo.p != winfo_before || ++c.epoch >= (1ULL << 24) || c.capturing) {
    /* a recorded frame runs many times with one epoch: it clears the weights */
    C3D_CUDA(cudaMemsetAsync(c.winfo.p, 0, c.winfo.cap, st));
    if (!c.capturing) c.epoch = 1;
  }
  /* the self-check counters (words 0-5), the z-buffer, overflow and
     classification error words */
  C3D_CUDA(cudaMemsetAsync(c.checks.p, 0, 64, st));
  if (async) {
    if (c.status.ensure(sizeof(unsigned long long) * kStatusWords, st) ||
        c.h_status.ensure(sizeof(unsigned long long) * kStatusWords))
      return 1;
    C3D_CUDA(cudaMemsetAsync(c.status.p, 0, sizeof(unsigned long long) * kStatusWords, st));
  }
  RasterDev R = {};
  R.zerr = c.checks.as<unsigned>() + kZbufErrWord;
  R.canvas = c.canvas.as<Slot>();
  R.zlo = c.zlo.as<unsigned>();
  R.winfo = c.winfo.as<ulonglong2>();
  R.epoch = c.epoch;
  R.xs = fc.xy;
  R.ys = R.xs + W;
  R.xsf = fc.xyf;
  R.ysf = R.xsf + W;
  /* canvas: background colour at depth -DBL_MAX (main.c:90-103); depth floors at -inf */
  const unsigned bg = ((unsigned)f.bg.r << 16) | ((unsigned)f.bg.g << 8) | f.bg.b;
  launch_canvas_init(c.canvas.as<Slot>(), R.zlo, (long long)npx, h_depth_key(-1. * DBL_MAX), bg, st);
  c.stats.kernel_launches += 1;
  unsigned long long order_base = 1;
  for (size_t g = 0; g < groups.size(); g++) {
    if (render_contour(c, f, sd, &f.contours[groups[g].first], groups[g].second - groups[g].first, order_base, R,
                       o.sink, fc.groups[g])) {
      if (!(c.capturing && t_capture_needs_growth)) log_error("contour processing failed");
      return 1;
    }
  }
  /* the lines after every contour object (line.c:121-170): pixels on the device */
  if (fc.nseg > 0) {
    launch_lines(fc.segs, fc.nseg, (long long)W, (long long)H, c.canvas.as<Slot>(), order_base, R.zerr, st);
    c.stats.kernel_launches += 1;
    order_base += (unsigned long long)fc.nseg;
  }
  /* resolve */
  uint8_t *rgb_dev = o.rgb_dev;
  const bool want_rgb = o.rgb_host || o.rgb_pinned;
  if (!rgb_dev && want_rgb) {
    if (c.rgb.ensure(3 * npx, st)) return 1;
    rgb_dev = c.rgb.as<uint8_t>();
  }
  if (rgb_dev) {
    launch_resolve(c.canvas.as<Slot>(), (long long)W, (long long)H, rgb_dev, nullptr, st);
    c.stats.kernel_launches += 1;
  }
  if (want_rgb) {
    if (c.h_rgb.ensure(3 * npx)) return 1;
    C3D_CUDA(cudaMemcpyAsync(c.h_rgb.p, rgb_dev, 3 * npx, cudaMemcpyDeviceToHost, st));
  }
  if (o.depth_host || o.pixels_host) {
    if (c.h_slots.ensure(sizeof(Slot) * npx)) return 1;
    C3D_CUDA(cudaMemcpyAsync(c.h_slots.p, c.canvas.p, sizeof(Slot) * npx, cudaMemcpyDeviceToHost, st));
  }
  trace_mark(c, st, "image resolved and copied out");
  if (!c.capturing) C3D_CUDA(cudaEventRecord(c.ev1, st));
  unsigned *h_checks = c.h_small.as<unsigned>() + 32;
  C3D_CUDA(cudaMemcpyAsync(h_checks, c.checks.p, 16 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  unsigned long long *hs = c.h_status.as<unsigned long long>();
  const size_t obj0 = kStatusHead + (size_t)kSlabRec * kStatusSlabs;
  if (async) {
    C3D_CUDA(cudaMemcpyAsync(hs, c.status.p, sizeof(unsigned long long) * (kStatusHead + kSlabRec * c.status_next),
                             cudaMemcpyDeviceToHost, st));
    C3D_CUDA(cudaMemcpyAsync(hs + obj0, c.status.as<unsigned long long>() + obj0,
                             sizeof(unsigned long long) * 3 * c.status_obj_next, cudaMemcpyDeviceToHost, st));
  }
  if (c.capturing) {
    /* the frame's work is recorded, not run: instantiate it and run it */
    if (end_capture_and_launch(c, st)) return 1;
  }
  C3D_CUDA(cudaStreamSynchronize(st));
  C3D_CUDA(cudaGetLastError());
  {
    const int rs = frame_status(c, async);
    if (rs) return rs;
  }
  if (o.rgb_host) memcpy(o.rgb_host, c.h_rgb.p, 3 * npx);
  if (o.depth_host || o.pixels_host) {
    const Slot *sl = c.h_slots.as<Slot>();
    for (size_t p = 0; p < npx; p++) {
      const double dep = depth_from_key(sl[p].hi);
      if (o.depth_host) o.depth_host[p] = dep;
      if (o.pixels_host) {
        PixelRec &r = o.pixels_host[p];
        r.depth = dep;
        r.r = (uint8_t)(sl[p].lo >> 16);
        r.g = (uint8_t)(sl[p].lo >> 8);
        r.b = (uint8_t)(sl[p].lo);
        memset(r.pad, 0, sizeof r.pad);
      }
    }
  }
  return 0;
}

static bool is_identity(conv_fn f) {
  if (!f || f == contour3d_gb300_identity) return true;
  for (int q = 0; q < g_nidentity; q++)
    if (g_identity[q] == f) return true;
  return false;
}

static int check_common(const V *cam, const V *light, const size_t sizes[2], const V *center, const V local[2],
                        const contour3d_color_t *bg) {
  if (!cam || !light || !sizes || !center || !local || !bg) {
    log_error("null scene argument");
    return 1;
  }
  return 0;
}

}  // namespace c3d

using namespace c3d;

extern "C" contour3d_vector_t contour3d_gb300_identity(const contour3d_vector_t p) { return p; }

extern "C" int contour3d_gb300_declare_identity(contour3d_vector_t (*fn)(const contour3d_vector_t)) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!fn) return 1;
  if (is_identity(fn)) return 0;
  if (g_nidentity >= 16) {
    log_error("too many identity converters declared");
    return 1;
  }
  g_identity[g_nidentity++] = fn;
  return 0;
}

extern "C" int contour3d_execute(const sdecomp_info_t *const sdecomp_info,
                                 const contour3d_vector_t *const camera_position,
                                 const contour3d_vector_t *const camera_look_at,
                                 const contour3d_vector_t *const light_direction, const size_t screen_sizes[2],
                                 const contour3d_vector_t *const screen_center,
                                 const contour3d_vector_t screen_local[2], const contour3d_color_t *const bg_color,
                                 const size_t num_contours, const contour3d_contour_obj_t *const objs,
                                 const size_t num_lines, const contour3d_line_obj_t *const lines,
                                 const char fname[]) {
  (void)camera_look_at; /* stored but unused by the reference (main.c:13-23) */
  const auto t_enter = std::chrono::steady_clock::now();
  std::lock_guard<std::mutex> lk(g_mu);
  if (check_common(camera_position, light_direction, screen_sizes, screen_center, screen_local, bg_color)) return 1;
  if ((num_contours && !objs) || (num_lines && !lines)) {
    log_error("null object array");
    return 1;
  }
  if (ctx_init(g_ctx)) return 1;
  FrameIn f;
  f.scene = make_scene(camera_position, light_direction, screen_sizes, screen_center, screen_local);
  f.bg = *bg_color;
  f.lines = lines;
  f.nlines = num_lines;
  f.stream = g_ctx.own_stream;
  bool multi = false;
  std::vector<std::vector<double>> ext_store(num_contours);
  for (size_t n = 0; n < num_contours; n++) {
    const contour3d_contour_obj_t *o = objs + n;
    if (!o->array || !o->grids[0] || !o->grids[1] || !o->grids[2]) {
      log_error("contour object %zu: null array or grid", n);
      return 1;
    }
    BlockInfo b;
    if (decomp_query(sdecomp_info, o, &b)) {
      log_error("failed to extend domain");
      return 1;
    }
    ContourIn ci;
    if (b.single) {
      ci.data = o->array;
    } else {
      multi = true;
      ext_store[n].resize(b.ext_size[0] * b.ext_size[1] * b.ext_size[2]);
      if (extend_block(sdecomp_info, o, b, ext_store[n].data())) {
        log_error("failed to extend domain");
        return 1;
      }
      ci.data = ext_store[n].data();
    }
    for (int d = 0; d < 3; d++) {
      ci.sz[d] = b.single ? b.mysize[d] : b.ext_size[d];
      ci.off[d] = b.single ? b.offset[d] : b.ext_offset[d];
      ci.grid[d] = o->grids[d] + ci.off[d];
    }
    ci.converter = o->converter;
    ci.threshold = o->threshold;
    ci.color = o->color;
    f.contours.push_back(ci);
  }
  MPI_Comm comm = MPI_COMM_NULL;
  sdecomp.get_comm_cart(sdecomp_info, &comm);
  int myrank = 0;
  sdecomp.get_comm_rank(sdecomp_info, &myrank);
  /* the world size decides whether a reduction is needed */
  multi = multi || comm_size(comm) > 1;
  const size_t W = screen_sizes[0], H = screen_sizes[1];
  FrameOut out;
  std::vector<uint8_t> rgb;
  std::vector<PixelRec> px;
  if (multi) {
    px.resize(W * H);
    out.pixels_host = px.data();
  } else {
    out.rgb_pinned = true; /* written to the file straight from the pinned copy */
  }
  if (render_frame(g_ctx, f, out)) return 1;
  const auto t_rendered = std::chrono::steady_clock::now();
  if (multi) {
    if (reduce_nearest(sdecomp_info, px.data(), W * H)) {
      log_error("image output failed");
      return 1;
    }
    if (myrank != 0) return 0;
    rgb.resize(3 * W * H);
    size_t q = 0;
    for (size_t j = 0; j < H; j++)
      for (size_t i = 0; i < W; i++) {
        const PixelRec &p = px[(H - j - 1) * W + i];
        rgb[q++] = p.r;
        rgb[q++] = p.g;
        rgb[q++] = p.b;
      }
  }
  if (myrank != 0) return 0;
  if (write_ppm(fname, W, H, multi ? rgb.data() : g_ctx.h_rgb.as<uint8_t>())) {
    log_error("image output failed");
    return 1;
  }
  if (trace_on()) {
    const auto t_written = std::chrono::steady_clock::now();
    const auto ms = [&](std::chrono::steady_clock::time_point t) {
      return std::chrono::duration<double, std::milli>(t - t_enter).count();
    };
    fprintf(stderr, "[c3d trace] host: frame rendered %.3f ms, ppm written %.3f ms after the call began\n",
            ms(t_rendered), ms(t_written));
  }
  return 0;
}

static int fill_from_objs(FrameIn &f, size_t num_contours, const contour3d_contour_obj_t *objs) {
  for (size_t n = 0; n < num_contours; n++) {
    const contour3d_contour_obj_t *o = objs + n;
    if (!o->array || !o->grids[0] || !o->grids[1] || !o->grids[2]) {
      log_error("contour object %zu: null array or grid", n);
      return 1;
    }
    ContourIn ci;
    ci.data = o->array;
    for (int d = 0; d < 3; d++) {
      ci.sz[d] = o->glsizes[d];
      ci.grid[d] = o->grids[d];
    }
    ci.converter = o->converter;
    ci.threshold = o->threshold;
    ci.color = o->color;
    f.contours.push_back(ci);
  }
  return 0;
}

extern "C" int contour3d_gb300_render(const contour3d_vector_t *camera_position,
                                      const contour3d_vector_t *light_direction, const size_t screen_sizes[2],
                                      const contour3d_vector_t *screen_center,
                                      const contour3d_vector_t screen_local[2], const contour3d_color_t *bg_color,
                                      size_t num_contours, const contour3d_contour_obj_t *objs, size_t num_lines,
                                      const contour3d_line_obj_t *lines, uint8_t *rgb_out, double *depth_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (check_common(camera_position, light_direction, screen_sizes, screen_center, screen_local, bg_color)) return 1;
  if ((num_contours && !objs) || (num_lines && !lines)) {
    log_error("null object array");
    return 1;
  }
  if (ctx_init(g_ctx)) return 1;
  FrameIn f;
  f.scene = make_scene(camera_position, light_direction, screen_sizes, screen_center, screen_local);
  f.bg = *bg_color;
  f.lines = lines;
  f.nlines = num_lines;
  f.stream = g_ctx.own_stream;
  if (fill_from_objs(f, num_contours, objs)) return 1;
  FrameOut out;
  out.rgb_host = rgb_out;
  out.depth_host = depth_out;
  return render_frame(g_ctx, f, out);
}

/* true for memory the device can address (device or managed allocations) */
static bool is_device_pointer(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

/* a device-resident frame description -> the internal frame */
static int frame_from_fields(FrameIn &f, const V *camera_position, const V *light_direction, const size_t sizes[2],
                             const V *screen_center, const V screen_local[2], const contour3d_color_t *bg,
                             size_t num_fields, const contour3d_gb300_field_t *fields, size_t num_lines,
                             const contour3d_line_obj_t *lines) {
  if (check_common(camera_position, light_direction, sizes, screen_center, screen_local, bg)) return 1;
  if ((num_fields && !fields) || (num_lines && !lines)) {
    log_error("null field or line array");
    return 1;
  }
  f.scene = make_scene(camera_position, light_direction, sizes, screen_center, screen_local);
  f.bg = *bg;
  f.lines = lines;
  f.nlines = num_lines;
  for (size_t n = 0; n < num_fields; n++) {
    const contour3d_gb300_field_t *fd = fields + n;
    if (!fd->device_array || !fd->grids[0] || !fd->grids[1] || !fd->grids[2] ||
        (fd->dtype != CONTOUR3D_GB300_F64 && fd->dtype != CONTOUR3D_GB300_F32)) {
      log_error("field %zu: null array/grid or unknown dtype", n);
      return 1;
    }
    if (!is_device_pointer(fd->device_array)) {
      log_error("field %zu: the array is not device memory", n);
      return 1;
    }
    ContourIn ci;
    ci.data = fd->device_array;
    ci.on_device = true;
    ci.f32 = fd->dtype == CONTOUR3D_GB300_F32;
    for (int d = 0; d < 3; d++) {
      ci.sz[d] = fd->sizes[d];
      ci.grid[d] = fd->grids[d];
    }
    ci.converter = fd->converter;
    ci.threshold = fd->threshold;
    ci.color = fd->color;
    f.contours.push_back(ci);
  }
  return 0;
}

extern "C" int contour3d_gb300_render_device(const contour3d_vector_t *camera_position,
                                             const contour3d_vector_t *light_direction, const size_t screen_sizes[2],
                                             const contour3d_vector_t *screen_center,
                                             const contour3d_vector_t screen_local[2],
                                             const contour3d_color_t *bg_color, size_t num_fields,
                                             const contour3d_gb300_field_t *fields, size_t num_lines,
                                             const contour3d_line_obj_t *lines, uint8_t *rgb_out, void *stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!rgb_out || !is_device_pointer(rgb_out)) {
    log_error("the output pointer is not device memory");
    return 1;
  }
  if (ctx_init(g_ctx)) return 1;
  FrameIn f;
  if (frame_from_fields(f, camera_position, light_direction, screen_sizes, screen_center, screen_local, bg_color,
                        num_fields, fields, num_lines, lines))
    return 1;
  f.stream = stream ? static_cast<cudaStream_t>(stream) : g_ctx.own_stream;
  FrameOut out;
  out.rgb_dev = rgb_out;
  return render_frame(g_ctx, f, out);
}

extern "C" int contour3d_gb300_last_stats(contour3d_gb300_stats_t *out) {
  if (!out) return 1;
  std::lock_guard<std::mutex> lk(g_mu);
  *out = g_ctx.stats;
  return 0;
}

extern "C" int contour3d_gb300_set_stage_timing(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_ctx.stage_timing = on != 0;
  return 0;
}

extern "C" int contour3d_gb300_set_filter_check(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_ctx.filter_check = on != 0;
  return 0;
}

extern "C" int contour3d_gb300_set_async(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_ctx.async_enabled = on != 0;
  return 0;
}

extern "C" int contour3d_gb300_set_server_async(int on) {
  g_async_default = on != 0;
  g_graphs_default = on != 0;
  return 0;
}

extern "C" int contour3d_gb300_set_graphs(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_ctx.graphs_enabled = on != 0;
  if (!on) {
    drop_graph(g_ctx);
    g_ctx.graph_key_seen = false;
  }
  return 0;
}

extern "C" int contour3d_gb300_set_launch_shape(int classify_slices, int emit_blocks_per_sm,
                                               int raster_blocks_per_sm) {
  if (set_launch_shape(LaunchShape{classify_slices, emit_blocks_per_sm, raster_blocks_per_sm})) {
    log_error("launch shape out of range (classify slices 1..1024, blocks per SM 1..32)");
    return 1;
  }
  return 0;
}

extern "C" int contour3d_gb300_set_dependent_launch(int on) {
  set_dependent_launch(on);
  return 0;
}

extern "C" int contour3d_gb300_set_upload_model(double link_gb_per_s, double slab_ps_per_cell,
                                                double slab_fixed_us) {
  if (!(link_gb_per_s > 0.0) || !(slab_ps_per_cell > 0.0) || !(slab_fixed_us >= 0.0) ||
      !std::isfinite(link_gb_per_s + slab_ps_per_cell + slab_fixed_us))
    return 1;
  std::lock_guard<std::mutex> lk(c3d::g_upload_mu);
  c3d::g_upload_model.link_bytes_per_s = link_gb_per_s * 1e9;
  c3d::g_upload_model.slab_s_per_cell = slab_ps_per_cell * 1e-12;
  c3d::g_upload_model.slab_fixed_s = slab_fixed_us * 1e-6;
  return 0;
}

extern "C" int contour3d_gb300_set_slab_cells(uint64_t max_cells) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (max_cells < 64) {
    log_error("slab size must be at least 64 cells");
    return 1;
  }
  g_ctx.slab_cells = max_cells;
  return 0;
}

extern "C" long contour3d_gb300_debug_triangles(const contour3d_contour_obj_t *obj, void *out, long capacity,
                                                long *num_triangulated) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!obj) return -1;
  if (ctx_init(g_ctx)) return -1;
  FrameIn f;
  const V cam = {0., 0., 0.}, light = {0., 0., 1.}, center = {0., 0., 0.};
  const V local[2] = {{1., 0., 0.}, {0., 1., 0.}};
  const size_t sizes[2] = {1, 1};
  f.scene = make_scene(&cam, &light, sizes, &center, local);
  f.bg = {0, 0, 0};
  f.stream = g_ctx.own_stream;
  if (fill_from_objs(f, 1, obj)) return -1;
  DebugSink sink;
  sink.out = static_cast<TriRecord *>(out);
  sink.capacity = out ? capacity : 0;
  sink.triangulated_only = true;
  const SceneDev sd = scene_dev(f.scene);
  unsigned long long order = 1;
  RasterDev R = {};
  FrameConsts fc;
  if (stage_frame_consts(g_ctx, f, field_groups(f, true), {}, fc)) return -1;
  if (render_contour(g_ctx, f, sd, &f.contours[0], 1, order, R, &sink, fc.groups[0])) return -1;
  if (num_triangulated) *num_triangulated = sink.triangulated;
  return sink.count;
}

extern "C" long contour3d_gb300_debug_cell_counts(const contour3d_contour_obj_t *obj, uint8_t *counts) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!obj || !obj->array) return -1;
  if (ctx_init(g_ctx)) return -1;
  const long long nx = (long long)obj->glsizes[0], ny = (long long)obj->glsizes[1], nz = (long long)obj->glsizes[2];
  if (nx < 2 || ny < 2 || nz < 2) return 0;
  Ctx &c = g_ctx;
  cudaStream_t st = c.own_stream;
  const size_t nn = (size_t)(nx * ny * nz);
  if (c.field.ensure(8 * nn, st) || c.counts.ensure((size_t)((nx - 1) * (ny - 1) * (nz - 1)), st)) return -1;
  c.field_src = nullptr;
  if (cudaMemcpyAsync(c.field.p, obj->array, 8 * nn, cudaMemcpyHostToDevice, st) != cudaSuccess) return -1;
  FieldDev F = {};
  F.data = c.field.p;
  F.nx = nx;
  F.ny = ny;
  F.nz = nz;
  F.threshold = obj->threshold;
  F.thr_key = h_key(obj->threshold);
  F.thr_nan = std::isnan(obj->threshold) ? 1 : 0;
  F.div_cx = make_fast_div((unsigned)(nx - 1));
  F.div_cy = make_fast_div((unsigned)(ny - 1));
  set_float_threshold(F);
  SlabDev S = {0, nz - 1, 0, 0};
  const size_t ncell = (size_t)((nx - 1) * (ny - 1) * (nz - 1));
  if (c.scratch.ensure(128, st)) return -1;
  unsigned *d_err = c.scratch.as<unsigned>();
  if (cudaMemsetAsync(d_err, 0, sizeof(unsigned), st) != cudaSuccess) return -1;
  unsigned char *codes = c.counts.as<unsigned char>();
  launch_classify(&F, 1, S, &codes, d_err, st);
  std::vector<uint8_t> h(ncell);
  unsigned herr = 0;
  if (cudaMemcpyAsync(h.data(), c.counts.p, ncell, cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
  if (cudaMemcpyAsync(&herr, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  if (herr) {
    log_error("device classification did not complete (error flags 0x%x)", herr);
    return -1;
  }
  std::vector<unsigned long long> lut;
  unsigned char count_of[256];
  build_tables(lut, count_of);
  long total = 0;
  for (size_t q = 0; q < ncell; q++) {
    h[q] = count_of[h[q]]; /* the classify pass stores cell codes */
    total += h[q];
  }
  if (counts) memcpy(counts, h.data(), ncell);
  return total;
}

static void ctx_release(Ctx &c);

extern "C" int contour3d_gb300_release(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  ctx_release(g_ctx);
  /* hand the pool's unused blocks back to the device */
  std::lock_guard<std::mutex> lp(g_pool_mu);
  for (cudaMemPool_t pool : g_pool)
    if (pool) cudaMemPoolTrimTo(pool, 0);
  return 0;
}

/* every device buffer of a context; the constant table (lut) first */
static std::vector<Buf *> ctx_bufs(Ctx &c) {
  std::vector<Buf *> v = {&c.lut, &c.counts, &c.scratch, &c.dbg, &c.field, &c.consts, &c.nodes, &c.canvas,
                          &c.rgb, &c.zlo, &c.winfo, &c.shade_check, &c.checks, &c.status};
  for (Ctx::Lane &L : c.lanes)
    for (Buf *b : {&L.offsets, &L.voffsets, &L.tile_state, &L.tri_cell, &L.tri, &L.verts, &L.cand, &L.tiny,
                   &L.win, &L.amb, &L.nb_ent, &L.nb_wn, &L.nb_span})
      v.push_back(b);
  return v;
}

static void ctx_release(Ctx &c) {
  /* every call of the context has completed, so its buffers go back to the
     pool in order on its own stream */
  for (Buf *b : ctx_bufs(c)) b->release(c.own_stream);
  if (c.ready) cudaStreamSynchronize(c.own_stream);
  c.h_small.release();
  c.h_rgb.release();
  c.h_slots.release();
  c.h_consts.release();
  c.h_status.release();
  if (c.ready) {
    cudaStreamDestroy(c.own_stream);
    cudaEventDestroy(c.ev0);
    cudaEventDestroy(c.ev1);
    cudaEventDestroy(c.ev_staged);
    for (auto &e : c.evs) cudaEventDestroy(e);
    cudaStreamSynchronize(c.copy_stream);
    cudaStreamDestroy(c.copy_stream);
    cudaEventDestroy(c.ev_field);
    cudaStreamDestroy(c.lane_stream);
    cudaEventDestroy(c.ev_lane_fork);
    cudaEventDestroy(c.ev_lane_join);
    for (auto &e : c.chunk_ev) cudaEventDestroy(e);
    c.chunk_ev.clear();
  }
  c.ready = false;
  c.device = -1;
  /* the sizes learnt for unsynchronised frames and the recorded frame go with the buffers */
  c.caps = Ctx::Caps();
  c.caps_known = false;
  drop_graph(c);
  c.graph_key_seen = false;
}

/* ------------------------------------------------------------------ */
/* batched and served forms                                           */
/* ------------------------------------------------------------------ */
/*
 * A server owns `slots` worker threads, each with its own context (stream and
 * device buffers), fed from one FIFO of requests.  A request starts as soon
 * as a slot is free and its estimated device working set fits the HBM budget
 * next to the requests in flight (continuous batching: requests arriving
 * while others run are admitted as slots and memory free up, and their
 * kernels overlap on the device).  The pipeline each request runs is the one
 * of contour3d_gb300_render_device, so a frame's image does not depend on
 * what else is in flight.
 */
namespace c3d {

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  const contour3d_gb300_frame_t *frame = nullptr;
  uint64_t ticket = 0;
  uint64_t estimate = 0;
  double t_submit = 0., t_start = 0., t_done = 0.;
  int rc = 0;
  bool done = false;
  double device_ms = 0.;
  uint64_t held_bytes = 0;
  /* per field of the frame, its codes classified by the batch (or null),
     ready once pre_ev has completed */
  std::vector<unsigned char *> pre_codes;
  cudaEvent_t pre_ev = nullptr;
};

/* the part of a request's working set known before it runs: per slab the
   code arrays, cell offsets and segment sums, and per frame the z-buffer,
   depth floors, winner weights and pixel lists.  The triangle-dependent
   buffers (triangle map and records, screen vertices, candidate lists) are
   sized from the scan's count after each slab's classification and are
   charged against the budget then (ServerHook). */
static uint64_t request_estimate(const contour3d_gb300_frame_t *fr, uint64_t slab_cells) {
  uint64_t peak = 0;
  for (size_t n = 0; n < fr->num_fields; n++) {
    const size_t *sz = fr->fields[n].sizes;
    if (sz[0] < 2 || sz[1] < 2 || sz[2] < 2) continue;
    const uint64_t per_slice = (uint64_t)(sz[0] - 1) * (sz[1] - 1);
    uint64_t cells = std::min<uint64_t>(per_slice * (sz[2] - 1), std::max<uint64_t>(slab_cells, per_slice * 3));
    /* the objects of one field keep one code array each for the slab */
    uint64_t sharing = 0;
    for (size_t q = 0; q < fr->num_fields; q++)
      sharing += fr->fields[q].device_array == fr->fields[n].device_array ? 1 : 0;
    /* codes, triangle offsets (4 bytes), vertex offsets (2 bytes and a
       word per scan segment), look-back state */
    peak = std::max(peak, cells * (sharing + 4 + 2) + cells / 256);
  }
  const uint64_t px = (uint64_t)fr->screen_sizes[0] * fr->screen_sizes[1];
  return peak + px * (sizeof(Slot) + 4 + 48 + 4 + 4 + 3) + (1ULL << 20);
}

}  // namespace c3d

struct contour3d_gb300_server {
  int slots = 0;
  int device = 0;
  uint64_t budget = 0;
  uint64_t resident = 0;
  int running = 0;
  bool stop = false;
  uint64_t next_ticket = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_budget;
  std::deque<c3d::Request *> queue;
  std::unordered_map<uint64_t, c3d::Request *> requests;
  std::vector<std::unique_ptr<c3d::Ctx>> ctxs;
  std::vector<std::unique_ptr<c3d::MemHook>> hooks;
  std::vector<std::thread> threads;
  std::atomic<int> init_failures{0};
  /* device memory of the contexts (under mu): held per slot, in total, and
     whether the slot is rendering a request */
  std::vector<uint64_t> held;
  std::vector<char> busy;
  uint64_t used = 0;
  uint64_t peak_used = 0;
  int blocked = 0;            /* contexts waiting in charge() */
  uint64_t overcommits = 0;   /* charges let through above the budget to keep the server moving */
  uint64_t trims = 0;         /* idle contexts whose buffers were released for another's growth */
};

namespace c3d {

/* bytes the contexts may hold next to the caller's resident fields */
static uint64_t budget_limit(const contour3d_gb300_server *sv) {
  return sv->budget > sv->resident ? sv->budget - sv->resident : 0;
}

/* release every buffer but the constant table of an idle context (its last
   frame has completed: its stream was synchronised); under sv->mu */
static void trim_idle(contour3d_gb300_server *sv, int slot) {
  Ctx &c = *sv->ctxs[slot];
  if (!c.ready) return;
  std::vector<Buf *> bufs = ctx_bufs(c);
  for (size_t q = 1; q < bufs.size(); q++) {
    Buf *b = bufs[q];
    if (!b->p) continue;
    MemHook *h = b->hook;
    b->hook = nullptr; /* credited here, not through the hook (mu is held) */
    sv->used -= b->cap;
    sv->held[slot] -= b->cap;
    b->release(c.own_stream);
    b->hook = h;
  }
  sv->trims++;
}

/*
 * The budget check of a context's buffer growth.  A growth that does not fit
 * first releases the buffers of idle contexts; if it still does not fit, the
 * context waits for running requests to finish or shrink -- unless every
 * other running request is waiting too, in which case it goes ahead above the
 * budget (counted in overcommits), so that waits always end.
 */
struct ServerHook : MemHook {
  contour3d_gb300_server *sv;
  int slot;
  ServerHook(contour3d_gb300_server *s, int q) : sv(s), slot(q) {}
  int charge(size_t bytes) override {
    std::unique_lock<std::mutex> lk(sv->mu);
    const uint64_t limit = budget_limit(sv);
    if (sv->budget != 0) {
      for (;;) {
        if (sv->used + bytes <= limit) break;
        for (int q = 0; q < sv->slots && sv->used + bytes > limit; q++)
          if (q != slot && !sv->busy[q] && sv->held[q] > sv->ctxs[q]->lut.cap) trim_idle(sv, q);
        if (sv->used + bytes <= limit) break;
        if (sv->blocked + 1 >= sv->running) {
          sv->overcommits++;
          break;
        }
        sv->blocked++;
        sv->cv_budget.wait(lk);
        sv->blocked--;
      }
    }
    sv->used += bytes;
    sv->held[slot] += bytes;
    sv->peak_used = std::max(sv->peak_used, sv->used);
    return 0;
  }
  void credit(size_t bytes) override {
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->used -= bytes;
      sv->held[slot] -= bytes;
    }
    sv->cv_budget.notify_all();
  }
};

/* a request starts when a slot is free and its known working set fits next
   to what the running requests hold (an oversized request runs alone) */
static bool admissible(contour3d_gb300_server *sv, const Request *r) {
  if (sv->running == 0) return true;
  if (sv->budget == 0) return true;
  uint64_t busy_held = 0;
  for (int q = 0; q < sv->slots; q++)
    if (sv->busy[q]) busy_held += sv->held[q];
  return busy_held + r->estimate <= budget_limit(sv);
}

static void worker_main(contour3d_gb300_server *sv, int slot) {
  cudaSetDevice(sv->device);
  Ctx &ctx = *sv->ctxs[slot];
  const bool ok = ctx_init(ctx) == 0;
  if (!ok) sv->init_failures++;
  for (;;) {
    Request *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      /* a request that does not fit waits for one in flight to finish (which
         notifies); with nothing in flight every request fits, so no wait is
         endless, also while stopping with requests still queued */
      sv->cv_work.wait(lk, [&] {
        return (sv->stop && sv->queue.empty()) || (!sv->queue.empty() && admissible(sv, sv->queue.front()));
      });
      if (sv->queue.empty()) break; /* stop requested and nothing left */
      r = sv->queue.front();
      sv->queue.pop_front();
      sv->running += 1;
      sv->busy[slot] = 1;
    }
    r->t_start = now_ms();
    int rc = ok ? 0 : 1;
    if (ok) {
      const contour3d_gb300_frame_t *fr = r->frame;
      FrameIn f;
      rc = frame_from_fields(f, &fr->camera_position, &fr->light_direction, fr->screen_sizes, &fr->screen_center,
                             fr->screen_local, &fr->bg_color, fr->num_fields, fr->fields, fr->num_lines, fr->lines);
      if (!rc && (!fr->rgb_out || !is_device_pointer(fr->rgb_out))) {
        log_error("frame output pointer is not device memory");
        rc = 1;
      }
      if (!rc) {
        f.stream = ctx.own_stream;
        if (r->pre_ev && r->pre_codes.size() == f.contours.size()) {
          /* the batch's classification of this frame's fields */
          for (size_t n = 0; n < f.contours.size(); n++) f.contours[n].pre_codes = r->pre_codes[n];
          if (cudaStreamWaitEvent(ctx.own_stream, r->pre_ev, 0) != cudaSuccess) {
            log_error("waiting for the batch's classification failed");
            rc = 1;
          }
        }
      }
      if (!rc) {
        FrameOut out;
        out.rgb_dev = fr->rgb_out;
        rc = render_frame(ctx, f, out);
        r->device_ms = ctx.stats.ms_total;
      }
    }
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      r->rc = rc;
      r->t_done = now_ms();
      r->done = true;
      r->held_bytes = sv->held[slot];
      sv->running -= 1;
      sv->busy[slot] = 0;
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();
    sv->cv_budget.notify_all(); /* one running request fewer: a waiting growth may now go ahead */
  }
  {
    /* the hook is not called once the context is released: credit by hand */
    std::lock_guard<std::mutex> lk(sv->mu);
    for (Buf *b : ctx_bufs(ctx)) b->hook = nullptr;
    sv->used -= sv->held[slot];
    sv->held[slot] = 0;
  }
  ctx_release(ctx);
}

}  // namespace c3d

extern "C" contour3d_gb300_server_t *contour3d_gb300_server_create(int slots, uint64_t hbm_budget_bytes,
                                                                   uint64_t resident_bytes) {
  if (slots < 1 || slots > 64) {
    log_error("server: slots must be in 1..64 (got %d)", slots);
    return nullptr;
  }
  auto *sv = new contour3d_gb300_server();
  sv->slots = slots;
  sv->budget = hbm_budget_bytes;
  sv->resident = resident_bytes;
  if (cudaGetDevice(&sv->device) != cudaSuccess) {
    log_error("server: no current device");
    delete sv;
    return nullptr;
  }
  sv->held.assign((size_t)slots, 0);
  sv->busy.assign((size_t)slots, 0);
  for (int q = 0; q < slots; q++) {
    sv->ctxs.emplace_back(new Ctx());
    sv->hooks.emplace_back(new ServerHook(sv, q));
    for (Buf *b : ctx_bufs(*sv->ctxs[q])) b->hook = sv->hooks[q].get();
  }
  for (int q = 0; q < slots; q++) sv->threads.emplace_back(worker_main, sv, q);
  return sv;
}

static int server_submit(contour3d_gb300_server_t *sv, const contour3d_gb300_frame_t *frame, uint64_t *ticket,
                         const std::vector<unsigned char *> *pre_codes, cudaEvent_t pre_ev) {
  if (!sv || !frame || !ticket) return 1;
  auto *r = new Request();
  r->frame = frame;
  if (pre_codes && pre_ev) {
    r->pre_codes = *pre_codes;
    r->pre_ev = pre_ev;
  }
  r->estimate = request_estimate(frame, kMaxSlabCells);
  r->t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) {
      delete r;
      return 1;
    }
    r->ticket = sv->next_ticket++;
    sv->requests[r->ticket] = r;
    sv->queue.push_back(r);
    *ticket = r->ticket;
  }
  sv->cv_work.notify_all();
  return 0;
}

extern "C" int contour3d_gb300_server_submit(contour3d_gb300_server_t *sv, const contour3d_gb300_frame_t *frame,
                                             uint64_t *ticket) {
  return server_submit(sv, frame, ticket, nullptr, nullptr);
}

extern "C" int contour3d_gb300_server_wait(contour3d_gb300_server_t *sv, uint64_t ticket,
                                           contour3d_gb300_request_stats_t *stats) {
  if (!sv) return 1;
  Request *r = nullptr;
  {
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->requests.find(ticket);
    if (it == sv->requests.end()) {
      log_error("server: unknown ticket %llu", (unsigned long long)ticket);
      return 1;
    }
    r = it->second;
    sv->cv_done.wait(lk, [&] { return r->done; });
    sv->requests.erase(it);
  }
  if (stats) {
    stats->latency_ms = r->t_done - r->t_submit;
    stats->queue_ms = r->t_start - r->t_submit;
    stats->device_ms = r->device_ms;
    stats->estimate_bytes = r->estimate;
    stats->held_bytes = r->held_bytes;
  }
  const int rc = r->rc;
  delete r;
  return rc;
}

extern "C" uint64_t contour3d_gb300_device_bytes(void) { return g_device_bytes.load(); }

extern "C" int contour3d_gb300_server_memory(contour3d_gb300_server_t *sv, contour3d_gb300_server_memory_t *out) {
  if (!sv || !out) return 1;
  std::lock_guard<std::mutex> lk(sv->mu);
  out->used_bytes = sv->used;
  out->peak_bytes = sv->peak_used;
  out->overcommits = sv->overcommits;
  out->trims = sv->trims;
  return 0;
}

extern "C" int contour3d_gb300_server_destroy(contour3d_gb300_server_t *sv) {
  if (!sv) return 1;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto &t : sv->threads) t.join();
  const int rc = sv->init_failures.load() ? 1 : 0;
  for (auto &kv : sv->requests) delete kv.second;
  delete sv;
  return rc;
}

namespace c3d {

static std::atomic<bool> g_batch_classify{true};

/* the batch's classification: one persistent launch over (field, brick) work
   items of every frame whose fields each take one slab */
struct BatchCodes {
  char *arena = nullptr;     /* device: the work counter, then 256-byte aligned code arrays */
  ClsItem *items = nullptr;  /* device: the work items */
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  std::vector<std::vector<unsigned char *>> codes; /* per frame and field */
  int nitems = 0;
  unsigned long long units = 0;
  ~BatchCodes() {
    if (st) cudaStreamSynchronize(st);
    if (items) cudaFree(items);
    if (arena) cudaFree(arena);
    if (ev) cudaEventDestroy(ev);
    if (st) cudaStreamDestroy(st);
  }
};

static int batch_classify(const contour3d_gb300_frame_t *frames, size_t num_frames, BatchCodes &bc) {
  /* objects of one frame that share a field's values, sizes and type are one
     item (up to kMaxThr of them): one pass over that field */
  struct Group {
    size_t frame;
    std::vector<size_t> objs;
    FieldDev F[kMaxThr];
    SlabDev S;
  };
  std::vector<Group> groups;
  std::vector<size_t> code_offs; /* per (group, object), in group order */
  size_t bytes = 256;             /* the work counter */
  const int cls_z = launch_shape().cls_z;
  bc.codes.assign(num_frames, {});
  for (size_t q = 0; q < num_frames; q++) {
    const contour3d_gb300_frame_t *fr = frames + q;
    FrameIn f;
    if (frame_from_fields(f, &fr->camera_position, &fr->light_direction, fr->screen_sizes, &fr->screen_center,
                          fr->screen_local, &fr->bg_color, fr->num_fields, fr->fields, fr->num_lines, fr->lines)) {
      cudaGetLastError();
      continue; /* the worker reports the frame's error */
    }
    bc.codes[q].assign(f.contours.size(), nullptr);
    const size_t first_group = groups.size();
    for (size_t n = 0; n < f.contours.size(); n++) {
      const ContourIn &ci = f.contours[n];
      const long long nx = (long long)ci.sz[0], ny = (long long)ci.sz[1], nz = (long long)ci.sz[2];
      if (nx < 2 || ny < 2 || nz < 4) continue;
      const long long per_slice = (nx - 1) * (ny - 1), ncz = nz - 1;
      /* the slab rule of the slab loop: the whole field in one slab */
      if (3 * per_slice > kMaxSlabCells || kMaxSlabCells / per_slice - 2 < ncz - 2) continue;
      FieldDev F;
      memset(&F, 0, sizeof F);
      F.data = ci.data;
      F.is_f32 = ci.f32 ? 1 : 0;
      F.nx = nx;
      F.ny = ny;
      F.nz = nz;
      F.threshold = ci.threshold;
      F.thr_key = h_key(ci.threshold);
      F.thr_nan = std::isnan(ci.threshold) ? 1 : 0;
      set_float_threshold(F);
      Group *g = nullptr;
      for (size_t k = first_group; k < groups.size(); k++) {
        const FieldDev &G = groups[k].F[0];
        if (G.data == F.data && G.is_f32 == F.is_f32 && G.nx == nx && G.ny == ny && G.nz == nz &&
            groups[k].objs.size() < (size_t)kMaxThr) {
          g = &groups[k];
          break;
        }
      }
      if (!g) {
        groups.push_back(Group());
        g = &groups.back();
        g->frame = q;
        g->S = SlabDev{0, ncz, 1, ncz - 1, cls_z};
      }
      g->F[g->objs.size()] = F;
      g->objs.push_back(n);
    }
  }
  std::vector<ClsItem> items;
  for (Group &g : groups) {
    const long long ncell = (g.F[0].nx - 1) * (g.F[0].ny - 1) * (g.F[0].nz - 1);
    for (size_t t = 0; t < g.objs.size(); t++) {
      code_offs.push_back(bytes);
      bytes += ((size_t)ncell + 255) & ~(size_t)255;
    }
  }
  if (groups.empty()) return 1;
  if (cudaMalloc(&bc.arena, bytes) != cudaSuccess ||
      cudaMalloc(&bc.items, sizeof(ClsItem) * groups.size()) != cudaSuccess) {
    cudaGetLastError();
    log_error("batch classification: device allocation of %zu bytes failed", bytes);
    return 1;
  }
  size_t o = 0;
  for (Group &g : groups) {
    unsigned char *codes[kMaxThr] = {};
    for (size_t t = 0; t < g.objs.size(); t++) {
      codes[t] = reinterpret_cast<unsigned char *>(bc.arena + code_offs[o++]);
      bc.codes[g.frame][g.objs[t]] = codes[t];
    }
    ClsItem it;
    make_cls_item(g.F, (int)g.objs.size(), g.S, codes, &it);
    it.first = bc.units;
    bc.units += (unsigned long long)it.nbx * it.nby * it.nbz;
    items.push_back(it);
  }
  bc.nitems = (int)items.size();
  C3D_CUDA(cudaStreamCreateWithFlags(&bc.st, cudaStreamNonBlocking));
  C3D_CUDA(cudaEventCreateWithFlags(&bc.ev, cudaEventDisableTiming));
  C3D_CUDA(cudaMemcpyAsync(bc.items, items.data(), sizeof(ClsItem) * items.size(), cudaMemcpyHostToDevice, bc.st));
  C3D_CUDA(cudaMemsetAsync(bc.arena, 0, sizeof(unsigned long long), bc.st));
  launch_classify_queue(bc.items, bc.nitems, bc.units, reinterpret_cast<unsigned long long *>(bc.arena), bc.st);
  C3D_CUDA(cudaGetLastError());
  C3D_CUDA(cudaEventRecord(bc.ev, bc.st));
  return 0;
}

}  // namespace c3d

extern "C" int contour3d_gb300_set_batch_classify(int on) {
  g_batch_classify = on != 0;
  return 0;
}

extern "C" int contour3d_gb300_render_batch(const contour3d_gb300_frame_t *frames, size_t num_frames, int workers,
                                            double *frame_ms) {
  if (num_frames && !frames) return 1;
  if (workers < 1) workers = 1;
  contour3d_gb300_server_t *sv = contour3d_gb300_server_create((int)std::min<size_t>((size_t)workers,
                                                                                     std::max<size_t>(num_frames, 1)),
                                                               0, 0);
  if (!sv) return 1;
  /* largest first, so that the last frames of the batch do not run alone */
  std::vector<size_t> order(num_frames);
  std::vector<uint64_t> est(num_frames);
  for (size_t n = 0; n < num_frames; n++) {
    order[n] = n;
    est[n] = request_estimate(frames + n, kMaxSlabCells);
  }
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return est[a] > est[b]; });
  /* every frame's classification first, in one launch; the frames' slab
     passes wait for it on their own streams */
  BatchCodes bc;
  const bool pre = g_batch_classify && num_frames > 0 && batch_classify(frames, num_frames, bc) == 0;
  std::vector<uint64_t> tickets(num_frames);
  int rc = 0;
  for (size_t q = 0; q < num_frames; q++) {
    const size_t n = order[q];
    rc |= server_submit(sv, frames + n, &tickets[n], pre ? &bc.codes[n] : nullptr, pre ? bc.ev : nullptr);
  }
  for (size_t n = 0; n < num_frames; n++) {
    contour3d_gb300_request_stats_t st;
    rc |= contour3d_gb300_server_wait(sv, tickets[n], &st);
    if (frame_ms) frame_ms[n] = st.device_ms;
  }
  rc |= contour3d_gb300_server_destroy(sv);
  return rc ? 1 : 0;
}
