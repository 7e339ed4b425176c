/*
 * c3d_common.cuh -- device arithmetic, tables and data layouts shared by the
 * isosurface kernels.
 *
 * Bit-exact parity with the reference rests on two rules kept everywhere in
 * device code:
 *   1. every double operation is an explicit round-to-nearest intrinsic
 *      (__dadd_rn, __dmul_rn, ...), which the compiler never fuses into an
 *      FMA -- the reference is ISO C99 built without contraction;
 *   2. operands are combined in the order the reference writes them
 *      (src/contour3d/vector.c:5-76, project.c:9-67, triangulate.c:40-93,
 *      normal.c:6-43, render.c:38-163).
 * Comparisons of doubles are done on integer keys where that is exact, to keep
 * them off the FP64 pipe (GB300's FP64 rate is ~1/60 of its FP32 rate).
 */
#pragma once
#include <cstdint>

namespace c3d {

/* ------------------------------------------------------------------ */
/* exact double arithmetic                                             */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
/* 1 / a, correctly rounded: the same value as ddiv(1.0, a) */
__device__ __forceinline__ double drcp(double a) { return __drcp_rn(a); }
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }

struct d3 {
  double x, y, z;
};

/* vector.c:5-76 */
__device__ __forceinline__ d3 v_add(d3 a, d3 b) { return {dadd(a.x, b.x), dadd(a.y, b.y), dadd(a.z, b.z)}; }
__device__ __forceinline__ d3 v_sub(d3 a, d3 b) { return {dsub(a.x, b.x), dsub(a.y, b.y), dsub(a.z, b.z)}; }
__device__ __forceinline__ d3 v_mul(double w, d3 a) { return {dmul(w, a.x), dmul(w, a.y), dmul(w, a.z)}; }
__device__ __forceinline__ double v_dot(d3 a, d3 b) {
  return dadd(dadd(dmul(a.x, b.x), dmul(a.y, b.y)), dmul(a.z, b.z));
}
__device__ __forceinline__ d3 v_cross(d3 a, d3 b) {
  return {dsub(dmul(a.y, b.z), dmul(a.z, b.y)), dsub(dmul(a.z, b.x), dmul(a.x, b.z)),
          dsub(dmul(a.x, b.y), dmul(a.y, b.x))};
}
__device__ __forceinline__ d3 v_normalise(d3 a) {
  const double inv = drcp(dsqrt(v_dot(a, a)));
  return {dmul(a.x, inv), dmul(a.y, inv), dmul(a.z, inv)};
}

/* ------------------------------------------------------------------ */
/* integer keys of doubles                                             */
/* ------------------------------------------------------------------ */
/* on the bit pattern b of a double: integer operations only */
__device__ __forceinline__ bool d_isnan_bits(long long b) {
  return (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL;
}
__device__ __forceinline__ long long d_key_bits(long long b) {
  if ((b << 1) == 0) b = 0;
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ bool d_isnan(double x) { return d_isnan_bits(__double_as_longlong(x)); }
/* signed key, monotone in x, equal for -0 and +0 (NaN excluded by callers) */
__device__ __forceinline__ long long d_key(double x) { return d_key_bits(__double_as_longlong(x)); }
/* a double of global memory as its bit pattern, through the read-only path
   (a value test on the bits then stays on the integer pipes; the same test
   on the loaded double issued FP64 instructions) */
__device__ __forceinline__ long long ld_bits(const double* p) {
  return __ldg(reinterpret_cast<const long long*>(p));
}
/* unsigned key for the depth buffer: unsigned order == numeric order */
__device__ __forceinline__ unsigned long long depth_key(double x) {
  long long k = d_key(x);
  return (unsigned long long)k ^ 0x8000000000000000ULL;
}
__host__ __device__ __forceinline__ double depth_from_key(unsigned long long u) {
  long long k = (long long)(u ^ 0x8000000000000000ULL);
  long long b = k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFLL);
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double d;
  __builtin_memcpy(&d, &b, sizeof d);
  return d;
#endif
}
/* |x| < 1e-8 exactly (fabs(NaN) < c is false, and so is this) */
__device__ __forceinline__ bool abs_lt_1e8(double x) {
  return (__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL) < 0x3E45798EE2308C3ALL;
}

/* ------------------------------------------------------------------ */
/* 128-bit depth-buffer slot                                           */
/* ------------------------------------------------------------------ */
/*
 * One pixel of the device z-buffer, 16 bytes:
 *   hi = depth_key(depth)        larger = nearer (reference depth is n . ray)
 *   lo = (order << 24) | rgb     order: position of the fragment's source in
 *                                the reference's drawing sequence
 * Updating to the lexicographic maximum of (hi, lo) reproduces the
 * reference's sequential z-test "dist0 < depth => skip" (render.c:120-125,
 * line.c:109-115), in which the LAST fragment of maximal depth wins.
 */
/*
 * Programmatic dependent launch.  A kernel launched with the programmatic
 * stream serialisation attribute may be scheduled while the kernel before it
 * on the stream is still finishing; pdl_wait() returns once that kernel has
 * completed and its memory is visible, so everything that reads (or
 * overwrites) what earlier work produced comes after it.  pdl_trigger() lets
 * the next kernel be scheduled once every block of this one has started.
 * Both are no-ops for a kernel launched without the attribute.
 */
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
  pdl_trigger();
  pdl_wait();
}

struct __align__(16) Slot {
  unsigned long long lo, hi;
};

__device__ __forceinline__ void cas128(Slot* addr, unsigned long long cmp_lo, unsigned long long cmp_hi,
                                       unsigned long long new_lo, unsigned long long new_hi,
                                       unsigned long long& old_lo, unsigned long long& old_hi) {
  asm volatile(
      "{\n\t.reg .b128 d, b, c;\n\t"
      "mov.b128 b, {%2, %3};\n\t"
      "mov.b128 c, {%4, %5};\n\t"
      "atom.global.cas.b128 d, [%6], b, c;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(old_lo), "=l"(old_hi)
      : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "l"(addr)
      : "memory");
}

/* raise the slot to max(slot, (hi, lo)); true when this call stored (hi, lo).
   A call that gives up after its retry bound sets bit 0 of *err, which the
   host reads after the frame and reports as an error: a fragment is never
   dropped silently */
__device__ __forceinline__ bool slot_max(Slot* s, unsigned long long hi, unsigned long long lo, unsigned* err) {
  unsigned long long cur_lo = 0, cur_hi = 0;
  /* an atomic read: a CAS whose compare value is never present (hi = 0 is
     the key of NaN-space and is never stored) returns the live contents */
  cas128(s, 0ULL, 0ULL, 0ULL, 0ULL, cur_lo, cur_hi);
  /* every failed CAS means another thread stored a larger value: bounded */
  for (int guard = 0; guard < 1 << 20; guard++) {
    if (hi < cur_hi || (hi == cur_hi && lo <= cur_lo)) return false;
    unsigned long long o_lo, o_hi;
    cas128(s, cur_lo, cur_hi, lo, hi, o_lo, o_hi);
    if (o_lo == cur_lo && o_hi == cur_hi) return true;
    cur_lo = o_lo;
    cur_hi = o_hi;
  }
  if (err) atomicOr(err, 1u);
  return false;
}

/* one 16-byte word stored atomically (atom.exch.b128) */
__device__ __forceinline__ void store128_atomic(void* addr, unsigned long long lo, unsigned long long hi) {
  asm volatile(
      "{\n\t.reg .b128 d, b;\n\t"
      "mov.b128 b, {%0, %1};\n\t"
      "atom.global.exch.b128 d, [%2], b;\n\t}"
      :
      : "l"(lo), "l"(hi), "l"(addr)
      : "memory");
}

/* ------------------------------------------------------------------ */
/* scene constants (project.c:9-67; main.c:25-63)                      */
/* ------------------------------------------------------------------ */
struct SceneDev {
  d3 cam, center, lx, ly, normal, light;
  double nc;   /* normal . camera */
  double d;    /* normal . screen centre */
  double lxx;  /* local_x . local_x */
  double lyy;  /* local_y . local_y */
  long long width, height;
  /* single-precision projection constants (k_emit):
     x = f_ax + f_bx (q . lx) / (n . q), y = f_ay + f_by (q . ly) / (n . q) */
  float f_cam[3], f_n[3], f_lx[3], f_ly[3];
  float f_cam_max, f_n1, f_lx1, f_lxm, f_ly1, f_lym;
  float f_ax, f_bx, f_ay, f_by, f_dq;
  float f_light[3]; /* the light direction rounded to float */
  int z_descending; /* the camera looks towards -z: traverse slices top down */
};

/* project.c:9-67; returns false when the point does not reach the screen */
__device__ __forceinline__ bool project(const SceneDev& s, d3 p, d3& q) {
  const d3 ray = v_sub(p, s.cam);
  const double nr = v_dot(s.normal, ray);
  if (-1.e-8 < nr && nr < 1.e-8) return false;
  const double t = ddiv(dsub(s.d, s.nc), nr);
  if (t <= 0. || 1. <= t) return false;
  const d3 delta = {dsub(dadd(s.cam.x, dmul(t, ray.x)), s.center.x),
                    dsub(dadd(s.cam.y, dmul(t, ray.y)), s.center.y),
                    dsub(dadd(s.cam.z, dmul(t, ray.z)), s.center.z)};
  q.x = ddiv(v_dot(delta, s.lx), s.lxx);
  q.y = ddiv(v_dot(delta, s.ly), s.lyy);
  q.z = nr;
  return true;
}

/* render.c:38-46 */
__device__ __forceinline__ double edge_fn(d3 v0, d3 v1, d3 v2) {
  return dsub(dmul(dsub(v2.x, v0.x), dsub(v1.y, v0.y)), dmul(dsub(v2.y, v0.y), dsub(v1.x, v0.x)));
}

/* ------------------------------------------------------------------ */
/* certified single-precision filters                                  */
/* ------------------------------------------------------------------ */
/*
 * The raster decides coverage and visibility with the reference's FP64
 * arithmetic, but only for fragments that a single-precision estimate cannot
 * settle.  Every estimate below carries an error bound, derived from the
 * standard model |fl(a op b) - (a op b)| <= u |a op b| (u = 2^-24 for FP32,
 * 2^-53 for FP64) and widened by a safety factor, that covers the distance
 * between the FP32 value and the value the reference's FP64 code computes.
 * A decision is "certain" only when the whole error interval lies on one
 * side of the reference's threshold; everything else goes to the exact path.
 */
constexpr float kU32 = 5.9604645e-08f; /* 2^-24 */

/* float key: unsigned order == numeric order, -0 == +0 */
__device__ __forceinline__ unsigned f_key(float x) {
  unsigned u = __float_as_uint(x);
  if ((u << 1) == 0) u = 0;
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/*
 * double -> float with integer operations only (the hardware conversion runs
 * on the FP64 pipe): the significand is truncated, so |result - x| <= 2^-23
 * |x| for |x| in the float normal range; smaller magnitudes flush to a
 * signed zero (error < 2^-126), larger ones become infinite, NaN stays NaN.
 * Every bound built on a converted value uses 2u for it.
 */
__device__ __forceinline__ float to_f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FF);
  if (e == 0x7FF) return __int_as_float(((hi & 0xFFFFF) | lo) ? 0x7FC00000 : (int)(sign | 0x7F800000u));
  const int fe = e - 1023 + 127;
  if (fe >= 255) return __int_as_float((int)(sign | 0x7F800000u));
  if (fe <= 0) return __int_as_float((int)sign);
  return __int_as_float((int)(sign | ((unsigned)fe << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29)));
}

/* ------------------------------------------------------------------ */
/* marching-tetrahedra tables                                           */
/* ------------------------------------------------------------------ */
/*
 * A cell's eight node-above bits (bit c set iff threshold < value at cube
 * corner c; corner bit 0 = +x, bit 1 = +y, bit 2 = +z) form its "code".
 * For each code and each triangle rank r inside the cell, TriLut holds the
 * triangle's three vertices as (tail corner, head corner) pairs in winding
 * order and their cube-edge ids (triangulate.c:23-32, 133-276).
 *   bits  0..17 : vertex q: tail corner at 6q, head corner at 6q+3
 *   bits 18..32 : vertex q: edge id (5 bits) at 18+5q
 */
constexpr int kLutEntries = 256 * 12;

}  // namespace c3d
