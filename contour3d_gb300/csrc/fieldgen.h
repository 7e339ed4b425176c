/*
 * fieldgen.h -- seeded synthetic scalar fields for the isosurface path.
 *
 * The reference's only workload is a field built in its example driver
 * (src/main.c:23-111: superposed sine modes with rand() phases).  The
 * workloads here are seeded stand-ins with the shapes and value
 * distributions of the benchmark configurations:
 *   - Gaussian blobs:   f(x) = sum_b a_b exp(-|x - c_b|^2 / (2 w_b^2))
 *   - Fourier modes:    f(x) = sum_m a_m sin(2 pi k_m . x + phi_m),
 *                       integer wave vectors k_m, a_m = |k_m|^(-p)
 * on the unit cube with uniform nodes x_i = i / (N - 1).
 *
 * Every value is produced by +, -, *, / and sqrt only (the elementary
 * functions below are written out as range reduction + polynomial), and the
 * callers compile without contraction (-ffp-contract=off on the host,
 * -fmad=false on the device).  The same seed therefore gives the same field
 * bytes on x86-64 and aarch64 hosts and on the GPU, which is what lets a
 * field be regenerated anywhere instead of shipped.
 */
#ifndef C3D_FIELDGEN_H
#define C3D_FIELDGEN_H

#include <stdint.h>
#include <stddef.h>
#include <math.h>

#if defined(__CUDACC__)
#define C3D_HD __host__ __device__ __forceinline__
#else
#define C3D_HD static inline
#endif

/* ---- PRNG: splitmix64 (Steele, Lea, Flood 2014) ---- */
C3D_HD uint64_t c3d_splitmix64(uint64_t *state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* uniform double in [0, 1) with 53 random bits */
C3D_HD double c3d_uniform(uint64_t *state) {
  return (double)(c3d_splitmix64(state) >> 11) * (1.0 / 9007199254740992.0);
}

/* 2^n as a double for -1022 <= n <= 1023 */
C3D_HD double c3d_pow2i(int n) {
  union { uint64_t u; double d; } v;
  v.u = (uint64_t)(n + 1023) << 52;
  return v.d;
}

/*
 * exp(x): Cody-Waite reduction x = n ln2 + r, |r| <= ln2/2, then the Taylor
 * series of e^r to degree 15 in Horner form, then scaling by 2^n.
 */
C3D_HD double c3d_exp(double x) {
  if (x < -740.0) return 0.0;
  if (x > 709.0) return 1.0e308 * 10.0;
  const double inv_ln2 = 1.4426950408889634;
  const double ln2_hi = 6.93147180369123816490e-01; /* 32 significant bits */
  const double ln2_lo = 1.90821492927058770002e-10;
  double t = x * inv_ln2;
  int n = (int)(t < 0.0 ? t - 0.5 : t + 0.5);
  double dn = (double)n;
  double r = (x - dn * ln2_hi) - dn * ln2_lo;
  double p = 1.0 / 1307674368000.0; /* 1/15! */
  p = p * r + 1.0 / 87178291200.0;
  p = p * r + 1.0 / 6227020800.0;
  p = p * r + 1.0 / 479001600.0;
  p = p * r + 1.0 / 39916800.0;
  p = p * r + 1.0 / 3628800.0;
  p = p * r + 1.0 / 362880.0;
  p = p * r + 1.0 / 40320.0;
  p = p * r + 1.0 / 5040.0;
  p = p * r + 1.0 / 720.0;
  p = p * r + 1.0 / 120.0;
  p = p * r + 1.0 / 24.0;
  p = p * r + 1.0 / 6.0;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  if (n < -1020) return (p * c3d_pow2i(n + 60)) * c3d_pow2i(-60);
  return p * c3d_pow2i(n);
}

/*
 * log(x) for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)), then
 * log(m) = 2 atanh(s), s = (m - 1) / (m + 1), odd series to s^31.
 */
C3D_HD double c3d_log(double x) {
  union { uint64_t u; double d; } v;
  v.d = x;
  int e = (int)((v.u >> 52) & 0x7FF) - 1023;
  v.u = (v.u & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull; /* m in [1,2) */
  double m = v.d;
  if (m > 1.4142135623730951) { m = m * 0.5; e += 1; }
  double s = (m - 1.0) / (m + 1.0);
  double s2 = s * s;
  double p = 1.0 / 31.0;
  for (int k = 29; k >= 1; k -= 2) p = p * s2 + 1.0 / (double)k;
  return 2.0 * s * p + (double)e * 0.6931471805599453;
}

/*
 * sin and cos of 2*pi*u for u in [0, 1): reflect u to v in [-1/8, 1/8]
 * around the nearest quarter turn, then Taylor series of sin/cos(2 pi v)
 * to degree 19/18.
 */
C3D_HD void c3d_sincos_turns(double u, double *s, double *c) {
  double q = u * 4.0;
  int quad = (int)(q + 0.5);           /* nearest quarter turn 0..4 */
  double v = (q - (double)quad) * 0.25; /* in [-1/8, 1/8] turns */
  double a = v * 6.283185307179586;
  double a2 = a * a;
  double ps = 1.0 / 121645100408832000.0; /* 1/19! */
  ps = ps * a2 - 1.0 / 355687428096000.0;
  ps = ps * a2 + 1.0 / 1307674368000.0;
  ps = ps * a2 - 1.0 / 6227020800.0;
  ps = ps * a2 + 1.0 / 39916800.0;
  ps = ps * a2 - 1.0 / 362880.0;
  ps = ps * a2 + 1.0 / 5040.0;
  ps = ps * a2 - 1.0 / 120.0;
  ps = ps * a2 + 1.0 / 6.0;
  double sv = a - a * a2 * ps;
  double pc = 1.0 / 6402373705728000.0; /* 1/18! */
  pc = pc * a2 - 1.0 / 20922789888000.0;
  pc = pc * a2 + 1.0 / 87178291200.0;
  pc = pc * a2 - 1.0 / 479001600.0;
  pc = pc * a2 + 1.0 / 3628800.0;
  pc = pc * a2 - 1.0 / 40320.0;
  pc = pc * a2 + 1.0 / 720.0;
  pc = pc * a2 - 1.0 / 24.0;
  pc = pc * a2 + 0.5;
  double cv = 1.0 - a2 * pc;
  switch (quad & 3) {
    case 0: *s = sv; *c = cv; break;
    case 1: *s = cv; *c = -sv; break;
    case 2: *s = -sv; *c = -cv; break;
    default: *s = -cv; *c = sv; break;
  }
}

/* ---- Gaussian-blob field ---- */
#define C3D_MAX_BLOBS 64
typedef struct {
  int nblobs;
  double cx[C3D_MAX_BLOBS], cy[C3D_MAX_BLOBS], cz[C3D_MAX_BLOBS];
  double inv2w2[C3D_MAX_BLOBS]; /* 1 / (2 w^2) */
  double amp[C3D_MAX_BLOBS];
} c3d_blobs_t;

/* centres U[0.2,0.8]^3, widths U[0.05,0.15], amplitudes U[0.5,1.0] */
C3D_HD void c3d_blobs_init(c3d_blobs_t *b, int nblobs, uint64_t seed) {
  uint64_t st = seed;
  b->nblobs = nblobs;
  for (int n = 0; n < nblobs; n++) {
    b->cx[n] = 0.2 + 0.6 * c3d_uniform(&st);
    b->cy[n] = 0.2 + 0.6 * c3d_uniform(&st);
    b->cz[n] = 0.2 + 0.6 * c3d_uniform(&st);
    double w = 0.05 + 0.10 * c3d_uniform(&st);
    b->inv2w2[n] = 1.0 / (2.0 * w * w);
    b->amp[n] = 0.5 + 0.5 * c3d_uniform(&st);
  }
}

C3D_HD double c3d_blobs_value(const c3d_blobs_t *b, double x, double y, double z) {
  double f = 0.0;
  for (int n = 0; n < b->nblobs; n++) {
    double dx = x - b->cx[n], dy = y - b->cy[n], dz = z - b->cz[n];
    double r2 = (dx * dx + dy * dy) + dz * dz;
    f = f + b->amp[n] * c3d_exp(-(r2 * b->inv2w2[n]));
  }
  return f;
}

/* ---- Fourier-mode field ---- */
#define C3D_MAX_MODES 256
typedef struct {
  int nmodes;
  int kx[C3D_MAX_MODES], ky[C3D_MAX_MODES], kz[C3D_MAX_MODES];
  double amp[C3D_MAX_MODES];
  double phase[C3D_MAX_MODES]; /* in turns, [0, 1) */
  double std;                  /* sqrt(sum amp^2 / 2) */
} c3d_modes_t;

/*
 * Integer wave vectors drawn uniformly from the ball kmin <= |k| <= kmax,
 * amplitude |k|^(-power), phase uniform in [0, 1) turns.
 */
C3D_HD void c3d_modes_init(c3d_modes_t *m, int nmodes, int kmin, int kmax,
                           double power, uint64_t seed) {
  uint64_t st = seed;
  m->nmodes = nmodes;
  double var = 0.0;
  for (int n = 0; n < nmodes; n++) {
    int kx, ky, kz, k2;
    do {
      kx = (int)(c3d_splitmix64(&st) % (uint64_t)(2 * kmax + 1)) - kmax;
      ky = (int)(c3d_splitmix64(&st) % (uint64_t)(2 * kmax + 1)) - kmax;
      kz = (int)(c3d_splitmix64(&st) % (uint64_t)(2 * kmax + 1)) - kmax;
      k2 = kx * kx + ky * ky + kz * kz;
    } while (k2 < kmin * kmin || k2 > kmax * kmax);
    m->kx[n] = kx; m->ky[n] = ky; m->kz[n] = kz;
    /* |k|^(-p) = exp(-p/2 * log(k2)) */
    m->amp[n] = c3d_exp(-0.5 * power * c3d_log((double)k2));
    m->phase[n] = c3d_uniform(&st);
    var = var + m->amp[n] * m->amp[n];
  }
  m->std = sqrt(var * 0.5);
}

/* e^{i 2 pi k x_i} with x_i = i / (n - 1): reduce k*i mod (n-1) exactly first */
C3D_HD void c3d_mode_axis(int k, long i, long n, double *re, double *im) {
  long d = n - 1;
  long r = ((long)k * i) % d;
  if (r < 0) r += d;
  c3d_sincos_turns((double)r / (double)d, im, re);
}

/*
 * One mode's contribution at node (i, j, k):
 *   a * Im( (ex * ey) * (ez * e^{i phi}) )
 * with complex products written out in a fixed order.
 */
C3D_HD double c3d_mode_term(double exr, double exi, double eyr, double eyi,
                            double ezpr, double ezpi, double a) {
  double tr = exr * eyr - exi * eyi;
  double ti = exr * eyi + exi * eyr;
  return a * (tr * ezpi + ti * ezpr);
}

#endif /* C3D_FIELDGEN_H */
