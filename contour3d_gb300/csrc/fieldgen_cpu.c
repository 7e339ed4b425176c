/*
 * Host-side seeded field generators (see fieldgen.h).  Built without
 * floating-point contraction so that the bytes match the device generator
 * in fieldgen.cu and the same generator built on another host.
 *
 * Every function fills the block [off, off + my) of a global grid of
 * gl[0] x gl[1] x gl[2] nodes, x fastest.
 */
#include <stdlib.h>
#include "fieldgen.h"

void c3d_fieldgen_blobs_f64(double *out, const long gl[3], const long off[3],
                            const long my[3], int nblobs, uint64_t seed) {
  c3d_blobs_t b;
  c3d_blobs_init(&b, nblobs, seed);
  size_t q = 0;
  for (long k = 0; k < my[2]; k++) {
    const double z = (double)(k + off[2]) / (double)(gl[2] - 1);
    for (long j = 0; j < my[1]; j++) {
      const double y = (double)(j + off[1]) / (double)(gl[1] - 1);
      for (long i = 0; i < my[0]; i++) {
        const double x = (double)(i + off[0]) / (double)(gl[0] - 1);
        out[q++] = c3d_blobs_value(&b, x, y, z);
      }
    }
  }
}

/* per-mode axis factors: re/im of e^{i 2 pi k x} (z axis includes the phase) */
static int mode_tables(const c3d_modes_t *m, const long gl[3], const long off[3],
                       const long my[3], double **tab) {
  for (int d = 0; d < 3; d++) {
    tab[d] = malloc(sizeof(double) * 2 * (size_t)m->nmodes * (size_t)my[d]);
    if (!tab[d]) return 1;
  }
  for (int n = 0; n < m->nmodes; n++) {
    const int kk[3] = {m->kx[n], m->ky[n], m->kz[n]};
    double pr, pi;
    c3d_sincos_turns(m->phase[n], &pi, &pr);
    for (int d = 0; d < 3; d++) {
      for (long i = 0; i < my[d]; i++) {
        double re, im;
        c3d_mode_axis(kk[d], i + off[d], gl[d], &re, &im);
        if (d == 2) {
          const double r2 = re * pr - im * pi;
          const double i2 = re * pi + im * pr;
          re = r2;
          im = i2;
        }
        tab[d][2 * ((size_t)n * (size_t)my[d] + (size_t)i) + 0] = re;
        tab[d][2 * ((size_t)n * (size_t)my[d] + (size_t)i) + 1] = im;
      }
    }
  }
  return 0;
}

double c3d_fieldgen_modes_f64(double *out, const long gl[3], const long off[3],
                              const long my[3], int nmodes, int kmin, int kmax,
                              double power, uint64_t seed) {
  c3d_modes_t *m = malloc(sizeof(c3d_modes_t));
  double *tab[3] = {0, 0, 0};
  if (!m) return -1.0;
  c3d_modes_init(m, nmodes, kmin, kmax, power, seed);
  const double std = m->std;
  if (!out) { free(m); return std; }
  if (mode_tables(m, gl, off, my, tab)) { free(m); return -1.0; }
  size_t q = 0;
  for (long k = 0; k < my[2]; k++)
    for (long j = 0; j < my[1]; j++)
      for (long i = 0; i < my[0]; i++) {
        double f = 0.0;
        for (int n = 0; n < nmodes; n++) {
          const double *ex = tab[0] + 2 * ((size_t)n * (size_t)my[0] + (size_t)i);
          const double *ey = tab[1] + 2 * ((size_t)n * (size_t)my[1] + (size_t)j);
          const double *ez = tab[2] + 2 * ((size_t)n * (size_t)my[2] + (size_t)k);
          f = f + c3d_mode_term(ex[0], ex[1], ey[0], ey[1], ez[0], ez[1], m->amp[n]);
        }
        out[q++] = f;
      }
  for (int d = 0; d < 3; d++) free(tab[d]);
  free(m);
  return std;
}

/* single-precision Fourier field: tables rounded to float, float accumulation */
double c3d_fieldgen_modes_f32(float *out, const long gl[3], const long off[3],
                              const long my[3], int nmodes, int kmin, int kmax,
                              double power, uint64_t seed) {
  c3d_modes_t *m = malloc(sizeof(c3d_modes_t));
  double *tab[3] = {0, 0, 0};
  if (!m) return -1.0;
  c3d_modes_init(m, nmodes, kmin, kmax, power, seed);
  const double std = m->std;
  if (mode_tables(m, gl, off, my, tab)) { free(m); return -1.0; }
  size_t q = 0;
  for (long k = 0; k < my[2]; k++)
    for (long j = 0; j < my[1]; j++)
      for (long i = 0; i < my[0]; i++) {
        float f = 0.0f;
        for (int n = 0; n < nmodes; n++) {
          const double *ex = tab[0] + 2 * ((size_t)n * (size_t)my[0] + (size_t)i);
          const double *ey = tab[1] + 2 * ((size_t)n * (size_t)my[1] + (size_t)j);
          const double *ez = tab[2] + 2 * ((size_t)n * (size_t)my[2] + (size_t)k);
          const float exr = (float)ex[0], exi = (float)ex[1], eyr = (float)ey[0],
                      eyi = (float)ey[1], ezr = (float)ez[0], ezi = (float)ez[1];
          const float tr = exr * eyr - exi * eyi;
          const float ti = exr * eyi + exi * eyr;
          f = f + (float)m->amp[n] * (tr * ezi + ti * ezr);
        }
        out[q++] = f;
      }
  for (int d = 0; d < 3; d++) free(tab[d]);
  free(m);
  return std;
}

/*
 * A smooth non-identity coordinate map, for exercising the converter path
 * (the reference's example uses the identity, src/main.c:12-21):
 *   x' = x + y z / 8,  y' = y - x^2 / 16,  z' = z + x y / 4
 */
typedef struct {
  double x, y, z;
} c3d_vec_t;

c3d_vec_t c3d_example_warp(const c3d_vec_t p) {
  c3d_vec_t q;
  q.x = p.x + 0.125 * p.y * p.z;
  q.y = p.y - 0.0625 * p.x * p.x;
  q.z = p.z + 0.25 * p.x * p.y;
  return q;
}
