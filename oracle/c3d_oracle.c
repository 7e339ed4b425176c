/*
 * c3d_oracle.c -- CPU restatement of Contour3D's isosurface-to-image path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the CUDA path is
 * compared with; the product never links, loads or calls it.  It is used by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.
 *
 * Parity pin: this restatement is compared bit-for-bit with the reference
 * library compiled from its own sources (oracle/Makefile target `ref`,
 * oracle/_ref/) and with golden fixtures generated from that build
 * (tests/golden/make_golden.py).  The reference ships no tests or golden
 * vectors of its own.
 *
 * Every floating-point expression keeps the operand order of the reference
 * and is compiled with -ffp-contract=off, because the reference is ISO C99
 * compiled without contraction and bit-exact parity depends on it:
 *   vector ops ........... src/contour3d/vector.c:5-76
 *   screen / light ....... src/contour3d/main.c:25-63
 *   projection ........... src/contour3d/project.c:9-67
 *   marching tetrahedra .. src/contour3d/contour/triangulate.c:23-342
 *   vertex normals ....... src/contour3d/contour/normal.c:6-165
 *   rasterisation ........ src/contour3d/contour/render.c:38-163
 *   slice loop / interior  src/contour3d/contour/main.c:38-112
 *   array extension ...... src/contour3d/contour/extend.c:150-282
 *   line overlay ......... src/contour3d/line.c:26-170
 *   nearest-depth reduce . src/contour3d/output.c:10-30
 *   ppm output ........... src/contour3d/output.c:90-150
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "contour3d.h"

typedef contour3d_vector_t vec3;
typedef contour3d_vector_t (*converter_fn)(const contour3d_vector_t);

/* ---------------- vector algebra (vector.c:5-76) ---------------- */
static inline vec3 v_add(vec3 a, vec3 b) { vec3 c = {a.x + b.x, a.y + b.y, a.z + b.z}; return c; }
static inline vec3 v_sub(vec3 a, vec3 b) { vec3 c = {a.x - b.x, a.y - b.y, a.z - b.z}; return c; }
static inline vec3 v_mul(double w, vec3 a) { vec3 c = {w * a.x, w * a.y, w * a.z}; return c; }
static inline double v_dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline vec3 v_cross(vec3 a, vec3 b) {
  vec3 c = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return c;
}
static inline vec3 v_normalise(vec3 a) {
  const double inv = 1. / sqrt(v_dot(a, a));
  vec3 c = {a.x * inv, a.y * inv, a.z * inv};
  return c;
}

/* ---------------- scene (main.c:13-63) ---------------- */
typedef struct {
  vec3 cam;
  vec3 center, lx, ly, normal;
  size_t width, height;
  vec3 light;
} scene_t;

static scene_t make_scene(const vec3 *cam, const vec3 *light, const size_t sizes[2],
                          const vec3 *center, const vec3 local[2]) {
  scene_t s;
  s.cam = *cam;
  s.light = v_normalise(*light);
  s.center = *center;
  s.lx = local[0];
  s.ly = local[1];
  s.normal = v_normalise(v_cross(s.lx, s.ly));
  s.width = sizes[0];
  s.height = sizes[1];
  return s;
}

/* project.c:9-67: 0 on success, 1 when the point does not reach the screen */
static int project(const scene_t *s, const vec3 *p0, vec3 *p1) {
  const vec3 ray = v_sub(*p0, s->cam);
  const double nc = v_dot(s->normal, s->cam);
  const double nr = v_dot(s->normal, ray);
  const double d = v_dot(s->normal, s->center);
  const double small = 1.e-8;
  if (-small < nr && nr < small) return 1;
  const double t = (d - nc) / nr;
  if (t <= 0. || 1. <= t) return 1;
  const vec3 delta = {
    s->cam.x + t * ray.x - s->center.x,
    s->cam.y + t * ray.y - s->center.y,
    s->cam.z + t * ray.z - s->center.z,
  };
  p1->x = v_dot(delta, s->lx) / v_dot(s->lx, s->lx);
  p1->y = v_dot(delta, s->ly) / v_dot(s->ly, s->ly);
  p1->z = nr;
  return 0;
}

/* canvas pixel: depth (larger is nearer) and colour (struct.h:31-34) */
typedef struct {
  double depth;
  contour3d_color_t color;
} pixel_t;

/* ---------------- marching tetrahedra (triangulate.c) ---------------- */

/* cube corners of the six tetrahedra around the 0-7 diagonal */
static const int TET[6][4] = {
  {0, 7, 3, 1}, {0, 7, 1, 5}, {0, 7, 5, 4}, {0, 7, 4, 6}, {0, 7, 6, 2}, {0, 7, 2, 3},
};

/*
 * Cube-edge id of the segment between two cube corners (corner bit 0 = x,
 * bit 1 = y, bit 2 = z): 0-3 x edges, 4-7 y edges, 8-11 z edges, 12-13 the
 * diagonals of the x faces, 14-15 of the y faces, 16-17 of the z faces,
 * 18 the 0-7 body diagonal.
 */
static int edge_id(int a, int b) {
  if (a > b) { int t = a; a = b; b = t; }
  const int d = a ^ b;
  switch (d) {
    case 1: return (a >> 1);              /* x edge at (y, z) = bits 1, 2 */
    case 2: return 4 + ((a & 1) | ((a >> 2) << 1));  /* y edge at (x, z) */
    case 4: return 8 + (a & 3);           /* z edge at (x, y) */
    case 6: return 12 + (a & 1);          /* y-z diagonal on the x face */
    case 5: return 14 + ((a >> 1) & 1);   /* x-z diagonal on the y face */
    case 3: return 16 + (a >> 2);         /* x-y diagonal on the z face */
    case 7: return 18;
    default: return 255;
  }
}

/*
 * Triangles per folded tetrahedron mask (1..7), as (tail, head) pairs of
 * tetrahedron-local vertices, in emission and winding order
 * (triangulate.c:204-270).
 */
static const int NTRI[8] = {0, 1, 1, 2, 1, 2, 2, 1};
static const int TRI_EDGES[8][2][3][2] = {
  {{{0}}},
  {{{0, 1}, {0, 3}, {0, 2}}},
  {{{1, 0}, {1, 2}, {1, 3}}},
  {{{0, 2}, {1, 3}, {0, 3}}, {{0, 2}, {1, 2}, {1, 3}}},
  {{{2, 0}, {2, 3}, {2, 1}}},
  {{{2, 1}, {0, 3}, {2, 3}}, {{2, 1}, {0, 1}, {0, 3}}},
  {{{0, 2}, {2, 3}, {1, 3}}, {{0, 2}, {1, 3}, {0, 1}}},
  {{{3, 0}, {3, 2}, {3, 1}}},
};

typedef struct {
  vec3 v[3];      /* vertices */
  vec3 fn;        /* face normal */
  double area;
  vec3 vn[3];     /* vertex normals */
  uint8_t e[3];   /* cube-edge id of each vertex */
} tri_t;

/* triangulate.c:40-73 */
static inline vec3 interpolate(double vt, vec3 p0, double v0, vec3 p1, double v1) {
  if (fabs(v1 - v0) < 1.e-8) return p0;
  const double f = (vt - v0) / (v1 - v0);
  return v_add(p0, v_mul(f, v_sub(p1, p0)));
}

/* triangulate.c:75-93 */
static inline void face_normal(tri_t *t) {
  t->fn = v_cross(v_sub(t->v[1], t->v[0]), v_sub(t->v[2], t->v[0]));
  t->area = sqrt(v_dot(t->fn, t->fn));
  t->fn = v_mul(1. / t->area, t->fn);
}

/*
 * All triangles of one cell, appended to `out` (at most 12).
 * pos[c], val[c]: Cartesian position and value of cube corner c.
 */
static int triangulate_cell(const vec3 pos[8], const double val[8], double thr, tri_t *out) {
  int n = 0;
  for (int t = 0; t < 6; t++) {
    int mask = 0;
    for (int m = 0; m < 4; m++) mask |= (thr < val[TET[t][m]]) << m;
    const int reverse = mask >= 8;
    if (reverse) mask = 15 - mask;
    for (int s = 0; s < NTRI[mask]; s++) {
      tri_t *tr = out + n++;
      for (int q = 0; q < 3; q++) {
        const int src = reverse ? 2 - q : q;
        const int a = TET[t][TRI_EDGES[mask][s][src][0]];
        const int b = TET[t][TRI_EDGES[mask][s][src][1]];
        tr->v[q] = interpolate(thr, pos[a], val[a], pos[b], val[b]);
        tr->e[q] = (uint8_t)edge_id(a, b);
      }
      face_normal(tr);
    }
  }
  return n;
}

/* number of triangles of a cell from its eight corner values */
int c3d_oracle_cell_count(const double val[8], double thr) {
  int n = 0;
  for (int t = 0; t < 6; t++) {
    int mask = 0;
    for (int m = 0; m < 4; m++) mask |= (thr < val[TET[t][m]]) << m;
    if (mask >= 8) mask = 15 - mask;
    n += NTRI[mask];
  }
  return n;
}

/* ---------------- vertex normals (normal.c:46-165) ---------------- */

/* neighbour cells sharing each cube edge: (dk, dj, di, their local edge id) */
static const int NB_COUNT[19] = {4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 2, 2, 2, 2, 2, 2, 1};
static const int NB[19][4][4] = {
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

/* one z-slice of triangulated cells: triangles of cell c are [start[c], start[c+1]) */
typedef struct {
  size_t ncells;
  size_t *start;
  tri_t *tris;
  size_t cap;
} slice_t;

static int slice_reserve(slice_t *s, size_t ncells) {
  s->ncells = ncells;
  s->start = malloc((ncells + 1) * sizeof(size_t));
  s->cap = ncells > 64 ? ncells : 64;
  s->tris = malloc(s->cap * sizeof(tri_t));
  return s->start && s->tris ? 0 : 1;
}

static void slice_free(slice_t *s) {
  free(s->start);
  free(s->tris);
}

/* ---------------- one contour object on one (emulated) rank ---------------- */

typedef struct {
  size_t sz[3];        /* extended local sizes */
  size_t off[3];       /* global offset of the extended block */
  const double *ext;   /* extended block, x fastest */
} block_t;

static vec3 corner_position(const contour3d_contour_obj_t *obj, converter_fn conv,
                            const block_t *b, size_t i, size_t j, size_t k) {
  vec3 c = {obj->grids[0][b->off[0] + i], obj->grids[1][b->off[1] + j],
            obj->grids[2][b->off[2] + k]};
  return conv ? conv(c) : c;
}

static int triangulate_slice(const contour3d_contour_obj_t *obj, converter_fn conv,
                             const block_t *b, size_t k, slice_t *s) {
  const size_t ni = b->sz[0] - 1, nj = b->sz[1] - 1;
  size_t n = 0;
  for (size_t j = 0; j < nj; j++) {
    for (size_t i = 0; i < ni; i++) {
      s->start[j * ni + i] = n;
      if (n + 12 > s->cap) {
        size_t cap = s->cap * 2;
        tri_t *t = realloc(s->tris, cap * sizeof(tri_t));
        if (!t) return 1;
        s->tris = t;
        s->cap = cap;
      }
      double val[8];
      vec3 pos[8];
      for (int c = 0; c < 8; c++) {
        const size_t ii = i + (c & 1), jj = j + ((c >> 1) & 1), kk = k + (c >> 2);
        val[c] = b->ext[(kk * b->sz[1] + jj) * b->sz[0] + ii];
        pos[c] = corner_position(obj, conv, b, ii, jj, kk);
      }
      n += (size_t)triangulate_cell(pos, val, obj->threshold, s->tris + n);
    }
  }
  s->start[ni * nj] = n;
  return 0;
}

/* normal.c:6-43 + :59-160 for the interior cells of the middle slice */
static void vertex_normals(size_t ni, size_t nj, slice_t *sl[3]) {
  for (size_t j = 1; j + 1 < nj; j++) {
    for (size_t i = 1; i + 1 < ni; i++) {
      slice_t *mid = sl[1];
      for (size_t t = mid->start[j * ni + i]; t < mid->start[j * ni + i + 1]; t++) {
        tri_t *tr = mid->tris + t;
        for (int m = 0; m < 3; m++) {
          const int e = tr->e[m];
          vec3 sum = {0., 0., 0.};
          for (int q = 0; q < NB_COUNT[e]; q++) {
            const slice_t *ns = sl[1 + NB[e][q][0]];
            const size_t c = (size_t)((long)j + NB[e][q][1]) * ni + (size_t)((long)i + NB[e][q][2]);
            const int le = NB[e][q][3];
            for (size_t u = ns->start[c]; u < ns->start[c + 1]; u++) {
              const tri_t *o = ns->tris + u;
              if (o->e[0] == le || o->e[1] == le || o->e[2] == le)
                sum = v_add(sum, v_mul(o->area, o->fn));
            }
          }
          tr->vn[m] = v_normalise(sum);
        }
      }
    }
  }
}

static inline long lmin(long a, long b) { return a < b ? a : b; }
static inline long lmax(long a, long b) { return b < a ? a : b; }
static inline double edge_fn(const vec3 *v0, const vec3 *v1, const vec3 *v2) {
  return (v2->x - v0->x) * (v1->y - v0->y) - (v2->y - v0->y) * (v1->x - v0->x);
}

/* render.c:48-163 */
static void render_triangle(const scene_t *s, const contour3d_color_t *col,
                            const tri_t *tr, pixel_t *canvas) {
  const size_t W = s->width, H = s->height;
  vec3 p[3];
  for (int d = 0; d < 3; d++)
    if (project(s, tr->v + d, p + d)) return;
  const vec3 *v0 = p + 0, *v1 = p + 1, *v2 = p + 2;
  const long xmin = (long)((0.5 + fmin(v0->x, fmin(v1->x, v2->x))) * W - 1);
  const long xmax = (long)((0.5 + fmax(v0->x, fmax(v1->x, v2->x))) * W + 1);
  const long ymin = (long)((0.5 + fmin(v0->y, fmin(v1->y, v2->y))) * H - 1);
  const long ymax = (long)((0.5 + fmax(v0->y, fmax(v1->y, v2->y))) * H + 1);
  const size_t imin = (size_t)lmin((long)W - 1, lmax(0, xmin));
  const size_t imax = (size_t)lmin((long)W - 1, lmax(0, xmax));
  const size_t jmin = (size_t)lmin((long)H - 1, lmax(0, ymin));
  const size_t jmax = (size_t)lmin((long)H - 1, lmax(0, ymax));
  const double area = edge_fn(v0, v1, v2);
  const double area_inv = 1. / (area < 0. ? fmin(area, -1.e-16) : fmax(area, +1.e-16));
  for (size_t j = jmin; j <= jmax; j++) {
    for (size_t i = imin; i <= imax; i++) {
      const vec3 v3 = {1. * (i + 0.5) / W - 0.5, 1. * (j + 0.5) / H - 0.5, 0.};
      const double w0 = area_inv * edge_fn(v1, v2, &v3);
      const double w1 = area_inv * edge_fn(v2, v0, &v3);
      const double w2 = area_inv * edge_fn(v0, v1, &v3);
      const double small = -1.e-8;
      if (w0 < small || w1 < small || w2 < small) continue;
      pixel_t *px = canvas + j * W + i;
      const double dist0 = 1. / (w0 / v0->z + w1 / v1->z + w2 / v2->z);
      if (dist0 < px->depth) continue;
      px->depth = dist0;
      const vec3 n = v_normalise(
          v_add(v_mul(w0, tr->vn[0]), v_add(v_mul(w1, tr->vn[1]), v_mul(w2, tr->vn[2]))));
      const double factor = fmax(0.15, fabs(v_dot(n, s->light)));
      px->color.r = (uint8_t)(factor * col->r);
      px->color.g = (uint8_t)(factor * col->g);
      px->color.b = (uint8_t)(factor * col->b);
    }
  }
}

/* optional per-triangle record sink, used by the parity tests */
typedef struct {
  double vertices[9];
  double vertex_normals[9];
  double face_normal[3];
  double area;
  int64_t cell[3];
  int64_t edge_ids[3];
} c3d_oracle_triangle_t;

typedef struct {
  c3d_oracle_triangle_t *out;
  long capacity;
  long count;        /* rendered triangles seen */
  long triangulated; /* triangles over every triangulated cell */
} sink_t;

/*
 * contour/main.c:11-119 for one block: triangulate every slice, and once
 * three slices exist, smooth and render the interior cells of the middle one.
 */
static int process_block(const scene_t *s, const contour3d_contour_obj_t *obj,
                         converter_fn conv, const block_t *b, pixel_t *canvas,
                         sink_t *sink) {
  if (b->sz[0] < 2 || b->sz[1] < 2 || b->sz[2] < 2) return 0;
  const size_t ni = b->sz[0] - 1, nj = b->sz[1] - 1;
  slice_t ring[3];
  for (int n = 0; n < 3; n++)
    if (slice_reserve(ring + n, ni * nj)) return 1;
  int rc = 0;
  for (size_t k = 0; k + 1 < b->sz[2]; k++) {
    if (triangulate_slice(obj, conv, b, k, ring + k % 3)) { rc = 1; break; }
    if (sink) sink->triangulated += (long)ring[k % 3].start[ni * nj];
    if (k < 2) continue;
    slice_t *three[3] = {ring + (k - 2) % 3, ring + (k - 1) % 3, ring + k % 3};
    vertex_normals(ni, nj, three);
    for (size_t j = 1; j + 1 < nj; j++) {
      for (size_t i = 1; i + 1 < ni; i++) {
        const slice_t *mid = three[1];
        for (size_t t = mid->start[j * ni + i]; t < mid->start[j * ni + i + 1]; t++) {
          const tri_t *tr = mid->tris + t;
          if (canvas) render_triangle(s, &obj->color, tr, canvas);
          if (sink) {
            if (sink->count < sink->capacity && sink->out) {
              c3d_oracle_triangle_t *o = sink->out + sink->count;
              for (int m = 0; m < 3; m++) {
                o->vertices[3 * m + 0] = tr->v[m].x;
                o->vertices[3 * m + 1] = tr->v[m].y;
                o->vertices[3 * m + 2] = tr->v[m].z;
                o->vertex_normals[3 * m + 0] = tr->vn[m].x;
                o->vertex_normals[3 * m + 1] = tr->vn[m].y;
                o->vertex_normals[3 * m + 2] = tr->vn[m].z;
                o->edge_ids[m] = tr->e[m];
              }
              o->face_normal[0] = tr->fn.x;
              o->face_normal[1] = tr->fn.y;
              o->face_normal[2] = tr->fn.z;
              o->area = tr->area;
              o->cell[0] = (int64_t)(b->off[0] + i);
              o->cell[1] = (int64_t)(b->off[1] + j);
              o->cell[2] = (int64_t)(b->off[2] + k - 1);
            }
            sink->count++;
          }
        }
      }
    }
  }
  for (int n = 0; n < 3; n++) slice_free(ring + n);
  return rc;
}

/* ---------------- lines (line.c:26-170) ---------------- */
static int draw_segment(const scene_t *s, converter_fn conv, const contour3d_color_t *col,
                        double lw, const vec3 *a, const vec3 *b, pixel_t *canvas) {
  const vec3 pa = conv(*a), pb = conv(*b);
  vec3 p0 = {0., 0., 0.}, p1 = {0., 0., 0.};
  if (project(s, &pa, &p0)) return 1;
  if (project(s, &pb, &p1)) return 1;
  const size_t W = s->width, H = s->height;
  p0.x = (0.5 + p0.x) * W;
  p0.y = (0.5 + p0.y) * H;
  p1.x = (0.5 + p1.x) * W;
  p1.y = (0.5 + p1.y) * H;
  const long xmin = (long)(fmin(p0.x, p1.x) - 1);
  const long xmax = (long)(fmax(p0.x, p1.x) + 1);
  const long ymin = (long)(fmin(p0.y, p1.y) - 1);
  const long ymax = (long)(fmax(p0.y, p1.y) + 1);
  const size_t imin = (size_t)lmin((long)W - 1, lmax(0, xmin));
  const size_t imax = (size_t)lmin((long)W - 1, lmax(0, xmax));
  const size_t jmin = (size_t)lmin((long)H - 1, lmax(0, ymin));
  const size_t jmax = (size_t)lmin((long)H - 1, lmax(0, ymax));
  const double la = +p1.y - p0.y;
  const double lb = -p1.x + p0.x;
  const double lc = +(p1.x - p0.x) * p0.y - (p1.y - p0.y) * p0.x;
  for (size_t j = jmin; j <= jmax; j++) {
    for (size_t i = imin; i <= imax; i++) {
      const double h = 0.5 * lw;
      const double threshold = h * h;
      const double num = la * i + lb * j + lc;
      const double distance = num * num / (la * la + lb * lb);
      if (threshold < distance) continue;
      const double dx = p1.x - p0.x, dy = p1.y - p0.y;
      const double param = -1. * ((p1.x - p0.x) * (p0.x - i) + (p1.y - p0.y) * (p0.y - j)) /
                           (dx * dx + dy * dy);
      const double dist0 = 1. / (param / p1.z + (1. - param) / p0.z);
      pixel_t *px = canvas + j * W + i;
      if (dist0 < px->depth) continue;
      px->color = *col;
      px->depth = dist0;
    }
  }
  return 0;
}

static int draw_line(const scene_t *s, const contour3d_line_obj_t *l, pixel_t *canvas) {
  const size_t np = l->nitems;
  if (np < 2) {
    fprintf(stderr, "[CONTOUR3D ERROR] give more than two points to draw a line, received %zu\n", np);
    return 1;
  }
  const vec3 *heads = l->edges + 0, *tails = l->edges + 1;
  const vec3 deltas = v_mul(1. / (np - 1), v_sub(*tails, *heads));
  for (size_t n = 0; n < np - 1; n++) {
    const vec3 a = v_add(*heads, v_mul(n + 0, deltas));
    const vec3 b = v_add(*heads, v_mul(n + 1, deltas));
    draw_segment(s, l->converter, &l->color, l->width, &a, &b, canvas);
  }
  return 0;
}

/* ---------------- emulated z-split ranks ---------------- */

/* balanced split of n points over p parts (own choice; results do not depend on it) */
static void split(size_t n, int p, int r, size_t *my, size_t *off) {
  const size_t base = n / (size_t)p, rem = n % (size_t)p;
  *my = base + ((size_t)r < rem ? 1 : 0);
  *off = (size_t)r * base + ((size_t)r < rem ? (size_t)r : rem);
}

/*
 * extend.c:150-282 for a z-only split into `nranks` blocks: the block of rank
 * r is widened by two layers towards every neighbouring rank and clipped at
 * the global boundary, exactly as the halo exchange + clipping produces it.
 */
static block_t rank_block(const contour3d_contour_obj_t *obj, int nranks, int r) {
  block_t b;
  size_t my, off;
  split(obj->glsizes[2], nranks, r, &my, &off);
  const size_t lo = r > 0 ? 2 : 0, hi = r < nranks - 1 ? 2 : 0;
  b.sz[0] = obj->glsizes[0];
  b.sz[1] = obj->glsizes[1];
  b.sz[2] = my + lo + hi;
  b.off[0] = 0;
  b.off[1] = 0;
  b.off[2] = off - lo;
  b.ext = obj->array + b.off[2] * obj->glsizes[0] * obj->glsizes[1];
  return b;
}

typedef struct {
  const scene_t *s;
  const contour3d_contour_obj_t *objs;
  size_t nobjs;
  const contour3d_line_obj_t *lines;
  size_t nlines;
  int nranks, rank;
  pixel_t *canvas;
  contour3d_color_t bg;
  int rc;
} rank_job_t;

static void canvas_init(pixel_t *c, size_t n, contour3d_color_t bg) {
  for (size_t p = 0; p < n; p++) {
    c[p].color = bg;
    c[p].depth = -1. * DBL_MAX;
  }
}

static void *rank_main(void *arg) {
  rank_job_t *job = arg;
  const size_t npx = job->s->width * job->s->height;
  canvas_init(job->canvas, npx, job->bg);
  job->rc = 0;
  for (size_t n = 0; n < job->nobjs && !job->rc; n++) {
    const contour3d_contour_obj_t *o = job->objs + n;
    const block_t b = rank_block(o, job->nranks, job->rank);
    job->rc = process_block(job->s, o, o->converter, &b, job->canvas, NULL);
  }
  for (size_t n = 0; n < job->nlines && !job->rc; n++)
    job->rc = draw_line(job->s, job->lines + n, job->canvas);
  return NULL;
}

/* output.c:10-30: keep the nearer pixel (larger depth) */
static void reduce_nearest(const pixel_t *in, pixel_t *inout, size_t n) {
  for (size_t p = 0; p < n; p++)
    if (inout[p].depth < in[p].depth) inout[p] = in[p];
}

/*
 * Render into an RGB image laid out as the ppm body (rows flipped,
 * output.c:113-123) and, when depth_out is given, the final depth buffer in
 * canvas order.  `nranks` > 1 emulates that many MPI ranks along z, one
 * thread each, reduced in rank order.  Returns 0 or 1 like contour3d_execute.
 */
int c3d_oracle_render(const contour3d_vector_t *camera_position,
                      const contour3d_vector_t *light_direction,
                      const size_t screen_sizes[2],
                      const contour3d_vector_t *screen_center,
                      const contour3d_vector_t screen_local[2],
                      const contour3d_color_t *bg_color, size_t num_contours,
                      const contour3d_contour_obj_t *objs, size_t num_lines,
                      const contour3d_line_obj_t *lines, int nranks,
                      uint8_t *rgb_out, double *depth_out) {
  const scene_t s = make_scene(camera_position, light_direction, screen_sizes,
                               screen_center, screen_local);
  const size_t W = s.width, H = s.height, npx = W * H;
  if (nranks < 1) nranks = 1;
  pixel_t **canvases = calloc((size_t)nranks, sizeof(pixel_t *));
  rank_job_t *jobs = calloc((size_t)nranks, sizeof(rank_job_t));
  pthread_t *th = calloc((size_t)nranks, sizeof(pthread_t));
  int rc = 0;
  if (!canvases || !jobs || !th) rc = 1;
  for (int r = 0; r < nranks && !rc; r++) {
    canvases[r] = malloc(npx * sizeof(pixel_t));
    if (!canvases[r]) { rc = 1; break; }
    rank_job_t j = {&s, objs, num_contours, lines, num_lines, nranks, r, canvases[r], *bg_color, 0};
    jobs[r] = j;
  }
  if (!rc) {
    if (nranks == 1) {
      rank_main(jobs);
    } else {
      for (int r = 0; r < nranks; r++) pthread_create(th + r, NULL, rank_main, jobs + r);
      for (int r = 0; r < nranks; r++) pthread_join(th[r], NULL);
    }
    for (int r = 0; r < nranks; r++) rc |= jobs[r].rc;
  }
  if (!rc) {
    for (int r = 1; r < nranks; r++) reduce_nearest(canvases[r], canvases[0], npx);
    const pixel_t *c = canvases[0];
    if (rgb_out) {
      size_t q = 0;
      for (size_t j = 0; j < H; j++) {
        for (size_t i = 0; i < W; i++) {
          const pixel_t *px = c + (H - j - 1) * W + i;
          rgb_out[q++] = px->color.r;
          rgb_out[q++] = px->color.g;
          rgb_out[q++] = px->color.b;
        }
      }
    }
    if (depth_out)
      for (size_t p = 0; p < npx; p++) depth_out[p] = c[p].depth;
  }
  for (int r = 0; r < nranks && canvases; r++) free(canvases[r]);
  free(canvases);
  free(jobs);
  free(th);
  return rc;
}

/* contour3d_execute with the same arguments (single rank) writing the ppm */
int c3d_oracle_execute(const void *unused_sdecomp_info,
                       const contour3d_vector_t *camera_position,
                       const contour3d_vector_t *camera_look_at,
                       const contour3d_vector_t *light_direction,
                       const size_t screen_sizes[2],
                       const contour3d_vector_t *screen_center,
                       const contour3d_vector_t screen_local[2],
                       const contour3d_color_t *bg_color, size_t num_contours,
                       const contour3d_contour_obj_t *objs, size_t num_lines,
                       const contour3d_line_obj_t *lines, const char fname[]) {
  (void)unused_sdecomp_info;
  (void)camera_look_at;
  const size_t W = screen_sizes[0], H = screen_sizes[1];
  uint8_t *rgb = malloc(W * H * 3);
  if (!rgb) return 1;
  int rc = c3d_oracle_render(camera_position, light_direction, screen_sizes, screen_center,
                             screen_local, bg_color, num_contours, objs, num_lines, lines,
                             1, rgb, NULL);
  if (!rc) {
    FILE *fp = fopen(fname, "w");
    if (!fp) {
      rc = 1;
    } else {
      fprintf(fp, "P6\n%zu %zu\n255\n", W, H);
      if (fwrite(rgb, 3, W * H, fp) != W * H) rc = 1;
      fclose(fp);
    }
  }
  free(rgb);
  return rc;
}

/*
 * Every rendered triangle of one contour object (single rank) in render
 * order.  Returns the rendered count (writes at most `capacity`), or -1.
 * *num_triangulated receives the count over all triangulated cells.
 */
long c3d_oracle_triangles(const contour3d_contour_obj_t *obj, c3d_oracle_triangle_t *out,
                          long capacity, long *num_triangulated) {
  const block_t b = rank_block(obj, 1, 0);
  sink_t sink = {out, capacity, 0, 0};
  const vec3 z = {0., 0., 0.};
  const vec3 loc[2] = {{1., 0., 0.}, {0., 1., 0.}};
  const size_t sizes[2] = {1, 1};
  const scene_t s = make_scene(&z, &loc[0], sizes, &z, loc);
  if (process_block(&s, obj, obj->converter, &b, NULL, &sink)) return -1;
  if (num_triangulated) *num_triangulated = sink.triangulated;
  return sink.count;
}

/*
 * Per-cell triangle counts over the whole triangulated set (cells
 * (nx-1)(ny-1)(nz-1), x fastest), single rank; returns the total.
 */
long c3d_oracle_cell_counts(const double *array, const size_t glsizes[3], double thr,
                            uint8_t *counts) {
  const size_t nx = glsizes[0], ny = glsizes[1], nz = glsizes[2];
  long total = 0;
  size_t c = 0;
  for (size_t k = 0; k + 1 < nz; k++)
    for (size_t j = 0; j + 1 < ny; j++)
      for (size_t i = 0; i + 1 < nx; i++, c++) {
        double v[8];
        for (int q = 0; q < 8; q++)
          v[q] = array[((k + (q >> 2)) * ny + j + ((q >> 1) & 1)) * nx + i + (q & 1)];
        const int n = c3d_oracle_cell_count(v, thr);
        if (counts) counts[c] = (uint8_t)n;
        total += n;
      }
  return total;
}

contour3d_vector_t c3d_oracle_identity(const contour3d_vector_t p) { return p; }

/* the same smooth non-identity map as oracle/ref_harness.c's c3dref_warp */
contour3d_vector_t c3d_oracle_warp(const contour3d_vector_t p) {
  contour3d_vector_t q;
  q.x = p.x + 0.125 * p.y * p.z;
  q.y = p.y - 0.0625 * p.x * p.x;
  q.z = p.z + 0.25 * p.x * p.y;
  return q;
}
