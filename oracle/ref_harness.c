/*
 * Harness around the reference library, compiled from the reference's own
 * sources into oracle/_ref/libc3dref.so (CPU checker only, never shipped).
 *
 * Exports, besides the reference's own contour3d_execute:
 *   c3dref_identity        identity converter (src/main.c:12-21 does the same)
 *   c3dref_warp            a smooth non-identity converter for tests
 *   c3dref_dump_triangles  runs the reference's stage functions for one
 *                          contour object in the order of
 *                          src/contour3d/contour/main.c:49-112 and returns
 *                          every rendered triangle with its vertices, vertex
 *                          normals and cube-edge ids.
 */
#include <stdio.h>
#include <string.h>
#include "contour3d.h"
#include "struct.h"
#include "memory.h"
#include "contour/internal.h"

contour3d_vector_t c3dref_identity(const contour3d_vector_t p) { return p; }

contour3d_vector_t c3dref_warp(const contour3d_vector_t p) {
  contour3d_vector_t q;
  q.x = p.x + 0.125 * p.y * p.z;
  q.y = p.y - 0.0625 * p.x * p.x;
  q.z = p.z + 0.25 * p.x * p.y;
  return q;
}

/* one rendered triangle, flat (25 doubles + 6 int64) */
typedef struct {
  double vertices[9];
  double vertex_normals[9];
  double face_normal[3];
  double area;
  int64_t cell[3];
  int64_t edge_ids[3];
} c3dref_triangle_t;

/*
 * Returns the number of rendered triangles (or -1 on failure); writes at most
 * `capacity` of them.  *num_triangulated receives the count over every
 * triangulated cell (including the outer layer that is never drawn).
 */
long c3dref_dump_triangles(const sdecomp_info_t *info,
                           const contour3d_contour_obj_t *obj,
                           c3dref_triangle_t *out, long capacity,
                           long *num_triangulated) {
  size_t sz[3] = {0}, off[3] = {0};
  double *ext = NULL;
  if (contour3d_contour_extend_domain(info, obj, sz, off, &ext)) return -1;
  const size_t ni = sz[0] - 1, nj = sz[1] - 1;
  lattice_t *ring[3];
  for (int n = 0; n < 3; n++) {
    ring[n] = contour3d_memory_alloc(ni * nj, sizeof(lattice_t));
    if (!ring[n]) return -1;
  }
  long count = 0, tri_all = 0;
  for (size_t k = 0; k + 1 < sz[2]; k++) {
    double *grids[3] = {obj->grids[0] + off[0], obj->grids[1] + off[1],
                        obj->grids[2] + off[2] + k};
    if (contour3d_contour_triangulate_slice((size_t[2]){sz[0], sz[1]}, grids,
                                            obj->converter,
                                            ext + k * sz[0] * sz[1],
                                            obj->threshold, ring[k % 3]))
      return -1;
    for (size_t c = 0; c < ni * nj; c++) tri_all += (long)ring[k % 3][c].num_triangles;
    if (k < 2) continue;
    lattice_t *three[3] = {ring[(k - 2) % 3], ring[(k - 1) % 3], ring[k % 3]};
    if (contour3d_contour_compute_vertex_normals((size_t[2]){sz[0], sz[1]}, three))
      return -1;
    for (size_t j = 1; j + 1 < nj; j++) {
      for (size_t i = 1; i + 1 < ni; i++) {
        const lattice_t *l = three[1] + j * ni + i;
        for (size_t t = 0; t < l->num_triangles; t++, count++) {
          if (count >= capacity) continue;
          const triangle_t *tr = l->triangles + t;
          c3dref_triangle_t *o = out + count;
          for (int m = 0; m < 3; m++) {
            o->vertices[3 * m + 0] = tr->vertices[m].x;
            o->vertices[3 * m + 1] = tr->vertices[m].y;
            o->vertices[3 * m + 2] = tr->vertices[m].z;
            o->vertex_normals[3 * m + 0] = tr->vertex_normals[m].x;
            o->vertex_normals[3 * m + 1] = tr->vertex_normals[m].y;
            o->vertex_normals[3 * m + 2] = tr->vertex_normals[m].z;
            o->edge_ids[m] = (int64_t)tr->cube_indices[m];
          }
          o->face_normal[0] = tr->face_normal.x;
          o->face_normal[1] = tr->face_normal.y;
          o->face_normal[2] = tr->face_normal.z;
          o->area = tr->area;
          o->cell[0] = (int64_t)i;
          o->cell[1] = (int64_t)j;
          o->cell[2] = (int64_t)(k - 1);
        }
      }
    }
  }
  for (int n = 0; n < 3; n++) contour3d_memory_free(ring[n]);
  contour3d_memory_free(ext);
  if (num_triangulated) *num_triangulated = tri_all;
  return count;
}

/* a single-rank decomposition handle for callers of contour3d_execute */
const sdecomp_info_t *c3dref_single_rank(void) {
  sdecomp_info_t *info = NULL;
  sdecomp.construct(0, 3, (size_t[3]){0, 0, 0}, (bool[3]){true, true, true}, &info);
  return info;
}
