/*
 * contour3d.h -- drop-in public interface of the GB300 isosurface-to-image path.
 *
 * This header declares the same types and the same single entry point as the
 * Contour3D library's public header (include/contour3d.h:1-88 of the
 * reference), member for member and argument for argument, so that a flow
 * solver compiled against the reference links against libcontour3d_gb300.so
 * unchanged.  Everything here is part of the ABI: do not reorder members.
 *
 * Semantics (reference src/contour3d/main.c:68-146):
 *   - returns 0 on success, 1 on any failure; failures are reported on stderr
 *     with the prefix "[CONTOUR3D ERROR] ";
 *   - collective over all ranks of the decomposition; only rank 0 writes the
 *     binary P6 image `fname`;
 *   - all caller-owned arrays (grids, fields, object arrays) are read-only and
 *     are host pointers; the library owns and frees all of its own memory
 *     (host and device) before returning.
 */
#if !defined(CONTOUR3D_H)
#define CONTOUR3D_H

#include <stddef.h> /* size_t */
#include <stdint.h> /* uint8_t */
#if defined(CONTOUR3D_EXTERNAL_SDECOMP)
#include <sdecomp.h> /* the caller's SimpleDecomp header, found through -I */
#else
#include "sdecomp.h"
#endif

#define CONTOUR3D_NDIMS 3

#if defined(__cplusplus)
extern "C" {
#endif

/* a point or a direction in three dimensions */
typedef struct {
  double x;
  double y;
  double z;
} contour3d_vector_t;

/* 8-bit RGB colour */
typedef struct {
  uint8_t r;
  uint8_t g;
  uint8_t b;
} contour3d_color_t;

/* one iso-surface: a pencil-local scalar field and the level at which it is cut */
typedef struct {
  /* pencil on which `array` is distributed */
  sdecomp_pencil_t pencil;
  /* global number of grid points in x, y, z */
  size_t glsizes[CONTOUR3D_NDIMS];
  /* global rectilinear node coordinates, glsizes[d] values per direction */
  double * grids[CONTOUR3D_NDIMS];
  /* maps a point of the solver's orthogonal coordinates to Cartesian space */
  contour3d_vector_t (* converter) (
      const contour3d_vector_t orthogonal
  );
  /* iso-level: a node is "inside" when threshold < value */
  double threshold;
  /* surface colour before shading */
  contour3d_color_t color;
  /* pencil-local field, x fastest: array[(k * ny + j) * nx + i] */
  double * array;
} contour3d_contour_obj_t;

/* one poly-line overlay, drawn after all iso-surfaces */
typedef struct {
  /* start and end point, in the solver's orthogonal coordinates */
  contour3d_vector_t edges[2];
  /* number of points along the line (>= 2) */
  size_t nitems;
  /* orthogonal -> Cartesian map */
  contour3d_vector_t (* converter) (
      const contour3d_vector_t orthogonal
  );
  /* line colour (not shaded) */
  contour3d_color_t color;
  /* line width in pixels */
  double width;
} contour3d_line_obj_t;

/*
 * Extract, shade and rasterise every iso-surface of `contour3d_contour_objs`,
 * draw every line of `contour3d_line_objs` over them, reduce the per-rank
 * images to rank 0 and write `fname` there.
 * Replaces reference include/contour3d.h:58-86 / src/contour3d/main.c:68-146.
 */
extern int contour3d_execute (
    const sdecomp_info_t * const sdecomp_info,
    const contour3d_vector_t * const camera_position,
    const contour3d_vector_t * const camera_look_at,
    const contour3d_vector_t * const light_direction,
    const size_t screen_sizes[2],
    const contour3d_vector_t * const screen_center,
    const contour3d_vector_t screen_local[2],
    const contour3d_color_t * const bg_color,
    const size_t num_contours,
    const contour3d_contour_obj_t * const contour3d_contour_objs,
    const size_t num_lines,
    const contour3d_line_obj_t * const contour3d_line_objs,
    const char fname[]
);

#if defined(__cplusplus)
}
#endif

#endif /* CONTOUR3D_H */
