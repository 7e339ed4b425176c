/*
 * c3d_host.h -- host-side helpers shared by runtime.cu and decomp.cpp.
 * Internal to the library.
 */
#pragma once
#include <cstddef>
#include <cstdint>
#include "contour3d.h"

namespace c3d {

/* "[CONTOUR3D ERROR] ..." on stderr, as the reference's logger (logger.c:5-18) */
void log_error(const char *fmt, ...);

/* one contour object's block on this rank */
struct BlockInfo {
  size_t mysize[3], offset[3];        /* pencil-local block */
  int nprocs[3], myrank[3];
  int neighbours[3][2];
  bool single;                        /* one process in every direction */
  size_t ext_size[3], ext_offset[3];  /* extended block (extend.c:239-252) */
  bool clip_lo[3];
};

/* canvas pixel with the layout of the reference's pixel_t (struct.h:31-34) */
struct PixelRec {
  double depth;
  uint8_t r, g, b;
  uint8_t pad[5];
};
static_assert(sizeof(PixelRec) == 16, "pixel record must be 16 bytes");

int decomp_query(const sdecomp_info_t *info, const contour3d_contour_obj_t *obj, BlockInfo *b);
int extend_block(const sdecomp_info_t *info, const contour3d_contour_obj_t *obj, const BlockInfo &b,
                 double *ext);
int comm_size(MPI_Comm comm);
int reduce_nearest(const sdecomp_info_t *info, PixelRec *px, size_t n);
/* the P6 ppm file of a W x H image, rows as given (output.c:113-148) */
int write_ppm(const char *fname, size_t W, size_t H, const uint8_t *rgb);

}  // namespace c3d

/* write_ppm with C linkage, for the host-side tests */
extern "C" int c3d_write_ppm(const char *fname, size_t W, size_t H, const uint8_t *rgb);
