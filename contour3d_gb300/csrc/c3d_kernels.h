/*
 * c3d_kernels.h -- launch interface between the host runtime (host.cpp) and
 * the device kernels (kernels.cu).  Internal to the library.
 */
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace c3d {

struct Slot;
struct SceneDev;

/* a scalar field on the device: an extended pencil block, x fastest */
struct FieldDev {
  const void* data;
  int is_f32;
  long long nx, ny, nz;     /* extended block sizes (nodes) */
  const double* gx;         /* node coordinates of the block, device */
  const double* gy;
  const double* gz;
  const double* nodes;      /* Cartesian node positions (3 per node) or null = identity */
  double threshold;
  long long thr_key;        /* integer key of the threshold (d_key) */
  int thr_nan;
};

/* one z-slab of cells: slices [kfirst, kfirst + nslices), rendered [krender0, krender1) */
struct SlabDev {
  long long kfirst;
  long long nslices;
  long long krender0;
  long long krender1;
};

/* triangle arrays (structure of arrays, indexed by emission order within a slab) */
struct TriDev {
  double* wn[3];      /* area * face normal */
  unsigned* meta;     /* edge ids (3 x 5 bits) | flags */
  double* proj[9];    /* projected vertices (x, y, depth) x 3 */
  double* vn[9];      /* vertex normals x 3 */
  double* dbg_vert;   /* optional: world vertices, 9 per triangle */
  double* dbg_fn;     /* optional: face normals, 3 per triangle */
  double* dbg_area;   /* optional: areas */
};
constexpr unsigned kMetaRendered = 1u << 15;
constexpr unsigned kMetaCulled = 1u << 16;

/* one line segment, already projected to pixel units on the host */
struct LineSegDev {
  double p0x, p0y, p0z, p1x, p1y, p1z;
  double width;
  unsigned rgb;
  int valid;
};

/* device error flags */
constexpr unsigned kErrScanTimeout = 1u;

int upload_tables(const unsigned char code_count[256], const signed char nb[19][4][4],
                  const unsigned char nb_count[19]);
long long scan_tiles(long long n);

void launch_classify(const FieldDev& F, const SlabDev& S, unsigned char* counts, cudaStream_t st);
void launch_scan(const unsigned char* counts, long long n, unsigned* offsets,
                 unsigned long long* tile_state, unsigned* tile_counter, unsigned long long* total,
                 unsigned* err, cudaStream_t st);
void launch_fill_tri_cell(const unsigned* offsets, long long n, unsigned* tri_cell, cudaStream_t st);
void launch_emit(const FieldDev& F, const SlabDev& S, const SceneDev& scene, const unsigned long long* lut,
                 const unsigned* offsets, const unsigned* tri_cell, const unsigned long long* total,
                 long long tri_bound, const TriDev& tri, cudaStream_t st);
void launch_normals(const FieldDev& F, const SlabDev& S, const unsigned* offsets, const unsigned* tri_cell,
                    const unsigned long long* total, long long tri_bound, const TriDev& tri, cudaStream_t st);
void launch_raster(const SceneDev& scene, const unsigned long long* total, long long tri_bound, const TriDev& tri,
                   const double* xs, const double* ys, Slot* canvas, unsigned long long order_base, unsigned rgb,
                   cudaStream_t st);
void launch_lines(const LineSegDev* segs, int nseg, long long W, long long H, Slot* canvas,
                  unsigned long long order_base, cudaStream_t st);
void launch_canvas_init(Slot* canvas, long long n, unsigned long long hi, unsigned long long lo, cudaStream_t st);
void launch_resolve(const Slot* canvas, long long W, long long H, unsigned char* rgb, double* depth,
                    cudaStream_t st);

}  // namespace c3d
