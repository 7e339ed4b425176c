/*
 * c3d_kernels.h -- launch interface between the host runtime (runtime.cu) and
 * the device kernels (kernels.cu).  Internal to the library.
 */
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace c3d {

struct Slot;
struct SceneDev;
struct RasterDev;

/*
 * Unsigned division by an invariant d >= 1 (Granlund and Montgomery, 1994):
 * with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1,
 * n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0), t = mulhi(m, n),
 * for every 32-bit n.
 */
struct FastDiv {
  unsigned m, s1, s2;
};

/* a scalar field on the device: an extended pencil block, x fastest */
struct FieldDev {
  const void* data;
  int is_f32;
  long long nx, ny, nz;     /* extended block sizes (nodes) */
  const double* gx;         /* node coordinates of the block, device */
  const double* gy;
  const double* gz;
  const double* nodes;      /* Cartesian node positions (3 per node) or null = identity */
  const float* gxf;         /* node coordinates rounded to float (identity converter) */
  const float* gyf;
  const float* gzf;
  double threshold;
  long long thr_key;        /* integer key of the threshold (d_key) */
  int thr_nan;
  /* float fields: threshold < (double)v  <=>  f_key(v) >= thr_f_key (when thr_f_ok) */
  unsigned thr_f_key;
  int thr_f_ok;
  FastDiv div_cx, div_cy;   /* division by the cells per row (nx - 1) and per column (ny - 1) */
  /* single-precision shading (identity converter only, else null): node
     spacings g[i + 1] - g[i] rounded to float, and an absolute allowance for
     the rounding of the reference's FP64 vertex coordinates */
  const float* dgx;
  const float* dgy;
  const float* dgz;
  float coord_eps;
  /* bound on the FP64 rounding of one screen coordinate in the reference's
     projection (project.c:26-66) of a point of this block, in this scene */
  float proj_eps;
  /* shading only: the cell codes of the whole block ((k ncy + j) ncx + i), when
     they are still in memory (the object took one slab), else null */
  const unsigned char* codes;
};

/* the constants of FastDiv for d >= 1 */
inline FastDiv make_fast_div(unsigned d) {
  unsigned l = 0;
  while (l < 32 && (1ULL << l) < d) l++;
  FastDiv f;
  f.m = (unsigned)((((1ULL << 32) * ((1ULL << l) - d)) / d) + 1);
  f.s1 = l < 1 ? l : 1;
  f.s2 = l > 1 ? l - 1 : 0;
  return f;
}

/* one z-slab of cells: slices [kfirst, kfirst + nslices), rendered [krender0, krender1) */
struct SlabDev {
  long long kfirst;
  long long nslices;
  long long krender0;
  long long krender1;
  int cls_z = 32; /* slices per classification brick (set from the launch shape) */
};

/* launch shape of the tunable kernels, process-wide: slices per
   classification brick, resident blocks per SM of k_emit's grid and of the
   raster passes' grids (k_raster, k_finish) */
struct LaunchShape {
  int cls_z;
  int emit_per_sm;
  int raster_per_sm;
};
int set_launch_shape(const LaunchShape& s);
LaunchShape launch_shape();
/* programmatic dependent launch of the library's kernels on (1) or off (0) */
void set_dependent_launch(int on);
int dependent_launch();

/* triangle arrays (structure of arrays, indexed by emission order within a slab) */
struct TriDev {
  double* wn[3];      /* inspection: area * face normal */
  unsigned* meta;     /* inspection: edge ids (3 x 5 bits) | flags | rank in the cell */
  /* k_cover's input, the compact list of triangles that reach it (k_emit
     appends them), 3 float4 each: x0 y0 z0 x1 | y1 z1 x2 y2 | z2 err_xy
     err_z t -- FP32 screen positions and depths, the bound on |screen x, y -
     the reference's value|, the relative depth bound and the emission index */
  float4* rec;
  double* vert[9];    /* inspection: exact vertices */
  double* vn[9];      /* inspection: vertex normals */
  double* dbg_fn;     /* inspection: face normals, 3 per triangle */
  double* dbg_area;   /* inspection: areas */
  unsigned long long cap; /* triangles the arrays (and the triangle -> cell map) hold */
  unsigned long long rec_cap; /* records the cover and sliver region holds (the arrays' size) */
  unsigned* ovf;      /* overflow flags (kOvf*): set when the slab's triangles exceed cap */
};
constexpr unsigned kMetaRendered = 1u << 15;
constexpr unsigned kMetaCulled = 1u << 16;
constexpr unsigned kMetaRankShift = 17;
constexpr unsigned kMetaUndecided = 1u << 21;

/* FP32 screen vertices of a slab's crossed edges (k_vertices), 16 bytes each:
   X, Y, Z and two bfloat16 rounded up (a bound only loosens): the bound on
   |X, Y - the reference's value| (high half), and the relative depth bound,
   or -1 (projection fails), -2 (undecided) (low half) */
struct VertDev {
  float4* pos;
  unsigned long long cap; /* records pos holds */
  unsigned* ovf;          /* overflow flags (kOvf*) */
};

/*
 * The vertex offset of every cell of a slab (its first owned crossed edge's
 * record in VertDev::pos), as a 16-bit offset from the start of the cell's
 * scan segment of 2^kVSegShift cells (a segment owns at most 7 of them per
 * cell: fewer than 2^16) plus the segment's first offset:
 *   offset(c) = seg[c >> kVSegShift] + rel[c],  c = 0 .. n.
 * Half the bytes of 32-bit offsets, and the scan stores them without waiting
 * for its segment's prefix.
 */
constexpr int kVSegShift = 13;
struct VOffDev {
  unsigned short* rel; /* n + 1 entries */
  unsigned* seg;       /* segments + 1 entries */
};
/* bytes of a VOffDev over n cells, and its layout at `base` (256-byte aligned) */
size_t voff_bytes(long long n);
VOffDev voff_layout(void* base, long long n);

/* overflow flags of a frame whose buffers were sized before the counts were
   known (the frame is then rendered again with larger buffers) */
constexpr unsigned kOvfTriangles = 1u; /* triangles beyond the triangle map or arrays */
constexpr unsigned kOvfVertices = 2u;  /* crossed edges beyond the vertex records */

/* triangle -> cell map entries: cell | rank << 28 (slabs hold fewer than 2^28 cells) */
constexpr unsigned kTcCellMask = 0x0FFFFFFFu;
constexpr unsigned kTcRankShift = 28;

/* what the exact path needs to rebuild a triangle from the field */
struct Geo {
  FieldDev F;
  SlabDev S;
  const unsigned long long* lut;
  const unsigned char* codes;
  const unsigned* tri_cell;
  const unsigned* offsets;  /* triangle offsets per cell (inspection) */
};

/* a fragment that k_exact resolves with the reference's arithmetic */
struct Candidate {
  unsigned t;       /* triangle (emission index in the slab) */
  unsigned pixel;   /* j * width + i */
  float dhi;        /* upper bound of its depth */
  unsigned pad;
};

/* per-frame raster state */
struct RasterDev {
  Slot* canvas;             /* 16-byte (depth, order | rgb) slots */
  unsigned* zlo;            /* per-pixel depth floor (float keys) */
  const double* xs;         /* pixel centres, render.c:100-104 */
  const double* ys;
  const float* xsf;         /* the same rounded to float */
  const float* ysf;
  Candidate* cand;
  unsigned long long cand_cap;
  unsigned long long* cand_count;
  unsigned* tiny;           /* triangles the FP32 filter cannot settle */
  unsigned long long tiny_cap;
  unsigned long long* tiny_count;
  unsigned long long* cover_count; /* entries of TriDev::rec: the cover triangles and the
                                      empty ends of k_emit's chunks (kNoTri) */
  float4* sliver_rec;       /* slivers, in the same records, from the top of TriDev::rec
                               down: entry s at sliver_rec - 3 s (cover + sliver entries
                               <= triangles + emit_list_slack) */
  unsigned long long* sliver_count;
  unsigned long long* listed_count; /* [0] cover, [1] sliver entries, without the empty ones */
  unsigned long long* live_count; /* candidates that can still win (counted by k_finish) */
  /* per pixel, the exact weights of the fragment that last won its CAS: three
     16-byte words (weight k, tag), tag = order << 24 | epoch, each stored
     atomically; shading uses them when all three tags name the final owner */
  ulonglong2* winfo;
  unsigned long long epoch; /* 1 .. 2^24 - 1, per frame */
  unsigned* win;            /* pixels won by the object being shaded */
  unsigned long long* win_count;
  unsigned* amb;            /* won pixels whose FP32 colour is not certain (shaded in FP64) */
  unsigned long long* amb_count;
  unsigned clamp_rgb;       /* the colour at the reference's factor 0.15, computed exactly */
  unsigned* shade_check;    /* self-check: per pixel, 1 << 24 | the FP32 colour when certain */
  unsigned* zerr;           /* bit 0: a z-buffer update gave up after its retry bound */
};

/* one line segment, already projected to pixel units on the host */
struct LineSegDev {
  double p0x, p0y, p0z, p1x, p1y, p1z;
  double width;
  unsigned rgb;
  int valid;
};

/* device error flags */
constexpr unsigned kErrClassifyTimeout = 2u;
constexpr unsigned kErrScanTimeout = 4u;

int upload_tables(const unsigned char code_count[256], const signed char nb[19][4][4],
                  const unsigned char nb_count[19], const unsigned short edge_tris[256 * 19]);

/* the thresholds of the objects of one field, for one classification pass,
   as ranges of sign-folded keys (bits ^ (sign ? 0x7FF..F : 0), signed order
   == numeric order, -0 just below +0, NaNs beyond +-inf): a node is above
   threshold t when (key - lo[t]) < cnt[t] as unsigned, i.e. lo <= key <=
   key(+inf).  cnt 0: nothing is above (NaN threshold, or none above it). */
constexpr int kMaxThr = 4;
struct ThrSet {
  int n;
  unsigned long long lo[kMaxThr], cnt[kMaxThr]; /* double fields */
  unsigned flo[kMaxThr], fcnt[kMaxThr];         /* float fields */
};
struct CodeOut {
  unsigned char* codes[kMaxThr];
};

/* cell codes of nf objects of one field (Fs differ only in the threshold)
   into codes[q]: TMA-staged planes when the field's layout allows it, one
   pass over the field per kMaxThr objects; `err` receives kErrClassifyTimeout.
   Returns the number of kernels launched. */
int launch_classify(const FieldDev* Fs, int nf, const SlabDev& S, unsigned char* const* codes, unsigned* err,
                    cudaStream_t st);
/* one field's classification in a batch, for up to kMaxThr objects: its
   values and sizes, the slab, the thresholds and code arrays, its bricks
   (kClsX x kClsY cells x S.cls_z slices) and the number of its first brick
   among all items' bricks */
struct ClsItem {
  const void* data;
  int is_f32;
  long long nx, ny;
  SlabDev S;
  ThrSet ts;
  CodeOut out;
  unsigned nbx, nby, nbz;
  unsigned long long first;
};
/* the item of objects Fs[0..nf) (one field, nf <= kMaxThr) over slab S */
void make_cls_item(const FieldDev* Fs, int nf, const SlabDev& S, unsigned char* const* codes, ClsItem* it);
/* every item's codes in one persistent launch; `next` (device) must start at 0 */
void launch_classify_queue(const ClsItem* items, int nitems, unsigned long long nunits, unsigned long long* next,
                           cudaStream_t st);
/* cells per slab for which the packed triangle and vertex sums of the scan stay below 2^31 */
constexpr long long kMaxSlabCells = 178956970;

/* 64-bit words of the scan's look-back state over n cells (one per segment
   of cells, then the segment ticket counter) */
long long scan_state_words(long long n);
/* the vertex offsets of cells 0..n, totals = (triangles, vertices), offsets[n], and
   offsets[0..n - 1] when want_offsets; the triangle -> cell map where the
   triangles fit tri_cap (where they do not, `ovf`, when given, receives
   kOvfTriangles: the caller scans again with a larger map).  `state` holds
   scan_state_words(n) words (zeroed here); `err` receives kErrScanTimeout. */
cudaError_t launch_scan(const unsigned char* codes, long long n, unsigned long long* state, unsigned* offsets,
                        const VOffDev& voff, unsigned long long* totals, unsigned* tri_cell,
                        unsigned long long tri_cap, bool want_offsets, unsigned* ovf, unsigned* err,
                        cudaStream_t st);
void launch_vertices(const FieldDev& F, const SlabDev& S, const SceneDev& scene, const unsigned char* codes,
                     const VOffDev& voff, long long n, const VertDev& V, cudaStream_t st);
/* record entries beyond the triangles that k_emit's lists may leave empty
   for a launch sized by tri_bound (the region must hold triangles + this) */
unsigned long long emit_list_slack(long long tri_bound);
void launch_emit(const FieldDev& F, const SlabDev& S, const SceneDev& scene, const unsigned long long* lut,
                 const unsigned char* codes, const unsigned* offsets, const VOffDev& voff,
                 const unsigned* tri_cell, const unsigned long long* total, long long tri_bound, const TriDev& tri,
                 const RasterDev& R, const VertDev& V, unsigned* checks, cudaStream_t st);
void launch_exact_all(const Geo& G, const unsigned long long* total, long long tri_bound, const TriDev& tri,
                      cudaStream_t st);
void launch_normals(const FieldDev& F, const SlabDev& S, const unsigned* offsets, const unsigned* tri_cell,
                    const unsigned long long* total, long long tri_bound, const TriDev& tri, cudaStream_t st);
/* the raster passes of one slab: the cover and sliver lists (k_raster),
   then the candidates that can still win (those below the depth floor
   dropped) and the tiny list in FP64 (k_finish); bounds size the grids */
void launch_raster(const Geo& G, const SceneDev& scene, long long tri_bound, const TriDev& tri,
                   const RasterDev& R, unsigned* checks, cudaStream_t st);
void launch_finish(const Geo& G, const SceneDev& scene, long long bound, const RasterDev& R,
                   unsigned long long order_base, unsigned* checks, cudaStream_t st);
/* winners, normal requests, weighted normals, colours; `between` (optional)
   is recorded before the colour passes; `checks` (self-check) counts FP32
   colours that differ from the FP64 ones */
/* after all slabs of a contour object: list the pixels it won (R.win) and
   colour those the FP32 pass settles; the others go to R.amb */
void launch_shade_f(const FieldDev& F, const SceneDev& scene, const RasterDev& R, const unsigned long long* lut,
                    unsigned long long obase, unsigned rgb, cudaStream_t st);
/* the FP64 colour of npix listed pixels (count on the device): ent (ent_cap
   entries, ent_count must start at 0), spans (3 per pixel) and wn (3 doubles
   per entry) are scratch; when *ent_count ends above ent_cap some pixels were
   left out and the call must be repeated with more entries */
void launch_shade_exact(const FieldDev& F, const SceneDev& scene, const RasterDev& R, const unsigned long long* lut,
                        const unsigned* pixels, const unsigned long long* count, long long npix,
                        unsigned long long obase, unsigned long long* ent, unsigned long long ent_cap,
                        unsigned long long* ent_count, uint2* spans, double* wn, unsigned rgb, unsigned* checks,
                        cudaStream_t st);
void launch_lines(const LineSegDev* segs, int nseg, long long W, long long H, Slot* canvas,
                  unsigned long long order_base, unsigned* zerr, cudaStream_t st);
void launch_canvas_init(Slot* canvas, unsigned* zlo, long long n, unsigned long long hi, unsigned long long lo,
                        cudaStream_t st);
void launch_resolve(const Slot* canvas, long long W, long long H, unsigned char* rgb, double* depth,
                    cudaStream_t st);

}  // namespace c3d
