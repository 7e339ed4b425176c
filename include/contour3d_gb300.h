/*
 * contour3d_gb300.h -- extensions of the GB300 isosurface library beside the
 * unchanged drop-in entry point of contour3d.h.
 *
 * All entry points are plain C: host or device pointers and sizes, int
 * return codes (0 = success, 1 = failure, with a "[CONTOUR3D ERROR] " line on
 * stderr), as in the reference library (src/contour3d/main.c:68-146).
 * None of them exists in the reference; each comment says which reference
 * behaviour it shares.
 */
#if !defined(CONTOUR3D_GB300_H)
#define CONTOUR3D_GB300_H

#include <stddef.h>
#include <stdint.h>
#include "contour3d.h"

#if defined(__cplusplus)
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* converters                                                          */
/* ------------------------------------------------------------------ */

/*
 * The identity map.  Passing it (or NULL) as a converter tells the library
 * that grid coordinates are Cartesian, so node positions are read from the
 * grids on the device.  Any other converter is called once per grid node on
 * the host and its results are uploaded (the reference calls it for every
 * tetrahedron corner, triangulate.c:156-173; the results are the same).
 */
contour3d_vector_t contour3d_gb300_identity(const contour3d_vector_t orthogonal);

/* declare a caller's own converter to be the identity (up to 16 may be declared) */
int contour3d_gb300_declare_identity(contour3d_vector_t (*converter)(const contour3d_vector_t));

/* ------------------------------------------------------------------ */
/* single-process rendering into caller memory                          */
/* ------------------------------------------------------------------ */

/*
 * contour3d_execute on one process, without the file: `rgb_out` receives the
 * ppm body (width * height * 3 bytes, rows flipped as output.c:113-123
 * writes them); `depth_out` (optional, width * height doubles, canvas order)
 * the final depth buffer, -DBL_MAX where nothing was drawn.
 * Fields and grids are host pointers, as in contour3d_execute.
 */
int contour3d_gb300_render(const contour3d_vector_t *camera_position,
                           const contour3d_vector_t *light_direction,
                           const size_t screen_sizes[2],
                           const contour3d_vector_t *screen_center,
                           const contour3d_vector_t screen_local[2],
                           const contour3d_color_t *bg_color, size_t num_contours,
                           const contour3d_contour_obj_t *contour_objs, size_t num_lines,
                           const contour3d_line_obj_t *line_objs, uint8_t *rgb_out,
                           double *depth_out);

/* ------------------------------------------------------------------ */
/* device-resident fields                                              */
/* ------------------------------------------------------------------ */

#define CONTOUR3D_GB300_F64 0
#define CONTOUR3D_GB300_F32 1

/*
 * A whole field already resident in device memory (x fastest), as an in-situ
 * solver on the same GPU holds it.  float32 fields are widened to double
 * exactly when read, so they give the result the double path gives for the
 * widened field.  `grids` are host node coordinates (sizes[d] values each).
 */
typedef struct {
  const void *device_array;
  int dtype;
  size_t sizes[3];
  const double *grids[3];
  contour3d_vector_t (*converter)(const contour3d_vector_t);
  double threshold;
  contour3d_color_t color;
} contour3d_gb300_field_t;

/*
 * Render device-resident fields.  `rgb_out` is a DEVICE pointer to
 * width * height * 3 bytes (ppm row order); `stream` a cudaStream_t (NULL =
 * the library's own stream).  The call returns when the image is complete.
 */
int contour3d_gb300_render_device(const contour3d_vector_t *camera_position,
                                  const contour3d_vector_t *light_direction,
                                  const size_t screen_sizes[2],
                                  const contour3d_vector_t *screen_center,
                                  const contour3d_vector_t screen_local[2],
                                  const contour3d_color_t *bg_color, size_t num_fields,
                                  const contour3d_gb300_field_t *fields, size_t num_lines,
                                  const contour3d_line_obj_t *line_objs, uint8_t *rgb_out,
                                  void *stream);

/*
 * Per-cell triangle offsets of one iso-level, for callers that cannot let a
 * library allocate device memory: an in-situ solver whose memory pool owns
 * the GPU's memory (a cudaMalloc would fail or break its accounting), or a
 * time-stepping loop that must not stall on the device synchronisation that
 * cudaFree implies.  No counterpart in the reference.
 *
 * `device_field` holds sizes[0] * sizes[1] * sizes[2] values of `dtype`
 * (x fastest).  Outputs, in device memory: `device_offsets` the exclusive
 * prefix sum of the triangle count of every cell, (nx-1)(ny-1)(nz-1) + 1
 * entries, the last one being the total; `device_total` the total again.
 * The call allocates nothing: its only scratch is a static device array of
 * 512 KiB that every GPU loading the library keeps until the process exits,
 * which limits the field to 268,435,455 cells (larger fields are rejected
 * with an error).  The first call on a device looks up that array's device
 * address, so make it before any stream capture on the device.  All calls
 * share the array; calls that overlap on the GPU race and must be serialised
 * by the caller.  `stream` (null: the legacy default stream) must belong to
 * the current device.  Every call copies a 4-byte error word back to the host
 * and synchronises `stream`, and returns when the result is in device memory.
 */
int contour3d_gb300_cell_offsets_noalloc(const void *device_field, int dtype, const size_t sizes[3],
                                         double threshold, uint32_t *device_offsets,
                                         unsigned long long *device_total, void *stream);

/* ------------------------------------------------------------------ */
/* batched and served forms                                           */
/* ------------------------------------------------------------------ */

/* one frame of device-resident fields (as contour3d_gb300_render_device) */
typedef struct {
  contour3d_vector_t camera_position;
  contour3d_vector_t light_direction;
  size_t screen_sizes[2];
  contour3d_vector_t screen_center;
  contour3d_vector_t screen_local[2];
  contour3d_color_t bg_color;
  size_t num_fields;
  const contour3d_gb300_field_t *fields;
  size_t num_lines;
  const contour3d_line_obj_t *lines;
  uint8_t *rgb_out; /* device, width * height * 3 bytes in ppm row order */
} contour3d_gb300_frame_t;

/*
 * Render many frames (each with its own fields, levels and camera) with
 * `workers` concurrent contexts; returns when all are done.  frame_ms
 * (optional) receives each frame's device time.  Images equal those of
 * contour3d_gb300_render_device frame by frame.
 */
int contour3d_gb300_render_batch(const contour3d_gb300_frame_t *frames, size_t num_frames, int workers,
                                 double *frame_ms);

/*
 * Served form: a request loop with `slots` concurrent contexts against an
 * HBM budget of `hbm_budget_bytes` (0 = unlimited), of which the caller's
 * resident fields take `resident_bytes`.  A submitted frame starts when a
 * slot is free and the part of its working set known before it runs (code
 * and offset arrays of its largest slab, z-buffer and per-pixel arrays) fits
 * next to what the running requests hold; requests arriving while others
 * run are admitted as slots and memory free up.  While a request runs, every
 * growth of its device buffers is charged against the budget when it is
 * sized -- the triangle-dependent buffers from the triangle count of each
 * slab's classification -- and waits while it does not fit, after first
 * releasing the buffers of idle contexts.  A growth that would wait while
 * every other running request waits too goes ahead above the budget (counted
 * in contour3d_gb300_server_memory), so no wait is endless.  The frame struct
 * and everything it points to must stay valid until
 * contour3d_gb300_server_wait returns for its ticket.
 */
typedef struct contour3d_gb300_server contour3d_gb300_server_t;
typedef struct {
  double latency_ms;      /* submit -> done */
  double queue_ms;        /* submit -> start */
  double device_ms;       /* device time of the frame */
  uint64_t estimate_bytes; /* the working-set part known at admission */
  uint64_t held_bytes;    /* device bytes its context held when it finished */
} contour3d_gb300_request_stats_t;

/* device memory of a server's contexts: bytes held now and at most so far,
   growths let through above the budget, idle contexts trimmed */
typedef struct {
  uint64_t used_bytes;
  uint64_t peak_bytes;
  uint64_t overcommits;
  uint64_t trims;
} contour3d_gb300_server_memory_t;
int contour3d_gb300_server_memory(contour3d_gb300_server_t *server, contour3d_gb300_server_memory_t *out);

contour3d_gb300_server_t *contour3d_gb300_server_create(int slots, uint64_t hbm_budget_bytes,
                                                        uint64_t resident_bytes);
int contour3d_gb300_server_submit(contour3d_gb300_server_t *server, const contour3d_gb300_frame_t *frame,
                                  uint64_t *ticket);
int contour3d_gb300_server_wait(contour3d_gb300_server_t *server, uint64_t ticket,
                                contour3d_gb300_request_stats_t *stats);
int contour3d_gb300_server_destroy(contour3d_gb300_server_t *server);

/* device bytes currently held by the library's buffers (all contexts) */
uint64_t contour3d_gb300_device_bytes(void);

/* statistics of the last render call */
typedef struct {
  uint64_t cells;             /* cells classified (cell x threshold) */
  uint64_t triangles;         /* triangles emitted (triangulated set, all slabs) */
  uint64_t candidates;        /* fragments the single-precision filter could not settle */
  uint64_t candidate_overflows; /* raster passes repeated because a list was full */
  uint64_t tiny;              /* triangles too small for the FP32 filter (resolved in FP64) */
  uint64_t winners;           /* pixels shaded (each object's won pixels, summed over objects) */
  uint64_t normals;           /* neighbour-triangle normals of the FP64 shading pass */
  uint64_t slabs;             /* slab passes */
  uint64_t kernel_launches;   /* kernels launched by the library */
  double ms_total;            /* device time of the whole frame (events) */
  /* per stage, when stage timing is on */
  double ms_classify, ms_scan, ms_emit, ms_cover, ms_exact, ms_shade;
  /* self-check counters when the filter check is on (all must stay 0):
     [0] projection cull decided wrongly, [1] projection outside its bound,
     [2] covered pixel dropped, [3] uncovered pixel called inside,
     [4] depth outside its interval */
  uint64_t filter_violations[5];
  uint64_t cover_triangles;   /* triangles whose extent may hold a pixel centre (FP32 filter input) */
  uint64_t exact_fragments;   /* candidates that reached the reference's FP64 arithmetic */
  uint64_t slivers;           /* triangles whose area may be clamped (reference box tested in FP32) */
  uint64_t vertices;          /* crossed edges whose screen position was computed (all slabs) */
  double ms_vertices;         /* stage timing: triangle -> cell map and screen vertices */
  double ms_normals;          /* stage timing: won pixels and the FP32 shading pass
                                 (ms_shade is then the FP64 shading pass) */
  uint64_t shade_exact;       /* won pixels whose colour the FP32 shading could not settle (shaded in FP64) */
  uint64_t shade_violations;  /* self-check: FP32 colours that differ from the FP64 ones (must stay 0) */
  uint64_t unsynchronised;    /* 1: the frame ran with one host synchronisation, at its end */
  uint64_t redone;            /* 1: an unsynchronised pass found more work than its buffers held, and
                                 the frame was rendered again with synchronisation */
  uint64_t graph;             /* 1: the frame was recorded as a CUDA graph, 2: it ran as the recorded graph */
} contour3d_gb300_stats_t;

int contour3d_gb300_last_stats(contour3d_gb300_stats_t *out);
/* 1 = record per-stage CUDA events (adds synchronisation), 0 = off (default) */
int contour3d_gb300_set_stage_timing(int on);
/*
 * 1 = also run the reference's FP64 arithmetic for every pixel the
 * single-precision filter classifies and count disagreements with its
 * certified bounds (slow; for tests), 0 = off (default)
 */
int contour3d_gb300_set_filter_check(int on);
/*
 * 1 (default) = a frame of a context that has completed one frame runs with
 * one host synchronisation, at its end: its buffers are sized from the
 * largest counts the context has seen, every pass's counts stay on the device
 * until the end, and a frame that finds more work than the buffers hold is
 * rendered again with synchronisation (which learns the larger counts);
 * 0 = synchronise after every slab's scan and raster pass and size every
 * buffer from the counts just read.  The image is the same either way.
 * Applies to the library's own context (contour3d_execute, the render
 * entry points).
 */
int contour3d_gb300_set_async(int on);
/*
 * The same, and graph recording, for the worker contexts of servers (and of
 * contour3d_gb300_render_batch) created afterwards: 0 (default) = worker
 * contexts synchronise after every slab pass; 1 = unsynchronised frames and
 * graphs.  Off by default: with unsynchronised workers the batched and
 * served workloads measured no faster (the other workers keep the GPU busy
 * while one waits), and a worker's sizes, learnt from frames of every size,
 * overflow more often.
 */
int contour3d_gb300_set_server_async(int on);
/*
 * 1 (default) = an unsynchronised frame drawn from device-resident fields
 * into device memory, on a stream other than the legacy default stream, is
 * recorded as a CUDA graph the second time in a row that a frame with the
 * same description comes (fields' addresses, types, sizes, grids and levels,
 * scene, lines, output and stream), and from the third time on the graph is
 * launched instead of the frame's individual calls; the field values may
 * change between frames (an in-situ solver's time steps).  A frame that finds
 * more work than the recorded sizes drops the graph.  0 = no graphs.
 * Applies to the library's own context.
 */
int contour3d_gb300_set_graphs(int on);
/*
 * Launch shape of the tunable kernels, for every context of the process:
 * node slices per classification brick (default 32), resident blocks per SM
 * of the triangle pass's grid and of the raster passes' grids (default 8
 * each).  Results do not depend on it.  contour3d_gb300/autotune.py chooses
 * it per GPU and workload size class.  Returns 1 for values out of range.
 */
int contour3d_gb300_set_launch_shape(int classify_slices, int emit_blocks_per_sm, int raster_blocks_per_sm);
/*
 * 1 = launch the library's kernels with programmatic dependent launch (a
 * kernel may be scheduled while its predecessor finishes and waits in
 * griddepcontrol.wait before touching earlier results); 0 (default) =
 * ordinary stream order.
 */
int contour3d_gb300_set_dependent_launch(int on);
/*
 * 1 (default) = contour3d_gb300_render_batch classifies the cells of every
 * frame whose fields each fit one slab in one persistent launch over
 * (field, brick) work items taken from a device counter, before the frames'
 * own passes; 0 = each frame classifies its own fields.  Images do not
 * depend on it.
 */
int contour3d_gb300_set_batch_classify(int on);
/*
 * The model that sizes the slabs of a host field uploaded while it is
 * processed (fields of 64 MB or more): the host link's rate, the slab
 * passes' cost per cell and contour object, and their fixed cost per object
 * and slab.  Defaults measured on GB300: 211 GB/s, 18.9 ps, 40 us.  Images do
 * not depend on it.  Returns 1 for values out of range.
 */
int contour3d_gb300_set_upload_model(double link_gb_per_s, double slab_ps_per_cell, double slab_fixed_us);
/* upper bound on cells per slab (default and maximum 178,956,970, the most the
   scan's packed 32-bit sums allow); smaller slabs use less memory */
int contour3d_gb300_set_slab_cells(uint64_t max_cells);

/* ------------------------------------------------------------------ */
/* inspection                                                          */
/* ------------------------------------------------------------------ */

/*
 * Every rendered triangle of one contour object (single process) in the
 * reference's drawing order (contour/main.c:92-112): per triangle 9 vertex
 * coordinates, 9 vertex-normal components, 3 face-normal components, area
 * (22 doubles), then cell (i, j, k) and the 3 cube-edge ids (6 int64) --
 * 224 bytes.  Returns the rendered count (writes at most `capacity`) or -1.
 * *num_triangulated receives the count over all triangulated cells.
 */
long contour3d_gb300_debug_triangles(const contour3d_contour_obj_t *obj, void *out,
                                     long capacity, long *num_triangulated);

/* per-cell triangle counts (uint8, (nx-1)(ny-1)(nz-1), x fastest); returns the total or -1 */
long contour3d_gb300_debug_cell_counts(const contour3d_contour_obj_t *obj, uint8_t *counts);

/* ------------------------------------------------------------------ */
/* multi-process transport (builds without MPI)                          */
/* ------------------------------------------------------------------ */

/*
 * Point-to-point exchange used for the halo exchange of extend.c:10-147 and
 * the nearest-depth reduction of output.c:32-88 when the library is built
 * without MPI.  sendrecv sends `sendbytes` to `dest` and receives
 * `recvbytes` from `source`; either peer may be MPI_PROC_NULL (that half is
 * skipped).  Returns 0 on success.
 */
typedef struct {
  int size;
  int rank;
  int (*sendrecv)(void *user, const void *sendbuf, size_t sendbytes, int dest, void *recvbuf,
                  size_t recvbytes, int source);
  void *user;
} contour3d_gb300_transport_t;

/* install (or, with NULL, remove) the transport behind MPI_COMM_WORLD */
int contour3d_gb300_install_transport(const contour3d_gb300_transport_t *transport);

/*
 * Host-side array extension of one contour object (extend.c:150-282): the
 * pencil-local block widened by two layers towards every neighbour rank and
 * clipped at the global boundary.  Call once with ext == NULL to get sizes
 * and offsets, then with a buffer of sizes[0]*sizes[1]*sizes[2] doubles.
 * Collective over the decomposition.
 */
int contour3d_gb300_extend(const sdecomp_info_t *info, const contour3d_contour_obj_t *obj,
                           size_t sizes[3], size_t offsets[3], double *ext);

/*
 * The nearest-depth reduction of per-rank images to rank 0 (output.c:32-88,
 * reduction_func output.c:10-30: keep the pixel with the larger depth), over
 * the installed transport.  `depth` holds num_pixels doubles, `rgb`
 * 3 * num_pixels bytes.  Collective over the decomposition; on rank 0 the
 * arrays receive the result, on the other ranks they are left partial.
 */
int contour3d_gb300_reduce_nearest(const sdecomp_info_t *info, double *depth, uint8_t *rgb, size_t num_pixels);

/* release every device and pinned-host buffer the library holds */
int contour3d_gb300_release(void);

#if defined(__cplusplus)
}
#endif

#endif /* CONTOUR3D_GB300_H */
