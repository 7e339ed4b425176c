/*
 * sdecomp.h -- the part of the SimpleDecomp pencil-decomposition interface
 * that contour3d_execute consumes.
 *
 * The reference takes its decomposition from the SimpleDecomp submodule
 * (reference .gitmodules:1-4), whose sources are not part of the reference
 * tree.  This header is written from the reference's call sites only:
 *   construct/destruct            src/main.c:119-125, :332
 *   get_pencil_mysize/_offset     src/contour3d/contour/extend.c:161-180
 *   get_comm_cart/get_neighbours  src/contour3d/contour/extend.c:17-21
 *   get_nprocs/get_myrank         src/contour3d/contour/extend.c:219-220
 *   get_comm_rank                 src/contour3d/output.c:98
 * A deployment that already links the real SimpleDecomp (and MPI) builds the
 * library with -DCONTOUR3D_USE_MPI -DCONTOUR3D_EXTERNAL_SDECOMP and that
 * project's include directory ahead of this one
 * (contour3d_gb300.build.build_mpi): contour3d.h then includes that
 * project's sdecomp.h, the library leaves out its own `sdecomp` table and
 * calls the caller's, and it uses only the names below.
 *
 * Without MPI (-DCONTOUR3D_USE_MPI not given) the library ships its own
 * `sdecomp` object and a minimal communicator: a single process by default,
 * or the ranks of a point-to-point transport installed with
 * contour3d_gb300_install_transport() (see contour3d_gb300.h).
 */
#if !defined(SDECOMP_H)
#define SDECOMP_H

#include <stdbool.h>
#include <stddef.h>

#if defined(CONTOUR3D_USE_MPI)
#include <mpi.h>
#else
#if defined(__cplusplus)
extern "C" {
#endif
/* opaque communicator handle standing in for MPI_Comm */
typedef struct c3d_comm_s * MPI_Comm;
#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_PROC_NULL (-2)
/* the world communicator: one process, or the installed transport's ranks */
extern MPI_Comm c3d_comm_world(void);
#define MPI_COMM_WORLD (c3d_comm_world())
#if defined(__cplusplus)
}
#endif
#endif

#if defined(__cplusplus)
extern "C" {
#endif

typedef enum {
  SDECOMP_XDIR = 0,
  SDECOMP_YDIR = 1,
  SDECOMP_ZDIR = 2,
} sdecomp_dir_t;

/*
 * Pencils: "X1"/"X2" are not split in x, "Y1"/"Y2" not in y, "Z1"/"Z2" not
 * in z.  The two split directions share the 2-D process grid (P0, P1); the
 * "1" and "2" variants assign its axes in opposite order.
 */
typedef enum {
  SDECOMP_X1PENCIL = 0,
  SDECOMP_Y1PENCIL = 1,
  SDECOMP_Z1PENCIL = 2,
  SDECOMP_X2PENCIL = 3,
  SDECOMP_Y2PENCIL = 4,
  SDECOMP_Z2PENCIL = 5,
} sdecomp_pencil_t;

typedef struct sdecomp_info_t sdecomp_info_t;

typedef struct {
  /* dims: process-grid sizes per direction, 0 = choose; periods: wrap-around */
  int (* construct) (MPI_Comm comm_default, size_t ndims, const size_t dims[],
                     const bool periods[], sdecomp_info_t ** info);
  int (* destruct) (sdecomp_info_t * info);
  int (* get_comm_cart) (const sdecomp_info_t * info, MPI_Comm * comm_cart);
  int (* get_comm_rank) (const sdecomp_info_t * info, int * rank);
  int (* get_nprocs) (const sdecomp_info_t * info, sdecomp_pencil_t pencil,
                      sdecomp_dir_t dir, int * nprocs);
  int (* get_myrank) (const sdecomp_info_t * info, sdecomp_pencil_t pencil,
                      sdecomp_dir_t dir, int * myrank);
  /* neighbours[0]: negative side, neighbours[1]: positive side (or MPI_PROC_NULL) */
  int (* get_neighbours) (const sdecomp_info_t * info, sdecomp_pencil_t pencil,
                          sdecomp_dir_t dir, int neighbours[2]);
  int (* get_pencil_mysize) (const sdecomp_info_t * info, sdecomp_pencil_t pencil,
                             sdecomp_dir_t dir, size_t glsize, size_t * mysize);
  int (* get_pencil_offset) (const sdecomp_info_t * info, sdecomp_pencil_t pencil,
                             sdecomp_dir_t dir, size_t glsize, size_t * offset);
} sdecomp_t;

extern const sdecomp_t sdecomp;

#if defined(__cplusplus)
}
#endif

#endif /* SDECOMP_H */
