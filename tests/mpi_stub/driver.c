/*
 * Two-rank check of the library's host code built with MPI (and, with
 * -DEXTERNAL_TABLE, with the SimpleDecomp table supplied by the caller as a
 * -DCONTOUR3D_EXTERNAL_SDECOMP build expects).  Rank 1 is a forked child;
 * the ranks talk through the stub MPI's socket.  The field is split along z
 * (pencil X1); each rank's extended block must equal the window of the
 * global field that extend.c:150-282 produces, and after the nearest-depth
 * reduction rank 0 must hold the per-pixel maximum (output.c:10-30).
 * Test infrastructure only.  Exit code 0 on success.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/socket.h>
#include <sys/wait.h>
#include <unistd.h>
#include "mpi.h"
#include "contour3d.h"
#include "contour3d_gb300.h"

enum { NX = 9, NY = 7, NZ = 12, NPIX = 301 };

static double value(size_t i, size_t j, size_t k) { return (double)(i + 10 * j + 100 * k) + 0.25; }

#if defined(EXTERNAL_TABLE)
/* the caller's SimpleDecomp: two ranks split along z, nothing else split */
struct sdecomp_info_t { MPI_Comm comm; int rank, size; };
static int t_construct(MPI_Comm c, size_t nd, const size_t dims[], const bool periods[], sdecomp_info_t **info) {
  (void)nd; (void)dims; (void)periods;
  sdecomp_info_t *p = calloc(1, sizeof *p);
  p->comm = c;
  MPI_Comm_rank(c, &p->rank);
  MPI_Comm_size(c, &p->size);
  *info = p;
  return 0;
}
static int t_destruct(sdecomp_info_t *info) { free(info); return 0; }
static int t_cart(const sdecomp_info_t *info, MPI_Comm *c) { *c = info->comm; return 0; }
static int t_rank(const sdecomp_info_t *info, int *r) { *r = info->rank; return 0; }
static int t_nprocs(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, int *n) {
  (void)p; *n = d == SDECOMP_ZDIR ? info->size : 1; return 0;
}
static int t_myrank(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, int *r) {
  (void)p; *r = d == SDECOMP_ZDIR ? info->rank : 0; return 0;
}
static int t_nb(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, int nb[2]) {
  (void)p;
  nb[0] = nb[1] = MPI_PROC_NULL;
  if (d == SDECOMP_ZDIR) {
    if (info->rank > 0) nb[0] = info->rank - 1;
    if (info->rank + 1 < info->size) nb[1] = info->rank + 1;
  }
  return 0;
}
static int t_mysize(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, size_t g, size_t *m) {
  (void)p;
  *m = d == SDECOMP_ZDIR ? g / info->size + ((size_t)info->rank < g % info->size ? 1 : 0) : g;
  return 0;
}
static int t_offset(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, size_t g, size_t *o) {
  (void)p;
  const size_t b = g / info->size, r = g % info->size, me = (size_t)info->rank;
  *o = d == SDECOMP_ZDIR ? me * b + (me < r ? me : r) : 0;
  return 0;
}
const sdecomp_t sdecomp = {t_construct, t_destruct, t_cart, t_rank, t_nprocs, t_myrank, t_nb, t_mysize, t_offset};
#endif

static int run(int rank) {
  sdecomp_info_t *info = NULL;
  const size_t dims[3] = {0, 0, 0};
  const bool periods[3] = {false, false, false};
  if (sdecomp.construct(MPI_COMM_WORLD, 3, dims, periods, &info)) return 10;
  const size_t gl[3] = {NX, NY, NZ};
  size_t my[3], off[3];
  for (int d = 0; d < 3; d++) {
    sdecomp.get_pencil_mysize(info, SDECOMP_X1PENCIL, (sdecomp_dir_t)d, gl[d], &my[d]);
    sdecomp.get_pencil_offset(info, SDECOMP_X1PENCIL, (sdecomp_dir_t)d, gl[d], &off[d]);
  }
  if (my[0] != NX || my[1] != NY || my[2] >= NZ) return 11; /* split along z only */
  double *local = malloc(sizeof(double) * my[0] * my[1] * my[2]);
  for (size_t k = 0; k < my[2]; k++)
    for (size_t j = 0; j < my[1]; j++)
      for (size_t i = 0; i < my[0]; i++) local[(k * my[1] + j) * my[0] + i] = value(i, j, k + off[2]);
  double grid[NZ];
  for (int n = 0; n < NZ; n++) grid[n] = n;
  contour3d_contour_obj_t obj;
  memset(&obj, 0, sizeof obj);
  obj.pencil = SDECOMP_X1PENCIL;
  obj.glsizes[0] = NX; obj.glsizes[1] = NY; obj.glsizes[2] = NZ;
  obj.grids[0] = grid; obj.grids[1] = grid; obj.grids[2] = grid;
  obj.array = local;
  size_t es[3], eo[3];
  if (contour3d_gb300_extend(info, &obj, es, eo, NULL)) return 12;
  const size_t lo = off[2] >= 2 ? off[2] - 2 : 0, hi = off[2] + my[2] + 2 < NZ ? off[2] + my[2] + 2 : NZ;
  if (es[0] != NX || es[1] != NY || eo[2] != lo || es[2] != hi - lo) return 13;
  double *ext = malloc(sizeof(double) * es[0] * es[1] * es[2]);
  if (contour3d_gb300_extend(info, &obj, es, eo, ext)) return 14;
  for (size_t k = 0; k < es[2]; k++)
    for (size_t j = 0; j < NY; j++)
      for (size_t i = 0; i < NX; i++)
        if (ext[(k * NY + j) * NX + i] != value(i, j, k + eo[2])) return 15;
  /* pixels: rank r has depth r at even pixels and -r at odd ones */
  double depth[NPIX];
  unsigned char rgb[3 * NPIX];
  for (int p = 0; p < NPIX; p++) {
    depth[p] = p % 2 ? -(double)rank : (double)rank;
    rgb[3 * p] = (unsigned char)(rank + 1);
    rgb[3 * p + 1] = (unsigned char)p;
    rgb[3 * p + 2] = 7;
  }
  if (contour3d_gb300_reduce_nearest(info, depth, rgb, NPIX)) return 16;
  if (rank == 0)
    for (int p = 0; p < NPIX; p++) {
      const int win = p % 2 ? 0 : 1; /* the nearer fragment (larger depth) */
      if (depth[p] != (p % 2 ? 0. : 1.) || rgb[3 * p] != win + 1) return 17;
    }
  free(ext);
  free(local);
  sdecomp.destruct(info);
  return 0;
}

int main(void) {
  int sv[2];
  if (socketpair(AF_UNIX, SOCK_STREAM, 0, sv)) return 2;
  const pid_t pid = fork();
  if (pid < 0) return 3;
  if (pid == 0) {
    close(sv[0]);
    c3d_stub_mpi_init(1, 2, sv[1]);
    _exit(run(1));
  }
  close(sv[1]);
  c3d_stub_mpi_init(0, 2, sv[0]);
  const int rc0 = run(0);
  int st = 0;
  waitpid(pid, &st, 0);
  const int rc1 = WIFEXITED(st) ? WEXITSTATUS(st) : 99;
  printf("rank0 %d rank1 %d\n", rc0, rc1);
  return rc0 || rc1 ? 1 : 0;
}
