/*
 * Single-process MPI and SimpleDecomp stand-ins for compiling the reference
 * library sources into oracle/_ref/ (CPU checker only, never shipped).
 * One rank: sizes are global sizes, offsets are zero, neighbours are
 * MPI_PROC_NULL, so every halo exchange of extend.c is a no-op and every
 * boundary is clipped (extend.c:229-252).
 */
#include <stdio.h>
#include <stdlib.h>
#include "mpi.h"
#include "sdecomp.h"

int MPI_Type_create_hvector(int count, int blocklength, MPI_Aint stride,
                            MPI_Datatype oldtype, MPI_Datatype *newtype) {
  (void)count; (void)blocklength; (void)stride; (void)oldtype;
  *newtype = 100; return 0;
}
int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype *newtype) {
  (void)count; (void)oldtype; *newtype = 101; return 0;
}
int MPI_Type_create_struct(int count, const int blocklengths[],
                           const MPI_Aint displacements[],
                           const MPI_Datatype types[], MPI_Datatype *newtype) {
  (void)count; (void)blocklengths; (void)displacements; (void)types;
  *newtype = 102; return 0;
}
int MPI_Type_commit(MPI_Datatype *datatype) { (void)datatype; return 0; }
int MPI_Type_free(MPI_Datatype *datatype) { *datatype = MPI_DATATYPE_NULL; return 0; }
int MPI_Op_create(MPI_User_function *fn, int commute, MPI_Op *op) {
  (void)fn; (void)commute; *op = 1; return 0;
}
int MPI_Op_free(MPI_Op *op) { *op = MPI_OP_NULL; return 0; }
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                 int dest, int sendtag, void *recvbuf, int recvcount,
                 MPI_Datatype recvtype, int source, int recvtag, MPI_Comm comm,
                 MPI_Status *status) {
  (void)sendbuf; (void)sendcount; (void)sendtype; (void)sendtag; (void)recvbuf;
  (void)recvcount; (void)recvtype; (void)recvtag; (void)comm; (void)status;
  if (dest != MPI_PROC_NULL || source != MPI_PROC_NULL) {
    fprintf(stderr, "ref shim: single-rank MPI_Sendrecv got a real peer\n");
    abort();
  }
  return 0;
}
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype datatype, MPI_Op op, int root, MPI_Comm comm) {
  (void)recvbuf; (void)count; (void)datatype; (void)op; (void)comm;
  if (sendbuf != MPI_IN_PLACE || root != 0) {
    fprintf(stderr, "ref shim: single-rank MPI_Reduce must be in place at root 0\n");
    abort();
  }
  return 0;
}

/* ---- single-process SimpleDecomp ---- */
struct sdecomp_info_t { int unused; };
static struct sdecomp_info_t the_info;

static int s_construct(MPI_Comm c, size_t ndims, const size_t dims[],
                       const bool periods[], sdecomp_info_t **info) {
  (void)c; (void)ndims; (void)dims; (void)periods; *info = &the_info; return 0;
}
static int s_destruct(sdecomp_info_t *info) { (void)info; return 0; }
static int s_comm_cart(const sdecomp_info_t *i, MPI_Comm *c) { (void)i; *c = MPI_COMM_WORLD; return 0; }
static int s_comm_rank(const sdecomp_info_t *i, int *r) { (void)i; *r = 0; return 0; }
static int s_nprocs(const sdecomp_info_t *i, sdecomp_pencil_t p, sdecomp_dir_t d, int *n) {
  (void)i; (void)p; (void)d; *n = 1; return 0;
}
static int s_myrank(const sdecomp_info_t *i, sdecomp_pencil_t p, sdecomp_dir_t d, int *r) {
  (void)i; (void)p; (void)d; *r = 0; return 0;
}
static int s_neighbours(const sdecomp_info_t *i, sdecomp_pencil_t p, sdecomp_dir_t d, int nb[2]) {
  (void)i; (void)p; (void)d; nb[0] = MPI_PROC_NULL; nb[1] = MPI_PROC_NULL; return 0;
}
static int s_mysize(const sdecomp_info_t *i, sdecomp_pencil_t p, sdecomp_dir_t d, size_t g, size_t *m) {
  (void)i; (void)p; (void)d; *m = g; return 0;
}
static int s_offset(const sdecomp_info_t *i, sdecomp_pencil_t p, sdecomp_dir_t d, size_t g, size_t *o) {
  (void)i; (void)p; (void)d; (void)g; *o = 0; return 0;
}
const sdecomp_t sdecomp = {
  s_construct, s_destruct, s_comm_cart, s_comm_rank, s_nprocs, s_myrank,
  s_neighbours, s_mysize, s_offset,
};
