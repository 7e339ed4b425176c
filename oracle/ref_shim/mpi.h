/*
 * Single-process stand-in for the few MPI calls made by the reference
 * library sources (src/contour3d/contour/extend.c:17-147,
 * src/contour3d/output.c:32-88).  Used ONLY to compile the reference into
 * oracle/_ref/ as a CPU checker; never linked into the product.
 *
 * With one rank every neighbour is MPI_PROC_NULL, so MPI_Sendrecv moves no
 * data, and MPI_Reduce with MPI_IN_PLACE at the root is the identity.
 */
#if !defined(C3D_REF_SHIM_MPI_H)
#define C3D_REF_SHIM_MPI_H
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef long MPI_Aint;
typedef struct { int dummy; } MPI_Status;
typedef void MPI_User_function(void *, void *, int *, MPI_Datatype *);

#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_PROC_NULL (-2)
#define MPI_DATATYPE_NULL 0
#define MPI_DOUBLE 1
#define MPI_UNSIGNED_CHAR 2
#define MPI_OP_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

int MPI_Type_create_hvector(int count, int blocklength, MPI_Aint stride,
                            MPI_Datatype oldtype, MPI_Datatype *newtype);
int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype *newtype);
int MPI_Type_create_struct(int count, const int blocklengths[],
                           const MPI_Aint displacements[],
                           const MPI_Datatype types[], MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *datatype);
int MPI_Type_free(MPI_Datatype *datatype);
int MPI_Op_create(MPI_User_function *fn, int commute, MPI_Op *op);
int MPI_Op_free(MPI_Op *op);
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                 int dest, int sendtag, void *recvbuf, int recvcount,
                 MPI_Datatype recvtype, int source, int recvtag, MPI_Comm comm,
                 MPI_Status *status);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype datatype, MPI_Op op, int root, MPI_Comm comm);
#endif
