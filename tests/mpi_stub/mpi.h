/*
 * A two-process stand-in for the MPI calls the library makes when it is built
 * with -DCONTOUR3D_USE_MPI (MPI_Comm_rank, MPI_Comm_size, MPI_Sendrecv).
 * Test infrastructure only: tests/test_mpi_build_cpu.py compiles the
 * library's host code against it to check that the MPI build compiles and
 * exchanges halos and pixels correctly.  The two ranks are a forked process
 * pair joined by a socket (mpi_stub.c).
 */
#if !defined(C3D_TEST_MPI_STUB_H)
#define C3D_TEST_MPI_STUB_H
#include <stddef.h>

#if defined(__cplusplus)
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int source, tag; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_PROC_NULL (-2)
#define MPI_BYTE 1
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status);

/* test set-up: this process is `rank` of `size` (1 or 2); `fd` reaches the peer */
void c3d_stub_mpi_init(int rank, int size, int fd);

#if defined(__cplusplus)
}
#endif
#endif
