/*
 * Two-process MPI stand-in (see mpi.h): MPI_Sendrecv writes its message to
 * the peer's socket from a helper thread while it reads the peer's message,
 * so two ranks that send to each other at once cannot block each other.
 * Test infrastructure only.
 */
#include <pthread.h>
#include <string.h>
#include <unistd.h>
#include "mpi.h"

static int g_rank = 0, g_size = 1, g_fd = -1;

void c3d_stub_mpi_init(int rank, int size, int fd) {
  g_rank = rank;
  g_size = size;
  g_fd = fd;
}

int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  if (comm == MPI_COMM_NULL) return 1;
  *rank = g_rank;
  return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int *size) {
  if (comm == MPI_COMM_NULL) return 1;
  *size = g_size;
  return MPI_SUCCESS;
}

typedef struct {
  const char *p;
  size_t n;
  int rc;
} job_t;

static void *writer(void *arg) {
  job_t *j = (job_t *)arg;
  while (j->n > 0) {
    const ssize_t w = write(g_fd, j->p, j->n);
    if (w <= 0) { j->rc = 1; return NULL; }
    j->p += w;
    j->n -= (size_t)w;
  }
  return NULL;
}

int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status) {
  (void)sendtag; (void)recvtag; (void)status;
  if (comm == MPI_COMM_NULL || sendtype != MPI_BYTE || recvtype != MPI_BYTE || sendcount < 0 || recvcount < 0)
    return 1;
  if ((dest != MPI_PROC_NULL && (dest < 0 || dest >= g_size)) ||
      (source != MPI_PROC_NULL && (source < 0 || source >= g_size)))
    return 1;
  if (dest == g_rank && source == g_rank) {
    memcpy(recvbuf, sendbuf, (size_t)(sendcount < recvcount ? sendcount : recvcount));
    return MPI_SUCCESS;
  }
  if (dest == g_rank || source == g_rank) return 1; /* half a self-exchange: not used */
  job_t j = {(const char *)sendbuf, dest == MPI_PROC_NULL ? 0 : (size_t)sendcount, 0};
  pthread_t th;
  const int threaded = j.n > 0;
  if (threaded && pthread_create(&th, NULL, writer, &j) != 0) return 1;
  int rc = MPI_SUCCESS;
  size_t want = source == MPI_PROC_NULL ? 0 : (size_t)recvcount;
  char *q = (char *)recvbuf;
  while (want > 0) {
    const ssize_t r = read(g_fd, q, want);
    if (r <= 0) { rc = 1; break; }
    q += r;
    want -= (size_t)r;
  }
  if (threaded) pthread_join(th, NULL);
  return rc != MPI_SUCCESS ? rc : j.rc;
}
