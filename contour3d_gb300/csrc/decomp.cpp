/*
 * decomp.cpp -- pencil decomposition, communicator and host-side array
 * extension.
 *
 *   sdecomp object     the subset of SimpleDecomp used by the reference
 *                      (call sites: src/contour3d/contour/extend.c:17-21,
 *                      161-180, 219-220; src/contour3d/output.c:98); not
 *                      built with -DCONTOUR3D_EXTERNAL_SDECOMP, where the
 *                      caller links the real SimpleDecomp
 *   c3d_comm_world     MPI_COMM_WORLD stand-in of builds without MPI: one
 *                      process, or the ranks of an installed point-to-point
 *                      transport
 *   c3d_extend_block   extend.c:150-282: local block + two halo layers from
 *                      each neighbour (x, then y, then z exchange, so edges
 *                      and corners arrive through the neighbours' halos),
 *                      clipped at the global boundary
 *   c3d_reduce_nearest output.c:10-30,82: the nearest-depth reduction to
 *                      rank 0, as a binary tree of pairwise exchanges
 *   write_ppm          output.c:113-148: the P6 file
 *
 * Every exchange is one pairwise send-and-receive (xfer): MPI_Sendrecv with
 * -DCONTOUR3D_USE_MPI (as extend.c:36-141 does), else the installed
 * transport's sendrecv.
 */
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "contour3d.h"
#include "contour3d_gb300.h"
#include "c3d_host.h"

#if defined(CONTOUR3D_EXTERNAL_SDECOMP) && !defined(CONTOUR3D_USE_MPI)
#error "-DCONTOUR3D_EXTERNAL_SDECOMP needs -DCONTOUR3D_USE_MPI (SimpleDecomp works on MPI communicators)"
#endif

#if defined(CONTOUR3D_USE_MPI)
/* exchanges and ranks through MPI; no transport to install */
extern "C" int contour3d_gb300_install_transport(const contour3d_gb300_transport_t *t) {
  if (!t) return 0;
  c3d::log_error("this library is built with MPI: exchanges use the decomposition's MPI communicator");
  return 1;
}

namespace {
int comm_rank_of(MPI_Comm c) {
  int r = 0;
  if (MPI_Comm_rank(c, &r) != MPI_SUCCESS) return 0;
  return r;
}
int comm_size_of(MPI_Comm c) {
  int n = 1;
  if (MPI_Comm_size(c, &n) != MPI_SUCCESS) return 1;
  return n;
}
}  // namespace
#else
struct c3d_comm_s {
  int size;
  int rank;
  bool has_transport;
  contour3d_gb300_transport_t t;
};

static c3d_comm_s g_world = {1, 0, false, {1, 0, nullptr, nullptr}};

extern "C" MPI_Comm c3d_comm_world(void) { return &g_world; }

extern "C" int contour3d_gb300_install_transport(const contour3d_gb300_transport_t *t) {
  if (!t) {
    g_world = {1, 0, false, {1, 0, nullptr, nullptr}};
    return 0;
  }
  if (t->size < 1 || t->rank < 0 || t->rank >= t->size || (t->size > 1 && !t->sendrecv)) {
    c3d::log_error("invalid transport (size %d, rank %d)", t->size, t->rank);
    return 1;
  }
  g_world.size = t->size;
  g_world.rank = t->rank;
  g_world.has_transport = t->size > 1;
  g_world.t = *t;
  return 0;
}

namespace {
int comm_rank_of(MPI_Comm c) { return c ? c->rank : 0; }
int comm_size_of(MPI_Comm c) { return c ? c->size : 1; }
}  // namespace
#endif

#if !defined(CONTOUR3D_EXTERNAL_SDECOMP)
struct sdecomp_info_t {
  MPI_Comm comm;
  int size, rank; /* of comm, when the decomposition was constructed */
  int p0, p1;     /* process grid shared by the two split directions */
  int c0, c1;     /* my coordinates in it */
  bool periods[3];
};
#endif

namespace {

#if !defined(CONTOUR3D_EXTERNAL_SDECOMP)

/* (number of processes, my coordinate) of `dir` in `pencil` */
void pencil_dir(const sdecomp_info_t *info, sdecomp_pencil_t pencil, sdecomp_dir_t dir, int *np, int *me) {
  /* undecomposed direction of each pencil, and which grid axis feeds the
     lower / higher remaining direction */
  const int undecomposed = (int)pencil % 3;
  const bool swap = (int)pencil >= 3;
  if ((int)dir == undecomposed) {
    *np = 1;
    *me = 0;
    return;
  }
  const int lower = undecomposed == 0 ? 1 : 0;
  const bool first_axis = ((int)dir == lower) != swap;
  *np = first_axis ? info->p0 : info->p1;
  *me = first_axis ? info->c0 : info->c1;
}

int s_construct(MPI_Comm comm, size_t ndims, const size_t dims[], const bool periods[], sdecomp_info_t **info) {
  if (!info || comm == MPI_COMM_NULL || (ndims != 3 && ndims != 2)) return 1;
  sdecomp_info_t *p = static_cast<sdecomp_info_t *>(calloc(1, sizeof(sdecomp_info_t)));
  if (!p) return 1;
  const int P = comm_size_of(comm);
  int p0 = 0;
  if (dims && ndims == 3 && dims[1] && dims[2] && (int)(dims[1] * dims[2]) == P) {
    p0 = (int)dims[1];
  } else {
    for (int d = 1; d * d <= P; d++)
      if (P % d == 0) p0 = d;
  }
  p->comm = comm;
  p->size = P;
  p->rank = comm_rank_of(comm);
  p->p0 = p0;
  p->p1 = P / p0;
  p->c0 = p->rank % p0;
  p->c1 = p->rank / p0;
  for (int d = 0; d < 3; d++) p->periods[d] = periods ? periods[d < (int)ndims ? d : 0] : false;
  *info = p;
  return 0;
}

int s_destruct(sdecomp_info_t *info) {
  free(info);
  return 0;
}

int s_comm_cart(const sdecomp_info_t *info, MPI_Comm *c) {
  *c = info ? info->comm : MPI_COMM_WORLD;
  return 0;
}

int s_comm_rank(const sdecomp_info_t *info, int *r) {
  *r = info ? info->rank : comm_rank_of(MPI_COMM_WORLD);
  return 0;
}

int s_nprocs(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, int *n) {
  int me;
  if (!info) { *n = 1; return 0; }
  pencil_dir(info, p, d, n, &me);
  return 0;
}

int s_myrank(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, int *r) {
  int np;
  if (!info) { *r = 0; return 0; }
  pencil_dir(info, p, d, &np, r);
  return 0;
}

int s_neighbours(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, int nb[2]) {
  nb[0] = nb[1] = MPI_PROC_NULL;
  if (!info) return 0;
  const int undecomposed = (int)p % 3;
  const bool periodic = info->periods[(int)d];
  if ((int)d == undecomposed) {
    /* one process along d: a periodic wrap leads back to myself */
    if (periodic) nb[0] = nb[1] = info->rank;
    return 0;
  }
  const bool swap = (int)p >= 3;
  const int lower = undecomposed == 0 ? 1 : 0;
  const bool first_axis = ((int)d == lower) != swap;
  const int np = first_axis ? info->p0 : info->p1;
  const int me = first_axis ? info->c0 : info->c1;
  for (int side = 0; side < 2; side++) {
    int c = me + (side ? 1 : -1);
    if (c < 0 || c >= np) {
      if (!periodic) continue;
      c = (c + np) % np;
    }
    nb[side] = first_axis ? c + info->p0 * info->c1 : info->c0 + info->p0 * c;
  }
  return 0;
}

void split(size_t n, int np, int r, size_t *my, size_t *off) {
  const size_t base = n / (size_t)np, rem = n % (size_t)np;
  *my = base + ((size_t)r < rem ? 1 : 0);
  *off = (size_t)r * base + ((size_t)r < rem ? (size_t)r : rem);
}

int s_mysize(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, size_t g, size_t *m) {
  int np = 1, me = 0;
  if (info) pencil_dir(info, p, d, &np, &me);
  size_t off;
  split(g, np, me, m, &off);
  return 0;
}

int s_offset(const sdecomp_info_t *info, sdecomp_pencil_t p, sdecomp_dir_t d, size_t g, size_t *o) {
  int np = 1, me = 0;
  if (info) pencil_dir(info, p, d, &np, &me);
  size_t my;
  split(g, np, me, &my, o);
  return 0;
}

#endif  // !CONTOUR3D_EXTERNAL_SDECOMP

/* one pairwise exchange through the communicator */
int xfer(MPI_Comm comm, const void *sbuf, size_t sbytes, int dest, void *rbuf, size_t rbytes, int src) {
  if (dest == MPI_PROC_NULL && src == MPI_PROC_NULL) return 0;
  const int me = comm_rank_of(comm);
  if (dest == me && src == me) {
    memcpy(rbuf, sbuf, rbytes < sbytes ? rbytes : sbytes);
    return 0;
  }
#if defined(CONTOUR3D_USE_MPI)
  /* MPI counts are int: pieces of at most 1 GiB; both partners of every
     exchange move the same byte count, so their piece sequences pair up */
  const size_t piece = (size_t)1 << 30;
  const size_t sb = dest == MPI_PROC_NULL ? 0 : sbytes, rb = src == MPI_PROC_NULL ? 0 : rbytes;
  size_t so = 0, ro = 0;
  do {
    const size_t sn = sb - so < piece ? sb - so : piece, rn = rb - ro < piece ? rb - ro : piece;
    const int rc = MPI_Sendrecv(sn ? static_cast<const char *>(sbuf) + so : nullptr, (int)sn, MPI_BYTE, dest, 3141,
                                rn ? static_cast<char *>(rbuf) + ro : nullptr, (int)rn, MPI_BYTE, src, 3141, comm,
                                MPI_STATUS_IGNORE);
    if (rc != MPI_SUCCESS) {
      c3d::log_error("rank %d: MPI_Sendrecv failed (send to %d, receive from %d; error %d)", me, dest, src, rc);
      return 1;
    }
    so += sn;
    ro += rn;
  } while (so < sb || ro < rb);
  return 0;
#else
  if (!comm->has_transport) {
    c3d::log_error("a peer rank was requested but no transport is installed");
    return 1;
  }
  const int rc = comm->t.sendrecv(comm->t.user, dest == MPI_PROC_NULL ? nullptr : sbuf,
                                  dest == MPI_PROC_NULL ? 0 : sbytes, dest,
                                  src == MPI_PROC_NULL ? nullptr : rbuf, src == MPI_PROC_NULL ? 0 : rbytes, src);
  if (rc != 0)
    c3d::log_error("rank %d: exchange failed (send to %d, receive from %d; transport returned %d)", comm->rank,
                   dest, src, rc);
  return rc != 0 ? 1 : 0;
#endif
}

}  // namespace

#if !defined(CONTOUR3D_EXTERNAL_SDECOMP)
extern "C" const sdecomp_t sdecomp = {
    s_construct, s_destruct, s_comm_cart, s_comm_rank, s_nprocs, s_myrank, s_neighbours, s_mysize, s_offset,
};
#endif

namespace c3d {

void log_error(const char *fmt, ...) {
  va_list a;
  va_start(a, fmt);
  fprintf(stderr, "[CONTOUR3D ERROR] ");
  vfprintf(stderr, fmt, a);
  fprintf(stderr, "\n");
  fflush(stderr);
  va_end(a);
}

/*
 * The header "P6\n<W> <H>\n255\n" and the W x H x 3 bytes, the same bytes as
 * the reference's fopen("w") + fwrite.  A regular file that already exists
 * is overwritten in place and then cut to the image's size instead of being
 * truncated first: a solver rewrites the same file every frame, and on ext4
 * the truncate-then-rewrite pattern makes close() start writing the new data
 * back (its auto_da_alloc safeguard), which took 6-7 ms per 1920 x 1080
 * frame against 0.8 ms in place on one host.  Other files (pipes, devices)
 * are written sequentially.
 */
int write_ppm(const char *fname, size_t W, size_t H, const uint8_t *rgb) {
  char hdr[64];
  const int hl = snprintf(hdr, sizeof hdr, "P6\n%zu %zu\n255\n", W, H);
  const size_t body = 3 * W * H;
  const int fd = open(fname, O_WRONLY | O_CREAT | O_CLOEXEC, 0666);
  if (fd < 0) {
    log_error("%s: %s", fname, strerror(errno));
    return 1;
  }
  struct stat st;
  const bool regular = fstat(fd, &st) == 0 && S_ISREG(st.st_mode);
  int err = 0;
  auto put = [&](const void *p, size_t n, off_t at) {
    const char *c = static_cast<const char *>(p);
    while (n > 0 && err == 0) {
      const ssize_t w = regular ? pwrite(fd, c, n, at) : write(fd, c, n);
      if (w < 0 && errno == EINTR) continue;
      if (w <= 0) {
        err = w < 0 ? errno : EIO;
        break;
      }
      c += w;
      n -= (size_t)w;
      at += w;
    }
  };
  put(hdr, (size_t)hl, 0);
  put(rgb, body, (off_t)hl);
  if (err == 0 && regular && ftruncate(fd, (off_t)hl + (off_t)body) != 0) err = errno;
  if (close(fd) != 0 && err == 0) err = errno;
  if (err != 0) {
    log_error("%s: %s", fname, strerror(err));
    return 1;
  }
  return 0;
}

int decomp_query(const sdecomp_info_t *info, const contour3d_contour_obj_t *obj, BlockInfo *b) {
  for (int d = 0; d < 3; d++) {
    const sdecomp_dir_t dir = (sdecomp_dir_t)d;
    if (sdecomp.get_pencil_mysize(info, obj->pencil, dir, obj->glsizes[d], &b->mysize[d]) ||
        sdecomp.get_pencil_offset(info, obj->pencil, dir, obj->glsizes[d], &b->offset[d])) {
      log_error("sdecomp.get_pencil_mysize failed");
      return 1;
    }
    sdecomp.get_nprocs(info, obj->pencil, dir, &b->nprocs[d]);
    sdecomp.get_myrank(info, obj->pencil, dir, &b->myrank[d]);
    sdecomp.get_neighbours(info, obj->pencil, dir, b->neighbours[d]);
  }
  b->single = b->nprocs[0] == 1 && b->nprocs[1] == 1 && b->nprocs[2] == 1;
  /* extension (extend.c:229-252): widen by 2 towards every neighbour rank,
     clip at the global boundary */
  for (int d = 0; d < 3; d++) {
    const bool clip_lo = b->myrank[d] == 0, clip_hi = b->myrank[d] == b->nprocs[d] - 1;
    b->ext_size[d] = b->mysize[d] + 4 - (clip_lo ? 2 : 0) - (clip_hi ? 2 : 0);
    b->ext_offset[d] = b->offset[d] - (clip_lo ? 0 : 2);
    b->clip_lo[d] = clip_lo;
  }
  return 0;
}

int extend_block(const sdecomp_info_t *info, const contour3d_contour_obj_t *obj, const BlockInfo &b, double *ext) {
  MPI_Comm comm = MPI_COMM_NULL;
  sdecomp.get_comm_cart(info, &comm);
  const size_t n = 2;
  const size_t tx = b.mysize[0] + 2 * n, ty = b.mysize[1] + 2 * n, tz = b.mysize[2] + 2 * n;
  std::vector<double> tmp(tx * ty * tz, 0.0);
  for (size_t k = 0; k < b.mysize[2]; k++)
    for (size_t j = 0; j < b.mysize[1]; j++)
      memcpy(&tmp[((k + n) * ty + (j + n)) * tx + n], obj->array + (k * b.mysize[1] + j) * b.mysize[0],
             sizeof(double) * b.mysize[0]);
  std::vector<double> sbuf, rbuf;
  /* x: two columns of every (y, z) row of the padded block */
  {
    const size_t cnt = n * ty * tz;
    sbuf.resize(cnt);
    rbuf.resize(cnt);
    for (int pass = 0; pass < 2; pass++) {
      const size_t so = pass == 0 ? tx - 2 * n : n, ro = pass == 0 ? 0 : tx - n;
      const int dest = b.neighbours[0][pass == 0 ? 1 : 0], src = b.neighbours[0][pass == 0 ? 0 : 1];
      size_t q = 0;
      for (size_t r = 0; r < ty * tz; r++)
        for (size_t i = 0; i < n; i++) sbuf[q++] = tmp[r * tx + so + i];
      if (xfer(comm, sbuf.data(), cnt * 8, dest, rbuf.data(), cnt * 8, src)) return 1;
      if (src != MPI_PROC_NULL) {
        q = 0;
        for (size_t r = 0; r < ty * tz; r++)
          for (size_t i = 0; i < n; i++) tmp[r * tx + ro + i] = rbuf[q++];
      }
    }
  }
  /* y: two full rows of every z plane */
  {
    const size_t cnt = n * tx * tz;
    sbuf.resize(cnt);
    rbuf.resize(cnt);
    for (int pass = 0; pass < 2; pass++) {
      const size_t so = pass == 0 ? ty - 2 * n : n, ro = pass == 0 ? 0 : ty - n;
      const int dest = b.neighbours[1][pass == 0 ? 1 : 0], src = b.neighbours[1][pass == 0 ? 0 : 1];
      size_t q = 0;
      for (size_t k = 0; k < tz; k++)
        for (size_t j = 0; j < n; j++)
          for (size_t i = 0; i < tx; i++) sbuf[q++] = tmp[(k * ty + so + j) * tx + i];
      if (xfer(comm, sbuf.data(), cnt * 8, dest, rbuf.data(), cnt * 8, src)) return 1;
      if (src != MPI_PROC_NULL) {
        q = 0;
        for (size_t k = 0; k < tz; k++)
          for (size_t j = 0; j < n; j++)
            for (size_t i = 0; i < tx; i++) tmp[(k * ty + ro + j) * tx + i] = rbuf[q++];
      }
    }
  }
  /* z: two full planes */
  {
    const size_t cnt = n * tx * ty;
    for (int pass = 0; pass < 2; pass++) {
      const size_t so = pass == 0 ? tz - 2 * n : n, ro = pass == 0 ? 0 : tz - n;
      const int dest = b.neighbours[2][pass == 0 ? 1 : 0], src = b.neighbours[2][pass == 0 ? 0 : 1];
      sbuf.assign(tmp.begin() + so * tx * ty, tmp.begin() + (so + n) * tx * ty);
      rbuf.resize(cnt);
      if (xfer(comm, sbuf.data(), cnt * 8, dest, rbuf.data(), cnt * 8, src)) return 1;
      if (src != MPI_PROC_NULL) memcpy(&tmp[ro * tx * ty], rbuf.data(), cnt * 8);
    }
  }
  /* clip (extend.c:262-278) */
  const size_t i0 = b.clip_lo[0] ? n : 0, j0 = b.clip_lo[1] ? n : 0, k0 = b.clip_lo[2] ? n : 0;
  size_t q = 0;
  for (size_t k = k0; k < k0 + b.ext_size[2]; k++)
    for (size_t j = j0; j < j0 + b.ext_size[1]; j++) {
      memcpy(ext + q, &tmp[(k * ty + j) * tx + i0], sizeof(double) * b.ext_size[0]);
      q += b.ext_size[0];
    }
  return 0;
}

int comm_size(MPI_Comm comm) { return comm == MPI_COMM_NULL ? 1 : comm_size_of(comm); }

int reduce_nearest(const sdecomp_info_t *info, PixelRec *px, size_t n) {
  MPI_Comm comm = MPI_COMM_NULL;
  sdecomp.get_comm_cart(info, &comm);
  const int P = comm_size(comm), r = comm == MPI_COMM_NULL ? 0 : comm_rank_of(comm);
  if (P == 1) return 0;
  std::vector<PixelRec> in(n);
  for (int s = 1; s < P; s <<= 1) {
    if (r % (2 * s) == s) {
      if (xfer(comm, px, n * sizeof(PixelRec), r - s, nullptr, 0, MPI_PROC_NULL)) return 1;
    } else if (r % (2 * s) == 0 && r + s < P) {
      if (xfer(comm, nullptr, 0, MPI_PROC_NULL, in.data(), n * sizeof(PixelRec), r + s)) return 1;
      /* output.c:18-29: keep the nearer pixel */
      for (size_t p = 0; p < n; p++)
        if (px[p].depth < in[p].depth) px[p] = in[p];
    }
  }
  return 0;
}

}  // namespace c3d

extern "C" int contour3d_gb300_extend(const sdecomp_info_t *info, const contour3d_contour_obj_t *obj,
                                      size_t sizes[3], size_t offsets[3], double *ext) {
  if (!obj) return 1;
  c3d::BlockInfo b;
  if (c3d::decomp_query(info, obj, &b)) return 1;
  for (int d = 0; d < 3; d++) {
    if (sizes) sizes[d] = b.ext_size[d];
    if (offsets) offsets[d] = b.ext_offset[d];
  }
  if (!ext) return 0;
  return c3d::extend_block(info, obj, b, ext);
}

extern "C" int contour3d_gb300_reduce_nearest(const sdecomp_info_t *info, double *depth, uint8_t *rgb,
                                              size_t num_pixels) {
  if (!info || (num_pixels && (!depth || !rgb))) {
    c3d::log_error("reduce_nearest: missing argument");
    return 1;
  }
  std::vector<c3d::PixelRec> px(num_pixels);
  for (size_t p = 0; p < num_pixels; p++) {
    px[p] = {};
    px[p].depth = depth[p];
    px[p].r = rgb[3 * p];
    px[p].g = rgb[3 * p + 1];
    px[p].b = rgb[3 * p + 2];
  }
  if (c3d::reduce_nearest(info, px.data(), num_pixels)) return 1;
  for (size_t p = 0; p < num_pixels; p++) {
    depth[p] = px[p].depth;
    rgb[3 * p] = px[p].r;
    rgb[3 * p + 1] = px[p].g;
    rgb[3 * p + 2] = px[p].b;
  }
  return 0;
}

extern "C" int c3d_write_ppm(const char *fname, size_t W, size_t H, const uint8_t *rgb) {
  return c3d::write_ppm(fname, W, H, rgb);
}
