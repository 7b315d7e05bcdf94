/*
 * Implementations behind the single-rank MPI, SimpleDecomp and FFTW stand-ins
 * (see mpi.h, sdecomp.h, fftw3.h in this directory), plus a few helpers that
 * let a test harness drive the reference solver's own operators through
 * ctypes without its file-I/O layer.
 *
 * Test infrastructure only: linked into oracle/_ref with the reference's
 * unmodified time-step sources.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <mpi.h>
#include <sdecomp.h>
#include <fftw3.h>
#include "../dct.h"

/* ---------------- MPI, one rank ---------------- */
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }
int MPI_Abort(MPI_Comm comm, int code) { (void)comm; fprintf(stderr, "MPI_Abort(%d)\n", code); exit(1); }
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm) {
  (void)op; (void)comm;
  if (sendbuf != MPI_IN_PLACE) memcpy(recvbuf, sendbuf, (size_t)count * (size_t)type);
  return 0;
}
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm) {
  (void)root;
  return MPI_Allreduce(sendbuf, recvbuf, count, type, op, comm);
}
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)type; (void)root; (void)comm; return 0;
}
int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype *newtype) {
  *newtype = (MPI_Datatype)count * oldtype; return 0;
}
int MPI_Type_commit(MPI_Datatype *type) { (void)type; return 0; }
int MPI_Type_free(MPI_Datatype *type) { *type = MPI_DATATYPE_NULL; return 0; }
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status) {
  (void)sendtag; (void)recvtag; (void)comm; (void)status; (void)recvcount; (void)recvtype;
  if (dest == MPI_PROC_NULL || source == MPI_PROC_NULL) return 0;
  /* one rank: the message goes to ourselves */
  memmove(recvbuf, sendbuf, (size_t)sendcount * (size_t)sendtype);
  return 0;
}
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1.e-9 * (double)ts.tv_nsec;
}

/* ---------------- SimpleDecomp, one rank ---------------- */
struct sdecomp_info_t_ { int dummy; };
struct sdecomp_transpose_plan_t_ {
  sdecomp_pencil_t from, to;
  size_t nx, ny, size;
};
static struct sdecomp_info_t_ g_info;

static int sd_construct(const MPI_Comm comm, const size_t ndims, const size_t *dims,
                        const bool *periods, sdecomp_info_t **info) {
  (void)comm; (void)ndims; (void)dims; (void)periods;
  *info = &g_info;
  return 0;
}
static int sd_destruct(sdecomp_info_t *info) { (void)info; return 0; }
static int sd_get_comm_cart(const sdecomp_info_t *info, MPI_Comm *comm) { (void)info; *comm = MPI_COMM_WORLD; return 0; }
static int sd_get_comm_rank(const sdecomp_info_t *info, int *rank) { (void)info; *rank = 0; return 0; }
static int sd_get_neighbours(const sdecomp_info_t *info, const sdecomp_pencil_t pencil,
                             const sdecomp_dir_t dir, int neighbours[2]) {
  (void)info; (void)pencil;
  if (dir == SDECOMP_XDIR) { neighbours[0] = MPI_PROC_NULL; neighbours[1] = MPI_PROC_NULL; }
  else { neighbours[0] = 0; neighbours[1] = 0; }
  return 0;
}
static int sd_get_pencil_mysize(const sdecomp_info_t *info, const sdecomp_pencil_t pencil,
                                const sdecomp_dir_t dir, const size_t glsize, size_t *mysize) {
  (void)info; (void)pencil; (void)dir; *mysize = glsize; return 0;
}
static int sd_get_pencil_offset(const sdecomp_info_t *info, const sdecomp_pencil_t pencil,
                                const sdecomp_dir_t dir, const size_t glsize, size_t *offset) {
  (void)info; (void)pencil; (void)dir; (void)glsize; *offset = 0; return 0;
}
static int sd_tr_construct(const sdecomp_info_t *info, const sdecomp_pencil_t from,
                           const sdecomp_pencil_t to, const size_t *glsizes,
                           const size_t size, sdecomp_transpose_plan_t **plan) {
  (void)info;
  sdecomp_transpose_plan_t *p = calloc(1, sizeof(*p));
  if (!p) return 1;
  p->from = from; p->to = to; p->nx = glsizes[0]; p->ny = glsizes[1]; p->size = size;
  *plan = p;
  return 0;
}
static int sd_tr_execute(sdecomp_transpose_plan_t *p, const void *sendbuf, void *recvbuf) {
  const char *s = sendbuf;
  char *r = recvbuf;
  const size_t nx = p->nx, ny = p->ny, sz = p->size;
  if (p->from == SDECOMP_X1PENCIL && p->to == SDECOMP_Y1PENCIL) {
    for (size_t j = 0; j < ny; j++)
      for (size_t i = 0; i < nx; i++)
        memcpy(r + sz * (i * ny + j), s + sz * (j * nx + i), sz);
  } else if (p->from == SDECOMP_Y1PENCIL && p->to == SDECOMP_X1PENCIL) {
    for (size_t i = 0; i < nx; i++)
      for (size_t j = 0; j < ny; j++)
        memcpy(r + sz * (j * nx + i), s + sz * (i * ny + j), sz);
  } else {
    memcpy(r, s, sz * nx * ny);
  }
  return 0;
}
static int sd_tr_destruct(sdecomp_transpose_plan_t *p) { free(p); return 0; }

const sdecomp_t sdecomp = {
  .construct = sd_construct,
  .destruct = sd_destruct,
  .get_comm_cart = sd_get_comm_cart,
  .get_comm_rank = sd_get_comm_rank,
  .get_neighbours = sd_get_neighbours,
  .get_pencil_mysize = sd_get_pencil_mysize,
  .get_pencil_offset = sd_get_pencil_offset,
  .transpose = {
    .construct = sd_tr_construct,
    .execute = sd_tr_execute,
    .destruct = sd_tr_destruct,
  },
};

/* ---------------- FFTW r2r subset ---------------- */
struct sbfs_fftw_plan_s {
  int n, howmany, istride, idist, ostride, odist;
  fftw_r2r_kind kind;
  double *in, *out;
  sbfs_dct_plan *dct;
};

fftw_plan fftw_plan_many_r2r(int rank, const int *n, int howmany,
                             double *in, const int *inembed, int istride, int idist,
                             double *out, const int *onembed, int ostride, int odist,
                             const fftw_r2r_kind *kind, unsigned flags) {
  (void)inembed; (void)onembed; (void)flags;
  if (rank != 1) return NULL;
  if (kind[0] != FFTW_REDFT10 && kind[0] != FFTW_REDFT01) return NULL;
  struct sbfs_fftw_plan_s *p = calloc(1, sizeof(*p));
  if (!p) return NULL;
  p->n = n[0]; p->howmany = howmany;
  p->istride = istride; p->idist = idist; p->ostride = ostride; p->odist = odist;
  p->kind = kind[0]; p->in = in; p->out = out;
  p->dct = sbfs_dct_plan_create(n[0]);
  if (!p->dct) { free(p); return NULL; }
  return p;
}

void fftw_execute(const fftw_plan p) {
  const int n = p->n;
  double *work = malloc(sizeof(double) * 6 * (size_t)n);
  double *line = work + 4 * (size_t)n;
  double *res = work + 5 * (size_t)n;
  for (int m = 0; m < p->howmany; m++) {
    for (int k = 0; k < n; k++) line[k] = p->in[(size_t)m * p->idist + (size_t)k * p->istride];
    if (p->kind == FFTW_REDFT10) sbfs_dct2(p->dct, line, res, work);
    else sbfs_dct3(p->dct, line, res, work);
    for (int k = 0; k < n; k++) p->out[(size_t)m * p->odist + (size_t)k * p->ostride] = res[k];
  }
  free(work);
}

void fftw_destroy_plan(fftw_plan p) {
  if (!p) return;
  sbfs_dct_plan_destroy(p->dct);
  free(p);
}

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

/* ---------------- harness helper ---------------- */
/* an sdecomp_info_t handle for a domain_t assembled by the test harness */
void *sbfs_refshim_info(void) { return &g_info; }
