/*
 * File side of the single-rank stand-ins: MPI-IO (see mpi.h), the NPY header
 * reader / writer of snpyio.h, and harness entry points that drive the
 * reference's own logging (src/logging/) and statistics (src/statistics.c)
 * through ctypes.
 *
 * Test infrastructure only: linked into oracle/_ref with the reference's
 * unmodified sources.  Never part of the product library.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>
#include <snpyio.h>
#include "domain.h"
#include "fluid.h"
#include "interface.h"
#include "logging.h"
#include "statistics.h"

/* ---------------- MPI-IO, one rank ---------------- */
struct sbfs_mpi_file_s {
  FILE *fp;
  int bad;  /* a view that one rank cannot satisfy was requested */
};

int MPI_File_open(MPI_Comm comm, const char *filename, int amode, MPI_Info info, MPI_File *fh) {
  (void)comm; (void)info;
  const char *mode = (amode & MPI_MODE_RDONLY) ? "rb" : "r+b";
  FILE *fp = fopen(filename, mode);
  if (!fp && (amode & MPI_MODE_CREATE)) fp = fopen(filename, "w+b");
  if (!fp) return MPI_ERR_OTHER;
  struct sbfs_mpi_file_s *f = calloc(1, sizeof(*f));
  if (!f) { fclose(fp); return MPI_ERR_OTHER; }
  f->fp = fp;
  *fh = f;
  return MPI_SUCCESS;
}

int MPI_File_close(MPI_File *fh) {
  if (!fh || !*fh) return MPI_ERR_OTHER;
  fclose((*fh)->fp);
  free(*fh);
  *fh = NULL;
  return MPI_SUCCESS;
}

/* a subarray datatype is its extent; one that is not the whole array gets a
 * negative extent, which the file view turns into an error */
int MPI_Type_create_subarray(int ndims, const int sizes[], const int subsizes[], const int starts[], int order,
                             MPI_Datatype oldtype, MPI_Datatype *newtype) {
  (void)order;
  long n = 1;
  int whole = 1;
  for (int d = 0; d < ndims; d++) {
    n *= sizes[d];
    whole = whole && subsizes[d] == sizes[d] && starts[d] == 0;
  }
  *newtype = whole ? (MPI_Datatype)n * oldtype : (MPI_Datatype)-1;
  if (!whole) fprintf(stderr, "refshim: a file view of part of an array needs more than one rank\n");
  return whole ? MPI_SUCCESS : MPI_ERR_OTHER;
}

int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype, const char *datarep,
                      MPI_Info info) {
  (void)etype; (void)datarep; (void)info;
  if (filetype < 0) fh->bad = 1;
  return fseek(fh->fp, disp, SEEK_SET) == 0 ? MPI_SUCCESS : MPI_ERR_OTHER;
}

int MPI_File_read_all(MPI_File fh, void *buf, int count, MPI_Datatype type, MPI_Status *status) {
  (void)status;
  if (fh->bad) return MPI_ERR_OTHER;
  return fread(buf, (size_t)type, (size_t)count, fh->fp) == (size_t)count ? MPI_SUCCESS : MPI_ERR_OTHER;
}

int MPI_File_write_all(MPI_File fh, const void *buf, int count, MPI_Datatype type, MPI_Status *status) {
  (void)status;
  if (fh->bad) return MPI_ERR_OTHER;
  return fwrite(buf, (size_t)type, (size_t)count, fh->fp) == (size_t)count ? MPI_SUCCESS : MPI_ERR_OTHER;
}

int MPI_Error_string(int errorcode, char *string, int *resultlen) {
  *resultlen = snprintf(string, MPI_MAX_ERROR_STRING, "refshim MPI-IO error %d", errorcode);
  return MPI_SUCCESS;
}

/* ---------------- NPY headers ---------------- */
int snpyio_w_header(const size_t ndims, const size_t *shape, const char dtype[], const bool is_fortran_order,
                    FILE *fp, size_t *header_size) {
  char dict[512];
  char dims[256] = "";
  size_t at = 0;
  for (size_t d = 0; d < ndims; d++) {
    const int w = snprintf(dims + at, sizeof(dims) - at, "%s%zu", d ? ", " : "", shape[d]);
    if (w < 0 || (size_t)w >= sizeof(dims) - at) return 1;
    at += (size_t)w;
  }
  if (ndims == 1 && at + 1 < sizeof(dims)) strcat(dims, ",");
  const int n = snprintf(dict, sizeof(dict), "{'descr': %s, 'fortran_order': %s, 'shape': (%s), }", dtype,
                         is_fortran_order ? "True" : "False", dims);
  if (n < 0 || (size_t)n >= sizeof(dict)) return 1;
  /* magic (6) + version (2) + length (2) + dict + padding + '\n', to 64 bytes */
  const size_t total = ((size_t)n + 11 + 63) / 64 * 64;
  const size_t hlen = total - 10;
  unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, (unsigned char)(hlen & 0xff),
                           (unsigned char)(hlen >> 8)};
  if (fseek(fp, 0, SEEK_SET) != 0 || fwrite(pre, 1, 10, fp) != 10 || fwrite(dict, 1, (size_t)n, fp) != (size_t)n)
    return 1;
  for (size_t k = 10 + (size_t)n; k + 1 < total; k++)
    if (fputc(' ', fp) == EOF) return 1;
  if (fputc('\n', fp) == EOF) return 1;
  *header_size = total;
  return 0;
}

/* value of key in a header dict: a pointer just past "'key':" and blanks */
static const char *dict_value(const char *dict, const char *key) {
  char pat[64];
  snprintf(pat, sizeof(pat), "'%s':", key);
  const char *p = strstr(dict, pat);
  if (!p) return NULL;
  p += strlen(pat);
  while (*p == ' ') p++;
  return p;
}

int snpyio_r_header(size_t *ndims, size_t **shape, char **dtype, bool *is_fortran_order, FILE *fp,
                    size_t *header_size) {
  unsigned char pre[12];
  if (fseek(fp, 0, SEEK_SET) != 0 || fread(pre, 1, 10, fp) != 10) return 1;
  if (memcmp(pre, "\x93NUMPY", 6) != 0) return 1;
  size_t hlen = 0, lead = 10;
  if (pre[6] == 1) {
    hlen = (size_t)pre[8] | ((size_t)pre[9] << 8);
  } else if (pre[6] == 2 || pre[6] == 3) {
    if (fread(pre + 10, 1, 2, fp) != 2) return 1;
    hlen = (size_t)pre[8] | ((size_t)pre[9] << 8) | ((size_t)pre[10] << 16) | ((size_t)pre[11] << 24);
    lead = 12;
  } else {
    return 1;
  }
  char *dict = malloc(hlen + 1);
  if (!dict) return 1;
  if (fread(dict, 1, hlen, fp) != hlen) { free(dict); return 1; }
  dict[hlen] = '\0';
  int rc = 1;
  const char *d = dict_value(dict, "descr");
  const char *f = dict_value(dict, "fortran_order");
  const char *s = dict_value(dict, "shape");
  if (d && f && s && (*d == '\'' || *d == '"') && *s == '(') {
    const char *e = strchr(d + 1, *d);
    size_t n = 0, cap = 8;
    size_t *sh = malloc(cap * sizeof(size_t));
    if (e && sh) {
      char *dt = malloc((size_t)(e - d) + 2);
      if (dt) {
        memcpy(dt, d, (size_t)(e - d) + 1);
        dt[e - d + 1] = '\0';
        const char *p = s + 1;
        while (*p && *p != ')') {
          while (*p == ' ' || *p == ',') p++;
          if (*p == ')') break;
          char *q = NULL;
          const unsigned long long v = strtoull(p, &q, 10);
          if (q == p) break;
          if (n == cap) {
            size_t *t = realloc(sh, 2 * cap * sizeof(size_t));
            if (!t) break;
            sh = t;
            cap *= 2;
          }
          sh[n++] = (size_t)v;
          p = q;
        }
        if (*p == ')') {
          *ndims = n;
          *shape = sh;
          *dtype = dt;
          *is_fortran_order = strncmp(f, "True", 4) == 0;
          *header_size = lead + hlen;
          sh = NULL;
          rc = 0;
        } else {
          free(dt);
        }
      }
    }
    free(sh);
  }
  free(dict);
  return rc;
}

/* ---------------- harness entry points ---------------- */
/* the reference's seven monitor files (src/logging/main.c:68-108), appended
 * to output/log/ under the current directory */
int sbfs_refshim_log(const domain_t *domain, size_t step, double time, double dt, double wtime, const fluid_t *fluid,
                     const interface_t *interface) {
  logging.check_and_output(domain, step, time, dt, wtime, fluid, interface);
  return 0;
}

/* statistics (src/statistics.c): the constructor reads stat_rate and
 * stat_after from the environment; output writes
 * output/stat/step<10 digits>/ under the current directory */
int sbfs_refshim_stats_init(const domain_t *domain, double time) { return statistics.init(domain, time); }
int sbfs_refshim_stats_collect(const domain_t *domain, const fluid_t *fluid, const interface_t *interface) {
  return statistics.collect(domain, fluid, interface);
}
int sbfs_refshim_stats_output(const domain_t *domain, size_t step) { return statistics.output(domain, step); }
