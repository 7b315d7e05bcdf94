// Initialisation and .npy I/O of the drop-in library (host code).
//
// Reference counterparts: src/domain.c:23-222 (domain_init/domain_save),
// src/fluid/init.c:84-109 + src/fluid/save.c (fluid_init/fluid_save),
// src/interface/init.c:55-69 + src/interface/save.c (interface_init/
// interface_save), src/array.c:80-206 and src/fileio.c:268-508 (array
// load/dump, NPY files).  Arrays are stored as in the reference: C-order
// (ny, nx + x ghosts) '<f8' slabs without y ghost rows; scalars and small
// vectors '<f8' / '<u8'.  The NPY container follows numpy's published format
// description (magic "\x93NUMPY", version, little-endian header length, a
// Python-literal dict with descr / fortran_order / shape, padded so the data
// starts on a 64-byte boundary).  One process, so no MPI-IO.
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sbfs_gb300.h"

namespace sbfs {
// the library's last-error message (sbfs_api.cu): every entry point reports
// through sbfs_last_error()
void set_last_error(const char *msg);
}  // namespace sbfs

namespace {

int io_fail(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  sbfs::set_last_error(buf);
  fprintf(stderr, "sbfs: %s\n", buf);
  return 1;
}

std::string path_of(const char *dir, const char *name) {
  std::string d(dir);
  if (!d.empty() && d.back() != '/') d += '/';
  return d + name + ".npy";
}

// parse "{'descr': '<f8', 'fortran_order': False, 'shape': (a, b), }"
bool parse_header(const std::string &h, std::string &descr, bool &fortran, std::vector<size_t> &shape) {
  auto key = [&](const char *k) -> size_t {
    const size_t p = h.find(k);
    return p == std::string::npos ? p : h.find(':', p) + 1;
  };
  size_t p = key("'descr'");
  if (p == std::string::npos) return false;
  size_t q1 = h.find('\'', p), q2 = h.find('\'', q1 + 1);
  if (q1 == std::string::npos || q2 == std::string::npos) return false;
  descr = h.substr(q1 + 1, q2 - q1 - 1);
  p = key("'fortran_order'");
  if (p == std::string::npos) return false;
  while (p < h.size() && h[p] == ' ') ++p;
  fortran = h.compare(p, 4, "True") == 0;
  p = key("'shape'");
  if (p == std::string::npos) return false;
  size_t a = h.find('(', p), b = h.find(')', a);
  if (a == std::string::npos || b == std::string::npos) return false;
  shape.clear();
  std::string s = h.substr(a + 1, b - a - 1);
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && (s[i] == ' ' || s[i] == ',')) ++i;
    if (i >= s.size()) break;
    char *end = nullptr;
    const unsigned long long v = strtoull(s.c_str() + i, &end, 10);
    if (end == s.c_str() + i) return false;
    shape.push_back((size_t)v);
    i = (size_t)(end - s.c_str());
  }
  return true;
}

// read a whole .npy whose dtype and shape must match exactly
int npy_read(const char *dir, const char *name, const char *descr, const std::vector<size_t> &shape, size_t elsize,
             void *out) {
  const std::string fn = path_of(dir, name);
  FILE *fp = fopen(fn.c_str(), "rb");
  if (!fp) return io_fail("%s: %s", fn.c_str(), strerror(errno));
  unsigned char pre[10];
  if (fread(pre, 1, 8, fp) != 8 || memcmp(pre, "\x93NUMPY", 6) != 0) {
    fclose(fp);
    return io_fail("%s: not an NPY file", fn.c_str());
  }
  size_t hlen = 0;
  if (pre[6] == 1) {
    unsigned char l[2];
    if (fread(l, 1, 2, fp) != 2) {
      fclose(fp);
      return io_fail("%s: truncated header", fn.c_str());
    }
    hlen = (size_t)l[0] | ((size_t)l[1] << 8);
  } else if (pre[6] == 2 || pre[6] == 3) {
    unsigned char l[4];
    if (fread(l, 1, 4, fp) != 4) {
      fclose(fp);
      return io_fail("%s: truncated header", fn.c_str());
    }
    hlen = (size_t)l[0] | ((size_t)l[1] << 8) | ((size_t)l[2] << 16) | ((size_t)l[3] << 24);
  } else {
    fclose(fp);
    return io_fail("%s: unsupported NPY version %d", fn.c_str(), pre[6]);
  }
  std::string h(hlen, '\0');
  if (fread(&h[0], 1, hlen, fp) != hlen) {
    fclose(fp);
    return io_fail("%s: truncated header", fn.c_str());
  }
  std::string d;
  bool fortran = false;
  std::vector<size_t> sh;
  if (!parse_header(h, d, fortran, sh)) {
    fclose(fp);
    return io_fail("%s: malformed NPY header", fn.c_str());
  }
  // checks of the reference (src/fileio.c:199-225)
  if (d != descr) {
    fclose(fp);
    return io_fail("%s: dtype %s expected, %s obtained", fn.c_str(), descr, d.c_str());
  }
  if (fortran) {
    fclose(fp);
    return io_fail("%s: fortran order not accepted", fn.c_str());
  }
  if (sh != shape) {
    std::string want, got;
    for (size_t v : shape) want += std::to_string(v) + ",";
    for (size_t v : sh) got += std::to_string(v) + ",";
    fclose(fp);
    return io_fail("%s: shape (%s) expected, (%s) obtained", fn.c_str(), want.c_str(), got.c_str());
  }
  size_t n = 1;
  for (size_t v : shape) n *= v;
  if (fread(out, elsize, n, fp) != n) {
    fclose(fp);
    return io_fail("%s: data truncated", fn.c_str());
  }
  fclose(fp);
  return 0;
}

int npy_write(const char *dir, const char *name, const char *descr, const std::vector<size_t> &shape, size_t elsize,
              const void *data) {
  std::string sh;
  if (shape.empty()) sh = "()";
  else if (shape.size() == 1) sh = "(" + std::to_string(shape[0]) + ",)";
  else {
    sh = "(";
    for (size_t i = 0; i < shape.size(); ++i) sh += (i ? ", " : "") + std::to_string(shape[i]);
    sh += ")";
  }
  std::string h = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + sh + ", }";
  const size_t base = 10;
  size_t total = base + h.size() + 1;
  const size_t pad = (64 - total % 64) % 64;
  h += std::string(pad, ' ');
  h += '\n';
  const std::string fn = path_of(dir, name);
  FILE *fp = fopen(fn.c_str(), "wb");
  if (!fp) return io_fail("%s: %s", fn.c_str(), strerror(errno));
  const unsigned char pre[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  const unsigned char l[2] = {(unsigned char)(h.size() & 0xff), (unsigned char)(h.size() >> 8)};
  size_t n = 1;
  for (size_t v : shape) n *= v;
  const bool ok = fwrite(pre, 1, 8, fp) == 8 && fwrite(l, 1, 2, fp) == 2 && fwrite(h.data(), 1, h.size(), fp) == h.size() &&
                  fwrite(data, elsize, n, fp) == n;
  fclose(fp);
  return ok ? 0 : io_fail("%s: write failed", fn.c_str());
}

int get_env_double(const char *key, double *v) {
  const char *s = getenv(key);
  if (!s) return io_fail("%s not found", key);
  errno = 0;
  *v = strtod(s, nullptr);
  if (errno != 0) return io_fail("%s: invalid value as double", key);
  return 0;
}

int prepare(const domain_t *d, const int nadds[2][2], size_t size, array_t *a) {
  const size_t nx = d->mysizes[0], ny = d->mysizes[1];
  const size_t items = (nx + nadds[0][0] + nadds[0][1]) * (ny + nadds[1][0] + nadds[1][1]);
  a->size = size;
  a->nadds = static_cast<int(*)[2]>(calloc(2, sizeof(int[2])));
  if (!a->nadds) return io_fail("allocation failed");
  memcpy(a->nadds, nadds, sizeof(int[2][2]));
  a->datasize = items * size;
  a->data = calloc(items, size);
  if (!a->data) return io_fail("allocation of %zu bytes failed", items * size);
  return 0;
}

void release(array_t *a) {
  free(a->nadds);
  free(a->data);
  a->nadds = nullptr;
  a->data = nullptr;
}

// load the interior rows (x ghosts included) of a field (src/array.c:80-139)
int load_array(const domain_t *d, const char *dir, const char *name, array_t *a) {
  const size_t nx = d->mysizes[0], ny = d->mysizes[1];
  const int ax = a->nadds[0][0] + a->nadds[0][1];
  const size_t row = (nx + ax) * (a->size / sizeof(double));
  double *dst = static_cast<double *>(a->data) + (size_t)a->nadds[1][0] * row;
  return npy_read(dir, name, "<f8", {ny, nx + ax}, sizeof(double), dst);
}

int dump_array(const domain_t *d, const char *dir, const char *name, const array_t *a) {
  const size_t nx = d->mysizes[0], ny = d->mysizes[1];
  const int ax = a->nadds[0][0] + a->nadds[0][1];
  const size_t row = (nx + ax) * (a->size / sizeof(double));
  const double *src = static_cast<const double *>(a->data) + (size_t)a->nadds[1][0] * row;
  return npy_write(dir, name, "<f8", {ny, nx + ax}, sizeof(double), src);
}

// periodic y ghost rows of a freshly loaded field
void fill_ghost_rows(const domain_t *d, array_t *a) {
  const int ny = (int)d->mysizes[1];
  const int g0 = a->nadds[1][0], g1 = a->nadds[1][1];
  const size_t row = (d->mysizes[0] + a->nadds[0][0] + a->nadds[0][1]) * (a->size / sizeof(double));
  double *p = static_cast<double *>(a->data);
  for (int J = 1 - g0; J <= ny + g1; ++J) {
    if (J >= 1 && J <= ny) continue;
    const int src = ((J - 1) % ny + ny) % ny + 1;
    memcpy(p + (size_t)(J - 1 + g0) * row, p + (size_t)(src - 1 + g0) * row, sizeof(double) * row);
  }
}

// x boundary values (src/fluid/boundary/*.c, src/interface/boundary.c)
void bc_x(const domain_t *d, array_t *a, int kind) {
  const int nx = (int)d->mysizes[0], ny = (int)d->mysizes[1];
  const int ax0 = a->nadds[0][0], g0 = a->nadds[1][0];
  const size_t row = (size_t)(nx + ax0 + a->nadds[0][1]);
  double *p = static_cast<double *>(a->data);
  for (int J = 1; J <= ny; ++J) {
    double *r = p + (size_t)(J - 1 + g0) * row;
    auto at = [&](int I) -> double & { return r[I - 1 + ax0]; };
    if (kind == 0) {  // ux: impermeable walls
      at(1) = 0.;
      at(nx + 1) = 0.;
    } else if (kind == 1) {  // uy: wall velocity 0, vof: 0 outside
      at(0) = 0.;
      at(nx + 1) = 0.;
    } else {  // p, psi: Neumann
      at(0) = at(1);
      at(nx + 1) = at(nx);
    }
  }
  fill_ghost_rows(d, a);
}

const int N_UX[2][2] = {{0, 1}, {1, 1}}, N_UY[2][2] = {{1, 1}, {1, 1}}, N_P[2][2] = {{1, 1}, {1, 1}};
const int N_VISUX[2][2] = {{0, 1}, {1, 1}}, N_TXX[2][2] = {{0, 0}, {1, 1}}, N_TXY[2][2] = {{0, 1}, {1, 1}};
const int N_SRCUX[2][2] = {{-1, 0}, {0, 0}}, N_SRCUY[2][2] = {{0, 0}, {0, 0}}, N_VOF[2][2] = {{1, 1}, {2, 2}};
const int N_DVOF[2][2] = {{0, 1}, {1, 2}}, N_NORMAL[2][2] = {{0, 0}, {1, 1}};

}  // namespace

extern "C" {

int domain_init(const char dir[], domain_t *d) {
  memset(d, 0, sizeof(*d));
  size_t gl[2];
  double len[2];
  if (npy_read(dir, "glsizes", "<u8", {2}, sizeof(size_t), gl)) return 1;
  if (npy_read(dir, "lengths", "<f8", {2}, sizeof(double), len)) return 1;
  const size_t nx = gl[0], ny = gl[1];
  if (nx < 1 || ny < 1) return io_fail("empty grid");
  d->xf = static_cast<double *>(calloc(nx + 1, sizeof(double)));
  d->xc = static_cast<double *>(calloc(nx + 2, sizeof(double)));
  d->hxxf = static_cast<double *>(calloc(nx + 1, sizeof(double)));
  d->hxxc = static_cast<double *>(calloc(nx, sizeof(double)));
  d->jdxf = static_cast<double *>(calloc(nx + 1, sizeof(double)));
  d->jdxc = static_cast<double *>(calloc(nx, sizeof(double)));
  if (!d->xf || !d->xc || !d->hxxf || !d->hxxc || !d->jdxf || !d->jdxc) return io_fail("allocation failed");
  if (npy_read(dir, "xf", "<f8", {nx + 1}, sizeof(double), d->xf)) return 1;
  if (npy_read(dir, "xc", "<f8", {nx + 2}, sizeof(double), d->xc)) return 1;
  for (int k = 0; k < 2; ++k) {
    d->glsizes[k] = gl[k];
    d->mysizes[k] = gl[k];
    d->offsets[k] = 0;
    d->lengths[k] = len[k];
  }
  // scale factors and Jacobians (src/domain.c:100-144)
  d->hy = len[1] / ny;
  for (size_t i = 1; i <= nx + 1; ++i) d->hxxf[i - 1] = d->xc[i] - d->xc[i - 1];
  for (size_t i = 1; i <= nx; ++i) d->hxxc[i - 1] = d->xf[i] - d->xf[i - 1];
  for (size_t i = 1; i <= nx + 1; ++i) d->jdxf[i - 1] = d->hxxf[i - 1] * d->hy;
  for (size_t i = 1; i <= nx; ++i) d->jdxc[i - 1] = d->hxxc[i - 1] * d->hy;
  double lo = 1e300, hi = -1e300;
  for (size_t i = 0; i < nx; ++i) {
    lo = fmin(lo, d->hxxc[i]);
    hi = fmax(hi, d->hxxc[i]);
  }
  if (!(fabs(hi - lo) < 1.e-15)) return io_fail("x grid is not uniform, which is not allowed");
  d->info = nullptr;
  return 0;
}

int domain_save(const char dir[], const domain_t *d) {
  const size_t nx = d->glsizes[0];
  if (npy_write(dir, "glsizes", "<u8", {2}, sizeof(size_t), d->glsizes)) return 1;
  if (npy_write(dir, "lengths", "<f8", {2}, sizeof(double), d->lengths)) return 1;
  if (npy_write(dir, "xf", "<f8", {nx + 1}, sizeof(double), d->xf)) return 1;
  return npy_write(dir, "xc", "<f8", {nx + 2}, sizeof(double), d->xc);
}

int fluid_init(const char dir[], const domain_t *d, fluid_t *f) {
  memset(f, 0, sizeof(*f));
  if (prepare(d, N_UX, 8, &f->ux) || prepare(d, N_UY, 8, &f->uy) || prepare(d, N_P, 8, &f->p)) return 1;
  for (int n = 0; n < 2; ++n)
    if (prepare(d, N_P, 8, &f->psi[n]) || prepare(d, N_P, 8, &f->den[n])) return 1;
  if (prepare(d, N_VISUX, 8, &f->visux) || prepare(d, N_UY, 8, &f->visuy)) return 1;
  if (prepare(d, N_TXX, 8, &f->txx) || prepare(d, N_TXY, 8, &f->txy) || prepare(d, N_TXX, 8, &f->tyy)) return 1;
  for (int n = 0; n < 3; ++n)
    if (prepare(d, N_SRCUX, 8, &f->srcux[n]) || prepare(d, N_SRCUY, 8, &f->srcuy[n])) return 1;
  if (load_array(d, dir, "ux", &f->ux) || load_array(d, dir, "uy", &f->uy) || load_array(d, dir, "p", &f->p) ||
      load_array(d, dir, "psi", &f->psi[0]))
    return 1;
  bc_x(d, &f->ux, 0);
  bc_x(d, &f->uy, 1);
  bc_x(d, &f->p, 2);
  bc_x(d, &f->psi[0], 2);
  if (get_env_double("Re", &f->Re) || get_env_double("Fr", &f->Fr) || get_env_double("denr", &f->denr) ||
      get_env_double("visr", &f->visr))
    return 1;
  f->refden = fmin(1., f->denr);
  return 0;
}

int fluid_save(const char dir[], const domain_t *d, const fluid_t *f) {
  if (npy_write(dir, "Re", "<f8", {}, 8, &f->Re) || npy_write(dir, "Fr", "<f8", {}, 8, &f->Fr)) return 1;
  return dump_array(d, dir, "ux", &f->ux) || dump_array(d, dir, "uy", &f->uy) || dump_array(d, dir, "p", &f->p) ||
         dump_array(d, dir, "psi", &f->psi[0]);
}

int interface_init(const char dir[], const domain_t *d, interface_t *itf) {
  memset(itf, 0, sizeof(*itf));
  if (prepare(d, N_VOF, 8, &itf->vof) || prepare(d, N_SRCUX, 8, &itf->ifrcx) || prepare(d, N_SRCUY, 8, &itf->ifrcy) ||
      prepare(d, N_DVOF, 16, &itf->dvof) || prepare(d, N_NORMAL, 24, &itf->normal) || prepare(d, N_P, 8, &itf->curv) ||
      prepare(d, N_VISUX, 8, &itf->fluxx) || prepare(d, N_UY, 8, &itf->fluxy) ||
      prepare(d, N_SRCUY, 8, &itf->src[0]) || prepare(d, N_SRCUY, 8, &itf->src[1]))
    return 1;
  if (load_array(d, dir, "vof", &itf->vof)) return 1;
  bc_x(d, &itf->vof, 1);
  return get_env_double("We", &itf->We);
}

int interface_save(const char dir[], const domain_t *d, const interface_t *itf) {
  if (npy_write(dir, "We", "<f8", {}, 8, &itf->We)) return 1;
  return dump_array(d, dir, "vof", &itf->vof);
}

int sbfs_statistics_output(const char dir[], const domain_t *d) {
  const size_t nx = d->glsizes[0], ny = d->glsizes[1];
  std::vector<double> ux1(ny * (nx + 1)), uy1(ny * (nx + 2)), vof1(ny * (nx + 2));
  size_t num = 0;
  if (sbfs_statistics_fetch(ux1.data(), uy1.data(), vof1.data(), &num)) return io_fail("%s", sbfs_last_error());
  if (num == 0) return 0;  // nothing collected: nothing to save, as the reference
  if (npy_write(dir, "num", "<u8", {}, sizeof(size_t), &num)) return 1;
  if (domain_save(dir, d)) return 1;
  if (npy_write(dir, "ux1", "<f8", {ny, nx + 1}, 8, ux1.data())) return 1;
  if (npy_write(dir, "uy1", "<f8", {ny, nx + 2}, 8, uy1.data())) return 1;
  return npy_write(dir, "vof1", "<f8", {ny, nx + 2}, 8, vof1.data());
}

int sbfs_free_state(domain_t *d, fluid_t *f, interface_t *itf) {
  if (f) {
    array_t *fa[] = {&f->ux, &f->uy, &f->p, &f->psi[0], &f->psi[1], &f->den[0], &f->den[1], &f->visux, &f->visuy,
                     &f->txx, &f->txy, &f->tyy, &f->srcux[0], &f->srcux[1], &f->srcux[2], &f->srcuy[0],
                     &f->srcuy[1], &f->srcuy[2]};
    for (array_t *a : fa) release(a);
  }
  if (itf) {
    array_t *ia[] = {&itf->vof, &itf->ifrcx, &itf->ifrcy, &itf->dvof, &itf->normal, &itf->curv, &itf->fluxx,
                     &itf->fluxy, &itf->src[0], &itf->src[1]};
    for (array_t *a : ia) release(a);
  }
  if (d) {
    double **dp[] = {&d->xf, &d->xc, &d->hxxf, &d->hxxc, &d->jdxf, &d->jdxc};
    for (double **p : dp) {
      free(*p);
      *p = nullptr;
    }
  }
  return 0;
}

}  // extern "C"
