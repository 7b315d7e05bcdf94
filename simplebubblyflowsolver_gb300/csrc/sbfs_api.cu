// C ABI of the GB300 time step: the reference solver's entry points
// (include/integrate.h, include/decide_dt.h, include/fluid_solver.h,
// include/interface_solver.h) on top of the kernels of sbfs_kernels.cu.
//
// One device context (grid, metrics, device buffers, stream, graphs) is kept
// per process and rebuilt when the grid changes; this replaces the
// reference's function-static solver state (src/fluid/compute_potential.c:
// 427-437, src/decide_dt.c:19-22).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "sbfs_gb300.h"
#include "sbfs_kernels.cuh"

using namespace sbfs;

namespace {

std::string g_err;

int fail(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return 1;
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) return fail("%s:%d %s: %s", __FILE__, __LINE__, #call,      \
                                       cudaGetErrorString(e_));                        \
  } while (0)

// RK3 coefficients (reference src/runge_kutta.c:8-15)
const double RK_A[3] = {32. / 60., 25. / 60., 45. / 60.};
const double RK_B[3] = {0. / 60., -17. / 60., -25. / 60.};
double rk_g(int k) { return RK_A[k] + RK_B[k]; }

int g_sync_mode = SBFS_SYNC_STATE;
int g_use_graphs = 1;
// strict-mode steps copy the state themselves when they can: 1 = any host
// memory the GPU addresses, 2 = registered memory only (as on a system
// without host page-table access), 0 = never
int g_host_link = 1;
bool g_link_used = false;  // the last integrate() did
// bumped whenever the library pins or unpins host arrays (or the caller says
// the host state changed): the registration of the linked arrays is looked at again
unsigned g_reg_epoch = 0;
double g_coef[3] = {-1., -1., -1.};

// extra cells of every field (reference include/array_macros/)
struct Layout {
  int ax0, ax1, ay0, ay1, nc;
};
const Layout L_UX{0, 1, 1, 1, 1}, L_UY{1, 1, 1, 1, 1}, L_P{1, 1, 1, 1, 1}, L_DEN{1, 1, 1, 1, 1};
const Layout L_VISUX{0, 1, 1, 1, 1}, L_VISUY{1, 1, 1, 1, 1}, L_TXX{0, 0, 1, 1, 1}, L_TXY{0, 1, 1, 1, 1};
const Layout L_TYY{0, 0, 1, 1, 1}, L_SRCUX{-1, 0, 0, 0, 1}, L_SRCUY{0, 0, 0, 0, 1}, L_VOF{1, 1, 2, 2, 1};
const Layout L_IFRCX{-1, 0, 0, 0, 1}, L_IFRCY{0, 0, 0, 0, 1}, L_DVOF{0, 1, 1, 2, 2}, L_NORMAL{0, 0, 1, 1, 3};
const Layout L_CURV{1, 1, 1, 1, 1}, L_FLUXX{0, 1, 1, 1, 1}, L_FLUXY{1, 1, 1, 1, 1}, L_SRC{0, 0, 0, 0, 1};

struct Ctx {
  int nx = 0, ny = 0;
  int nc = 1;     // cases on this grid (batches); every field holds nc case slabs
  int kcase = 0;  // case slab that h2d / d2h address
  Phys *phys_dev = nullptr;  // per-case physics (batches)
  std::vector<Phys> phys_host;
  double lx = 0., ly = 0.;
  Grid g{};
  Metrics m{};
  Phys ph{};
  Bufs b{};
  cudaStream_t s = nullptr;
  std::vector<void *> allocs;
  std::vector<double> hxxf;  // host copy used to detect a changed grid
  double Re = NAN;
  double dt_fixed = 0.;
  double *small_host = nullptr;  // pinned: scalars block read back
  // metrics arrays (device)
  double *met = nullptr;
  // role state of the fused step: current velocity, potential, density,
  // RK-source buffers
  double *U[2], *V[2], *PSI[2], *DEN[2], *SX[2], *SY[2], *SV[2];
  // CSF force buffers: substage k uses IFX[k & 1], IFY[k & 1] (the last
  // substage's in b.ifrcx, b.ifrcy, the reference's arrays)
  double *IFX[3], *IFY[3];
  double *VOF0 = nullptr;  // the first vof buffer (which of the two holds the current vof keys the graphs)
  int iu = 0, ipsi = 0, iden = 0, isrc = 0;
  bool resident = false;  // device holds the current state
  bool tuned = false;     // launch shapes picked by the autotuner
  std::map<int, cudaGraphExec_t> graphs;
  // kernel arguments the graphs were captured with (physics, fixed dt, dt
  // safety factor); graphs are dropped when any of them changes
  std::vector<double> graph_sig;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  // side stream of the step: decide_dt beside k_props and the interface
  // kernels, the bulk fluxes and the force beside the listed interface
  // faces, the next substage's k_props beside the predictor, the Poisson
  // solve and the correction (fork / join events)
  cudaStream_t s2 = nullptr;
  cudaEvent_t evf = nullptr, evd = nullptr, evp = nullptr, evx = nullptr, evF = nullptr;
  bool props_ahead = false;  // the next substage's k_props is already on the side stream
  bool geo_ahead = false;    // the next substage's interface geometry and force are already on the side stream
  // device-resident steps: the last step formed the next step's first-substage
  // geometry and force (into IFX[2]) from its final vof and density, for the
  // configuration geo_next_cfg; any change of the state or of that
  // configuration clears it (state_touched)
  bool geo_next = false;
  unsigned long long geo_next_cfg = 0;
  // this step: its first substage's geometry came from the last step
  // (pre_first), it forms the next step's (make_next); set by launch_step
  bool pre_first = false, make_next = false;
  // host-linked step (strict sync mode, host arrays the GPU can address): the
  // step copies the state in and out itself, on the copy stream s3, each
  // field as early as the step allows.  link_tab: page-locked table of the
  // caller's arrays as the GPU addresses them (HL_* slots), read by the copy
  // kernels; link_host: the same arrays' host addresses, for the copy-engine
  // copies (baked into a captured graph: graph_hosts keeps them per graph)
  bool link = false;
  cudaStream_t s3 = nullptr;
  cudaEvent_t evh[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // vof, velocity, p, psi in; fork
  double **link_tab = nullptr, **link_tab_dev = nullptr;
  std::vector<const void *> link_host;
  // which of link_host are page-locked (bit per slot), for the arrays and the
  // registration epoch it was found for: a captured copy-engine copy depends on
  // it, so a linked graph is captured again when it changes
  std::vector<const void *> link_prev;
  unsigned link_epoch = ~0u;
  uintptr_t link_reg = 0;
  std::map<int, std::vector<const void *>> graph_hosts;
  // diagnostics partials / result and statistics sums (allocated on first use)
  double *diag_part = nullptr, *diag_out = nullptr;
  double *st_ux1 = nullptr, *st_uy1 = nullptr, *st_vof1 = nullptr;
  size_t st_num = 0;

  ~Ctx() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    for (void *p : allocs) cudaFree(p);
    if (small_host) cudaFreeHost(small_host);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (evf) cudaEventDestroy(evf);
    if (evd) cudaEventDestroy(evd);
    if (evp) cudaEventDestroy(evp);
    if (evx) cudaEventDestroy(evx);
    if (evF) cudaEventDestroy(evF);
    for (cudaEvent_t e : evh)
      if (e) cudaEventDestroy(e);
    if (link_tab) cudaFreeHost(link_tab);
    if (s3) cudaStreamDestroy(s3);
    if (s2) cudaStreamDestroy(s2);
    if (s) cudaStreamDestroy(s);
  }
};

std::unique_ptr<Ctx> g_ctx;

}  // namespace

namespace sbfs {
void set_last_error(const char *msg) { g_err = msg; }
}  // namespace sbfs

namespace {

int dalloc(Ctx &c, double **p, size_t n) {
  void *q = nullptr;
  CK(cudaMalloc(&q, n * sizeof(double)));
  CK(cudaMemsetAsync(q, 0, n * sizeof(double), c.s));
  c.allocs.push_back(q);
  *p = static_cast<double *>(q);
  return 0;
}

bool layout_ok(const array_t &a, const Layout &l) {
  if (!a.nadds || !a.data) return false;
  return a.nadds[0][0] == l.ax0 && a.nadds[0][1] == l.ax1 && a.nadds[1][0] == l.ay0 && a.nadds[1][1] == l.ay1 &&
         a.size == sizeof(double) * l.nc;
}

int pitch_of(const Ctx &c, const Layout &l) { return l.nc == 1 ? c.g.p1 : (l.nc == 2 ? c.g.p2 : c.g.p3); }

// start of case slab c.kcase of a device field
size_t case_off(const Ctx &c, const Layout &l) {
  return (size_t)c.kcase * (l.nc == 1 ? c.g.cs1 : (l.nc == 2 ? c.g.cs2 : c.g.cs3));
}

// host array (reference layout, rows J = 1 - ay0 .. ny + ay1) -> device rows J = 1..ny
int h2d(Ctx &c, const array_t &a, const Layout &l, double *dev) {
  if (!layout_ok(a, l)) return fail("array layout does not match the reference's (nadds/size)");
  const size_t row = (size_t)(c.nx + l.ax0 + l.ax1) * l.nc;
  const double *src = static_cast<const double *>(a.data) + (size_t)l.ay0 * row;
  dev += case_off(c, l);
  CK(cudaMemcpy2DAsync(dev, sizeof(double) * pitch_of(c, l), src, sizeof(double) * row, sizeof(double) * row, c.ny,
                       cudaMemcpyHostToDevice, c.s));
  return 0;
}

// device rows -> host array, ghost rows filled from the periodic images
int d2h(Ctx &c, array_t &a, const Layout &l, const double *dev) {
  if (!layout_ok(a, l)) return fail("array layout does not match the reference's (nadds/size)");
  const size_t row = (size_t)(c.nx + l.ax0 + l.ax1) * l.nc;
  const size_t pitch = sizeof(double) * pitch_of(c, l);
  double *dst = static_cast<double *>(a.data);
  dev += case_off(c, l);
  CK(cudaMemcpy2DAsync(dst + (size_t)l.ay0 * row, sizeof(double) * row, dev, pitch, sizeof(double) * row, c.ny,
                       cudaMemcpyDeviceToHost, c.s));
  for (int J = 1 - l.ay0; J <= c.ny + l.ay1; ++J) {
    if (J >= 1 && J <= c.ny) continue;
    int r = J - 1;
    while (r < 0) r += c.ny;
    while (r >= c.ny) r -= c.ny;
    CK(cudaMemcpyAsync(dst + (size_t)(J - 1 + l.ay0) * row, reinterpret_cast<const char *>(dev) + pitch * r,
                       sizeof(double) * row, cudaMemcpyDeviceToHost, c.s));
  }
  return 0;
}

int sync(Ctx &c) {
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c.s));
  return 0;
}

int load_coefs() {
  if (g_coef[0] >= 0. && g_coef[1] >= 0. && g_coef[2] >= 0.) return 0;
  const char *keys[3] = {"coef_dt_adv", "coef_dt_dif", "coef_dt_int"};
  for (int k = 0; k < 3; ++k) {
    const char *v = getenv(keys[k]);
    if (!v) return fail("%s not found", keys[k]);
    g_coef[k] = strtod(v, nullptr);
  }
  return 0;
}

int check_domain(const domain_t *d) {
  if (!d || !d->hxxf || !d->hxxc || !d->jdxf || !d->jdxc) return fail("domain_t is not initialised");
  const long nx = (long)d->mysizes[0], ny = (long)d->mysizes[1];
  if (d->glsizes[0] != d->mysizes[0] || d->glsizes[1] != d->mysizes[1])
    return fail("domain is decomposed; this library runs the whole domain on one GPU");
  if (nx < 4 || nx > 8192) return fail("nx = %ld outside 4..8192", nx);
  if (ny < 8 || ny > 8192 || (ny & (ny - 1)) != 0) return fail("ny = %ld must be a power of two in 8..8192", ny);
  // the reference accepts uniform x grids only (src/domain.c:78-98, 213-219)
  double lo = 1e300, hi = -1e300;
  for (long i = 0; i < nx; ++i) {
    lo = fmin(lo, d->hxxc[i]);
    hi = fmax(hi, d->hxxc[i]);
  }
  if (!(fabs(hi - lo) < 1.e-15)) return fail("x grid is not uniform");
  return 0;
}

// per-column coefficients (see Metrics)
// (batches: one block of NCOL columns per case, Re[k] per case; the kernels
// offset the columns that depend on the case: nuf, nuc, c4nuc, c2nuf)
int upload_metrics(Ctx &c, const domain_t *d, const double *Re) {
  const int nx = c.nx, n = nx + 3;
  const double hy = d->hy;
  const double dx = d->hxxc[0];
  constexpr int NCOL = 15;
  std::vector<double> h(NCOL * (size_t)n * c.nc, 0.);
  for (int k = 0; k < c.nc; ++k) {
    const double nu = 1. / Re[k];
    auto A = [&](int q, int I) -> double & { return h[((size_t)k * NCOL + q) * n + I]; };
    for (int I = 1; I <= nx + 1; ++I) {
      const double hf = d->hxxf[I - 1];
      A(0, I) = 1. / hf;
      A(2, I) = 0.25 / hf;
      A(3, I) = 0.25 * dx / (hf * hy);
      A(4, I) = nu / hf;
      A(5, I) = hf;
      A(8, I) = 0.5 * (1. / hf);
      A(10, I) = dx / hf;
      A(12, I) = 2. * (nu / hf);
      A(14, I) = 0.5 * (hy / hf);
    }
    for (int I = 1; I <= nx; ++I) {
      const double ihc = 1. / d->hxxc[I - 1];
      A(1, I) = ihc;
      A(6, I) = nu * ihc;
      A(7, I) = 0.25 * ihc;
      A(9, I) = 0.5 * ihc;
      A(11, I) = 4. * (nu * ihc);
      A(13, I) = 2. * (hy * ihc);
    }
  }
  c.g.cm = c.nc > 1 ? NCOL * n : 0;
  if (!c.met) {
    if (dalloc(c, &c.met, h.size())) return 1;
  }
  CK(cudaMemcpyAsync(c.met, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.s));
  CK(cudaStreamSynchronize(c.s));
  const double *b = c.met;
  c.m.ihxxf = b + 0 * n;
  c.m.ihxxc = b + 1 * n;
  c.m.q4f = b + 2 * n;
  c.m.q4fy = b + 3 * n;
  c.m.nuf = b + 4 * n;
  c.m.hxxf = b + 5 * n;
  c.m.nuc = b + 6 * n;
  c.m.q4c = b + 7 * n;
  c.m.hihxxf = b + 8 * n;
  c.m.hihxxc = b + 9 * n;
  c.m.rq = b + 10 * n;
  c.m.c4nuc = b + 11 * n;
  c.m.c2nuf = b + 12 * n;
  c.m.c4nucs = b + 13 * n;
  c.m.c2nufs = b + 14 * n;
  c.Re = Re[0];
  return 0;
}

Phys phys_of(const fluid_t *f, const interface_t *itf) {
  Phys p{};
  p.denr = f->denr;
  p.visr = f->visr;
  p.refden = f->refden;
  p.den_lo = fmin(1., f->denr);
  p.den_hi = fmax(1., f->denr);
  p.vis_lo = fmin(1., f->visr);
  p.vis_hi = fmax(1., f->visr);
  p.grav = -1. / f->Fr / f->Fr;
  p.force_coef = itf ? 2. / (1. + f->denr) / itf->We : 0.;
  p.irefden = 1. / f->refden;
  p.nu = 1. / f->Re;
  p.dm1 = f->denr - 1.;
  p.vm1 = f->visr - 1.;
  p.hvm1 = 0.5 * p.vm1;
  p.hgrav = 0.5 * p.grav;
  p.qf = 0.25 * p.force_coef;
  p.rref2 = 2. * p.refden;
  return p;
}

// the constants of a case that depend on the grid
void finish_phys(Phys &p, const Grid &g) {
  p.nuy = p.nu * g.ihy;
  p.qfy = p.qf * g.ihy;
  p.nuy2 = 2. * p.nuy;
  p.nuy4 = 4. * p.nuy;
  p.vsx_c = p.vm1 * p.nuy2;
  p.vsx_c2 = p.hvm1 * p.nuy2;
  p.vsx_1 = p.nuy2;
  p.vsx_lo = p.vis_lo * p.nuy2;
  p.vsx_hi = p.vis_hi * p.nuy2;
  p.vsy_c2 = p.hvm1 * p.nuy4;
  p.vsy_1 = p.nuy4;
  p.vsy_lo = p.vis_lo * p.nuy4;
  p.vsy_hi = p.vis_hi * p.nuy4;
  p.inuy2 = 1. / p.nuy2;
  p.inuy4 = 1. / p.nuy4;
}

void set_phys(Ctx &c, const fluid_t *f, const interface_t *itf) {
  Phys p = phys_of(f, itf);
  finish_phys(p, c.g);
  // other physics: a first-substage geometry formed ahead is stale
  if (memcmp(&p, &c.ph, sizeof(Phys)) != 0) c.geo_next = false;
  c.ph = p;
}

double fixed_dt(const Ctx &c, const domain_t *d, const fluid_t *f, const interface_t *itf) {
  double hxmin = 1.79769313486231570e+308;
  for (int i = 2; i <= c.nx; ++i) hxmin = fmin(hxmin, d->hxxf[i - 1]);
  const double h[2] = {hxmin, d->hy};
  const double diffusivity = 1. / f->Re;
  const double tension = 1. / itf->We;
  const double pi = 3.1415926535897932384626433832;
  double out = 1.e300;
  for (int k = 0; k < 2; ++k) {
    double dif = fmin(1., f->denr / f->visr) / diffusivity * 0.5 / 2 * pow(h[k], 2.);
    dif *= g_coef[1];
    out = fmin(out, dif);
  }
  double cap = 1.;
  for (int k = 0; k < 2; ++k) cap = fmin(cap, sqrt(1. / tension / 4. / pi * pow(h[k], 3.)));
  cap *= g_coef[2];
  return fmin(out, cap);
}

// Thomas pivots of the x operator per y wavenumber, in the chunked layout of
// k_poisson_tdm, and the FFT twiddles
int upload_poisson(Ctx &c, const domain_t *d) {
  const int nx = c.nx, ny = c.ny, M1 = ny / 2 + 1;
  const double pi = 3.14159265358979323846;
  const double dx = d->lengths[0] / nx;
  const double offx = 1. / (dx * dx);
  const double offy = 1. / d->hy / d->hy;
  // Thomas pivots per wavenumber: x_i = w_i r_i - v_i x_{i-1} forward,
  // x_i -= v_i x_{i+1} backward
  std::vector<double> W((size_t)M1 * nx), V((size_t)M1 * nx);
  for (int m = 0; m < M1; ++m) {
    const double s = sin(pi * m / ny);
    const double lam = -4. * offy * s * s;
    double v_prev = 0.;
    for (int i = 0; i < nx; ++i) {
      const double diag = (i == 0 || i == nx - 1 ? -offx : -2. * offx) + lam;
      const double piv = diag - (i == 0 ? 0. : offx * v_prev);
      double w, v;
      if (i == nx - 1 && fabs(piv) < 1.e-10 * offx) {
        // singular mode (m = 0, Neumann-Neumann): pin the last unknown; the
        // kernel removes the mean afterwards
        w = 0.;
        v = 0.;
      } else {
        w = 1. / piv;
        v = offx * w;
      }
      W[(size_t)m * nx + i] = w;
      V[(size_t)m * nx + i] = v;
      v_prev = v;
    }
  }
  // chunked layouts for 1, 2 and 4 warps per system: fac[((m L + k) lanes + l)]
  // = (w, v, P, Q) of row l L + k, P and Q the cumulative products of -v
  // within the chunk (forward, backward); padding rows decouple and solve to 0
  for (int gi = 0; gi < 3; ++gi) {
    const int G = 1 << gi, lanes = 32 * G, L = tdm_chunk(nx, G), NP = lanes * L;
    std::vector<double> fac((size_t)M1 * NP * 4);
    std::vector<double> w(NP), v(NP), P(NP), Q(NP);
    for (int m = 0; m < M1; ++m) {
      for (int i = 0; i < NP; ++i) {
        w[i] = i < nx ? W[(size_t)m * nx + i] : 0.;
        v[i] = i < nx ? V[(size_t)m * nx + i] : 0.;
      }
      for (int l = 0; l < lanes; ++l) {
        const int s0 = l * L, e0 = s0 + L - 1;
        double acc = 1.;
        for (int i = s0; i <= e0; ++i) P[i] = acc *= -v[i];
        acc = 1.;
        for (int i = e0; i >= s0; --i) Q[i] = acc *= -v[i];
      }
      for (int i = 0; i < NP; ++i) {
        const int l = i / L, k = i % L;
        double *o = &fac[(((size_t)m * L + k) * lanes + l) * 4];
        o[0] = w[i];
        o[1] = v[i];
        o[2] = P[i];
        o[3] = Q[i];
      }
    }
    CK(cudaMemcpyAsync(c.b.tdm_fac[gi], fac.data(), fac.size() * sizeof(double), cudaMemcpyHostToDevice, c.s));
    // fac dies at the end of this iteration: wait for the copy
    CK(cudaStreamSynchronize(c.s));
  }
  // tw[m] = exp(-2 pi i m / ny), m = 0..M (the real-to-complex splits), then
  // the butterflies' W_M^e, e < M, forward and inverse: W_M^e = tw[2e] or
  // -tw[2e - M], the inverse its conjugate (exact sign flips of the same values)
  const int M = ny / 2;
  std::vector<double2> tw(M1 + 2 * (size_t)M);
  for (int m = 0; m < M1; ++m) tw[m] = make_double2(cos(2. * pi * m / ny), -sin(2. * pi * m / ny));
  for (int e = 0; e < M; ++e) {
    const double2 w = 2 * e <= M ? tw[2 * e] : make_double2(-tw[2 * e - M].x, -tw[2 * e - M].y);
    tw[M1 + e] = w;
    tw[M1 + M + e] = make_double2(w.x, -w.y);
  }
  CK(cudaMemcpyAsync(c.b.twiddle, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice, c.s));
  // the staging vectors die here: wait for the copies
  CK(cudaStreamSynchronize(c.s));
  return 0;
}

// device context for nc cases on the grid of d
int build_ctx(Ctx *c, const domain_t *d, int nc) {
  c->nc = nc;
  c->nx = (int)d->mysizes[0];
  c->ny = (int)d->mysizes[1];
  c->lx = d->lengths[0];
  c->ly = d->lengths[1];
  c->hxxf.assign(d->hxxf, d->hxxf + c->nx + 1);
  // the main and copy streams at the highest priority, the side stream at
  // the default (lowest): see g_stream_prio
  int prio_lo = 0, prio_hi = 0;
  CK(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
  CK(cudaStreamCreateWithPriority(&c->s, cudaStreamNonBlocking, prio_hi));
  CK(cudaEventCreate(&c->e0));
  CK(cudaStreamCreateWithPriority(&c->s2, cudaStreamNonBlocking, prio_lo));
  CK(cudaEventCreateWithFlags(&c->evf, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&c->evd, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&c->evp, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&c->evx, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&c->evF, cudaEventDisableTiming));
  CK(cudaStreamCreateWithPriority(&c->s3, cudaStreamNonBlocking, prio_hi));
  for (cudaEvent_t &e : c->evh) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CK(cudaHostAlloc(reinterpret_cast<void **>(&c->link_tab), sizeof(double *) * kLinkSlots * nc, cudaHostAllocMapped));
  CK(cudaHostGetDevicePointer(reinterpret_cast<void **>(&c->link_tab_dev), c->link_tab, 0));
  CK(cudaEventCreate(&c->e1));
  cudaError_t e = configure_kernels();
  if (e != cudaSuccess) return fail("configure_kernels: %s", cudaGetErrorString(e));
  Grid &g = c->g;
  g.nx = c->nx;
  g.ny = c->ny;
  auto rnd = [](int n) { return (n + 31) / 32 * 32; };
  g.p1 = rnd(c->nx + 2);
  g.p2 = rnd(2 * (c->nx + 1));
  g.p3 = rnd(3 * c->nx);
  g.hy = d->hy;
  g.ihy = 1. / d->hy;
  g.q4y = 0.25 * g.ihy;
  g.hihy = 0.5 * g.ihy;
  g.dx = d->hxxc[0];
  g.idx = 1. / d->hxxc[0];
  const size_t n1 = (size_t)g.p1 * g.ny, n2 = (size_t)g.p2 * g.ny, n3 = (size_t)g.p3 * g.ny;
  const int M1 = g.ny / 2 + 1;
  g.nc = nc;
  g.cs1 = n1;
  g.cs2 = n2;
  g.cs3 = n3;
  g.css = (size_t)c->nx * M1;
  g.cm = 0;
  g.ct = rnd(c->nx + 2);
  g.phys = nullptr;
  Bufs &b = c->b;
  b.tiles = default_tiles(c->ny);
  b.tiles.tdm_g = tdm_warps_for(c->nx, c->ny, nc);
  double **scal[] = {&b.ux, &b.uy, &b.p, &b.psi0, &b.psi1, &b.vof, &b.ux_star, &b.uy_star, &b.den0, &b.den1,
                     &b.visux, &b.visuy, &b.txx, &b.txy, &b.tyy, &b.curv, &b.ifrcx, &b.ifrcy, &b.fluxx, &b.fluxy,
                     &b.mfluxx, &b.mfluxy, &b.srcux[0], &b.srcux[1], &b.srcux[2], &b.srcuy[0], &b.srcuy[1],
                     &b.srcuy[2], &b.srcvof[0], &b.srcvof[1], &b.egx, &b.egy, &b.pxx, &b.pyy, &b.pxy, &b.pyx,
                     &b.ifrcx2, &b.ifrcy2, &b.vof_alt, &b.ifrcx3, &b.ifrcy3, &b.qx, &b.qy,
                     &b.rhofx, &b.rhofy, &b.dpsix, &b.dpsiy};
  for (double **p : scal)
    if (dalloc(*c, p, n1 * nc)) return 1;
  if (dalloc(*c, &b.dvof, n2 * nc)) return 1;
  if (dalloc(*c, &b.normal, n3 * nc)) return 1;
  double *tmp = nullptr;
  if (dalloc(*c, &tmp, 2 * (size_t)c->nx * M1 * nc)) return 1;
  b.spec = reinterpret_cast<double2 *>(tmp);
  for (int gi = 0; gi < 3; ++gi) {
    const int G = 1 << gi;
    if (dalloc(*c, &tmp, 4 * (size_t)32 * G * tdm_chunk(c->nx, G) * M1)) return 1;
    b.tdm_fac[gi] = reinterpret_cast<double2 *>(tmp);
  }
  b.tdm_stage = nullptr;
  if (const size_t ns = tdm_stage_doubles(c->nx, c->ny, nc, b.tiles.tdm_g))
    if (dalloc(*c, &b.tdm_stage, ns)) return 1;
  if (dalloc(*c, &tmp, 2 * ((size_t)M1 + 2 * (size_t)(c->ny / 2)))) return 1;
  b.twiddle = reinterpret_cast<double2 *>(tmp);
  if (dalloc(*c, &tmp, ((size_t)c->nx + 8) * nc)) return 1;
  b.dt_acc = reinterpret_cast<unsigned long long *>(tmp);
  if (dalloc(*c, &tmp, ((size_t)c->nx * c->ny * nc + 2) / 2 + 1)) return 1;
  b.ilist = reinterpret_cast<int *>(tmp);
  if (dalloc(*c, &tmp, (4 * (size_t)c->nx * c->ny * nc + 2) / 2 + 1)) return 1;
  b.flist = reinterpret_cast<int *>(tmp);
  if (dalloc(*c, &tmp, (size_t)nc + 1)) return 1;  // nc cell counts, then nc face counts
  b.icount = reinterpret_cast<int *>(tmp);
  b.fcount = b.icount + nc;
  if (dalloc(*c, &b.tf, (size_t)kThincTabs * c->nx * c->ny * nc)) return 1;
  // scalars of every case, then one status word per case
  if (dalloc(*c, &tmp, (size_t)kScalars * nc + nc / 2 + 2)) return 1;
  b.scalars = tmp;
  b.status = reinterpret_cast<int *>(tmp + (size_t)kScalars * nc);
  if (dalloc(*c, &b.coltab, (size_t)3 * kColTabs * g.ct * nc)) return 1;
  CK(cudaMallocHost(&c->small_host, sizeof(double) * ((size_t)kScalars * nc + nc / 2 + 2)));
  if (nc > 1) {
    void *q = nullptr;
    CK(cudaMalloc(&q, sizeof(Phys) * nc));
    c->allocs.push_back(q);
    c->phys_dev = static_cast<Phys *>(q);
    g.phys = c->phys_dev;
  }
  if (upload_poisson(*c, d)) return 1;
  c->U[0] = b.ux;
  c->U[1] = b.ux_star;
  c->V[0] = b.uy;
  c->V[1] = b.uy_star;
  c->PSI[0] = b.psi0;
  c->PSI[1] = b.psi1;
  c->DEN[0] = b.den0;
  c->DEN[1] = b.den1;
  c->SX[0] = b.srcux[0];
  c->SX[1] = b.srcux[1];
  c->SY[0] = b.srcuy[0];
  c->SY[1] = b.srcuy[1];
  c->SV[0] = b.srcvof[0];
  c->SV[1] = b.srcvof[1];
  c->IFX[0] = b.ifrcx;
  c->IFX[1] = b.ifrcx2;
  c->IFY[0] = b.ifrcy;
  c->IFY[1] = b.ifrcy2;
  c->IFX[2] = b.ifrcx3;
  c->IFY[2] = b.ifrcy3;
  c->VOF0 = b.vof;
  return 0;
}

int make_ctx(const domain_t *d) {
  g_ctx.reset();
  auto c = std::make_unique<Ctx>();
  if (build_ctx(c.get(), d, 1)) return 1;
  g_ctx = std::move(c);
  return 0;
}

// context for this domain and physics; rebuilt when the grid changes
Ctx *get_ctx(const domain_t *d, const fluid_t *f, const interface_t *itf) {
  if (check_domain(d)) return nullptr;
  Ctx *c = g_ctx.get();
  bool same_grid = c && c->nx == (int)d->mysizes[0] && c->ny == (int)d->mysizes[1] && c->lx == d->lengths[0] &&
                   c->ly == d->lengths[1] && c->g.hy == d->hy &&
                   memcmp(c->hxxf.data(), d->hxxf, sizeof(double) * (c->nx + 1)) == 0;
  if (!same_grid) {
    if (make_ctx(d)) return nullptr;
    c = g_ctx.get();
  }
  const double Re = f ? f->Re : (std::isnan(c->Re) ? 1. : c->Re);
  if (!c->met || !(c->Re == Re)) {
    if (upload_metrics(*c, d, &Re)) return nullptr;
  }
  if (f) set_phys(*c, f, itf);
  return c;
}

// scalars block for a fine-grained call: substage k of step size dt, and/or
// explicit dt_old / dt_new in slot 0 (the same expressions as the step kernel)
int put_scalars(Ctx &c, double dt, int k, double dt_old, double dt_new) {
  double *h = c.small_host;
  for (int i = 0; i < kScalars; ++i) h[i] = 0.;
  h[0] = dt;
  if (k >= 0) {
    h[sc_adt(k)] = RK_A[k] * dt;
    h[sc_bdt(k)] = RK_B[k] * dt;
    h[sc_gdt(k)] = rk_g(k) * dt;
    h[sc_adt2(k)] = 2. * (RK_A[k] * dt);
    h[sc_bdt2(k)] = 2. * (RK_B[k] * dt);
    h[sc_gdt2(k)] = 2. * (rk_g(k) * dt);
  }
  if (dt_new != 0.) {
    const Grid &g = c.g;
    h[sc_dtold(0)] = dt_old;
    h[sc_dtnew(0)] = dt_new;
    const double cdiv = c.ph.refden / dt_new * (0.5 / g.ny);
    const double cadd = -(dt_old / dt_new) * (0.5 / g.ny);
    h[sc_pdx(0)] = cdiv * g.idx;
    h[sc_pdy(0)] = cdiv * g.ihy;
    h[sc_pax(0)] = cadd * (g.idx * g.idx);
    h[sc_pay(0)] = cadd * (g.ihy * g.ihy);
    h[sc_cnew(0)] = dt_new * c.ph.irefden;
    h[sc_cold(0)] = -dt_old * c.ph.irefden;
    h[sc_cnewy(0)] = h[sc_cnew(0)] * g.ihy;
    h[sc_coldy(0)] = h[sc_cold(0)] * g.ihy;
    h[sc_coldyp(0)] = h[sc_coldy(0)] / h[sc_pay(0)];
    h[sc_rpx(0)] = c.ph.rref2 * h[sc_pax(0)];
    h[sc_rpy(0)] = c.ph.rref2 * h[sc_pay(0)];
    // the correction's per-column coefficients of slot 0, as k_decide_dt
    // writes them for the fused step
    std::vector<double> ct(2 * (size_t)g.ct, 0.);
    const double cop = h[sc_cold(0)] / h[sc_pax(0)];
    for (int I = 1; I <= c.nx + 1; ++I) {
      const double ih = 1. / c.hxxf[I - 1];
      ct[I] = h[sc_cnew(0)] * ih;
      ct[g.ct + I] = cop * ih;
    }
    CK(cudaMemcpyAsync(c.b.coltab + (size_t)ct_cnewx(0) * g.ct, ct.data(), sizeof(double) * ct.size(),
                       cudaMemcpyHostToDevice, c.s));
    CK(cudaStreamSynchronize(c.s));  // ct dies here
  }
  CK(cudaMemcpyAsync(c.b.scalars, h, sizeof(double) * kScalars, cudaMemcpyHostToDevice, c.s));
  // h is reused by the next call: wait for the copy
  CK(cudaStreamSynchronize(c.s));
  return 0;
}

void swap_data(array_t &a, array_t &b) {
  void *t = a.data;
  a.data = b.data;
  b.data = t;
}

// ---------------------------------------------------------------------------
// fused step
// ---------------------------------------------------------------------------

// optional per-kernel event timing of the fused step (eager launches only)
struct Prof {
  bool on = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  cudaEvent_t get() {
    if (used == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[used++];
  }
} g_prof;

enum KernelClass {
  KC_PROPS, KC_CURV_LIST, KC_INTERFACE, KC_FLUX_FORCE, KC_VOF_ADVANCE, KC_MOMFLUX, KC_PREDICT,
  KC_POISSON_FWD, KC_POISSON_TDM, KC_POISSON_INV, KC_CORRECT, KC_DECIDE_DT, KC_MLP_CURV,
  KC_CSF_FORCE, KC_FACE_FLUX, KC_BULK_FLUX, KC_COUNT
};
const char *kKernelNames[KC_COUNT] = {"k_props", "k_curv_list", "k_interface_cells", "k_flux_force", "k_vof_advance", "k_momflux",
                                      "k_predict_mf", "k_poisson_fwd", "k_poisson_tdm", "k_poisson_inv", "k_correct",
                                      "k_decide_dt", "k_mlp_curv", "k_csf_force", "k_face_flux", "k_bulk_flux"};

// 1: the interface geometry of a substage (curvature, interface-cell list,
// THINC factors, CSF force) runs ahead of its velocity, beside the previous
// substage's predictor and Poisson solve, and the VOF update forms the face
// fluxes itself (k_vof_advance_itf, into the second vof buffer); 0: after
// the correction, with the listed faces (k_curv_list<true>,
// k_interface_cells, k_flux_force) and the VOF update in place.  The same
// results bit for bit.
int g_geo_ahead = 1;

// curvature model of the fused step: 0 = the reference's kappa = -div n,
// 1 = the learned closure in interface cells (plain kappa outside its range)
int g_curv_model = 0;

// the configuration the next step's ahead geometry was formed for: the
// curvature model and the closure's parameters and range
unsigned long long geo_cfg() {
  return (unsigned long long)g_curv_model | ((unsigned long long)g_geo_ahead << 1) |
         ((unsigned long long)(g_sync_mode == SBFS_SYNC_ALL) << 2) | ((unsigned long long)g_mlp_epoch << 8);
}

// the fused step keeps its viscosities pre-scaled for k_momflux, except when
// every array is synchronised to the host (the reference's visux, visuy)
bool scaled_vis() { return g_sync_mode != SBFS_SYNC_ALL; }

// the device state or its configuration changes outside a step: a first
// substage geometry formed ahead by the last step is stale
void state_touched(Ctx &c) { c.geo_next = false; }


template <class F>
void timed(Ctx &c, int cls, F &&launch) {
  if (!g_prof.on) {
    launch();
    return;
  }
  cudaEvent_t a = g_prof.get(), b = g_prof.get();
  cudaEventRecord(a, c.s);
  launch();
  cudaEventRecord(b, c.s);
  g_prof.marks.push_back({cls, {a, b}});
}

// ---- host-linked step: slots of Ctx::link_tab, the arrays read at the start
// of the step and those written at its end (the psi pointers as the reference
// leaves them, swapped)
enum { HL_UX_IN, HL_UY_IN, HL_P_IN, HL_PSI_IN, HL_VOF_IN, HL_UX_OUT, HL_UY_OUT, HL_P_OUT, HL_PSI0_OUT, HL_PSI1_OUT,
       HL_VOF_OUT, HL_COUNT };

HostRows host_rows(const Ctx &c, int slot, const Layout &l, double *dev) {
  return HostRows{slot, c.nx + l.ax0 + l.ax1, l.ay0, l.ay1, dev};
}

// Copies that run beside the step's kernels go through the copy engines: a
// kernel copying over the CPU-GPU link slows the kernels sharing its SMs by
// about its own duration (measured on the bubble swarm).  Copies with nothing
// beside them are kernels on the whole GPU: they reach the link's full read
// rate.  A batch of many cases copies by kernels only (one launch for all its
// cases instead of a copy-engine call per case), beside the step on few blocks.
constexpr int kLinkWide = 2 * 152, kLinkNarrow = 64;

// copy-engine copy of a scalar field between a host array (slot) and its
// device rows; out also fills the host's y ghost rows from their periodic
// images
void link_dma(Ctx &c, bool in, int slot, const Layout &l, double *dev) {
  const size_t row = (size_t)c.nx + l.ax0 + l.ax1, pitch = sizeof(double) * c.g.p1;
  double *h = const_cast<double *>(static_cast<const double *>(c.link_host[slot]));
  if (in) {
    cudaMemcpy2DAsync(dev, pitch, h + (size_t)l.ay0 * row, sizeof(double) * row, sizeof(double) * row, c.ny,
                      cudaMemcpyHostToDevice, c.s3);
    return;
  }
  cudaMemcpy2DAsync(h + (size_t)l.ay0 * row, sizeof(double) * row, dev, pitch, sizeof(double) * row, c.ny,
                    cudaMemcpyDeviceToHost, c.s3);
  for (int J = 1 - l.ay0; J <= c.ny + l.ay1; ++J) {
    if (J >= 1 && J <= c.ny) continue;
    const int r = J < 1 ? J - 1 + c.ny : J - 1 - c.ny;
    cudaMemcpyAsync(h + (size_t)(J - 1 + l.ay0) * row, dev + (size_t)r * c.g.p1, sizeof(double) * row,
                    cudaMemcpyDeviceToHost, c.s3);
  }
}

// a copy beside the step's kernels, on the copy stream: by copy engine for a
// single case's page-locked array; by a narrow copy kernel for a batch (one
// launch for all its cases) and for pageable arrays, which the copy engines
// move with a fixed cost of several microseconds per call (13 calls a step
// with the ghost rows)
void link_side(Ctx &c, bool in, int slot, const Layout &l, double *dev) {
  if (c.nc == 1 && ((c.link_reg >> slot) & 1))
    link_dma(c, in, slot, l, dev);
  else
    launch_host_rows(c.s3, c.g, c.link_tab_dev, in, host_rows(c, slot, l, dev), HostRows{}, 1, kLinkNarrow);
}

// the copies in, on the copy stream in the order the step first needs them:
// vof (densities, viscosities, corner normals), the velocity (everything
// else of the interface chain), p (first predictor), psi (first Poisson
// right-hand side); rho^k as soon as vof is in
void link_in(Ctx &c) {
  cudaEventRecord(c.evh[4], c.s);
  cudaStreamWaitEvent(c.s3, c.evh[4], 0);
  launch_host_rows(c.s3, c.g, c.link_tab_dev, true, host_rows(c, HL_VOF_IN, L_VOF, c.b.vof), HostRows{}, 1,
                   kLinkWide);
  cudaEventRecord(c.evh[0], c.s3);
  launch_host_rows(c.s3, c.g, c.link_tab_dev, true, host_rows(c, HL_UX_IN, L_UX, c.U[c.iu]),
                   host_rows(c, HL_UY_IN, L_UY, c.V[c.iu]), 2, kLinkWide);
  cudaEventRecord(c.evh[1], c.s3);
  link_side(c, true, HL_P_IN, L_P, c.b.p);
  cudaEventRecord(c.evh[2], c.s3);
  link_side(c, true, HL_PSI_IN, L_P, c.PSI[c.ipsi]);
  cudaEventRecord(c.evh[3], c.s3);
  cudaStreamWaitEvent(c.s, c.evh[0], 0);
  launch_props(c.s, c.g, c.m, c.ph, c.b, true, false, false, c.DEN[c.iden]);
}

// a copy out on the copy stream, of a field the main stream has finished
void link_out(Ctx &c, int slot, const Layout &l, double *dev) {
  cudaEventRecord(c.evh[4], c.s);
  cudaStreamWaitEvent(c.s3, c.evh[4], 0);
  link_side(c, false, slot, l, dev);
}

// par: decide_dt runs on the side stream (forked by enqueue_step, joined
// before the first use of its scalars when wait_dt), and so does whatever
// does not wait for the main stream's latest result; the main stream waits
// for it before anything reads what it writes.  With the geometry ahead
// (g_geo_ahead, the default) the side stream runs:
//   * the bulk fluxes beside the listed faces (in substage 0 beside k_props
//     and the geometry too);
//   * in substage 0, the CSF force beside the listed faces, the VOF update
//     (which writes vof^{k+1} to the other vof buffer) and k_momflux;
//   * once k_momflux (the last reader of the viscosities and corner normals)
//     is enqueued, the next substage's k_props, geometry and CSF force (into
//     the other force buffer) from the new vof and density, beside this
//     substage's predictor, Poisson solve and correction.
// Otherwise (the first form): the bulk fluxes and the force beside the
// listed interface faces, the next substage's k_props ahead.
void enqueue_substage(Ctx &c, int k, bool par, bool wait_dt) {
  Bufs &b = c.b;
  if (k != 0) c.isrc ^= 1;  // stash the previous stage's sources (pointer swap)
  double *ux = c.U[c.iu], *uy = c.V[c.iu], *uxs = c.U[c.iu ^ 1], *uys = c.V[c.iu ^ 1];
  double *den0 = c.DEN[c.iden], *den1 = c.DEN[c.iden ^ 1];
  double *psio = c.PSI[c.ipsi], *psin = c.PSI[c.ipsi ^ 1];
  double *sxa = c.SX[c.isrc], *sxb = c.SX[c.isrc ^ 1];
  double *sya = c.SY[c.isrc], *syb = c.SY[c.isrc ^ 1];
  double *sva = c.SV[c.isrc], *svb = c.SV[c.isrc ^ 1];
  const double *sc = b.scalars;
  const bool learned = g_curv_model != 0;
  const bool ahead = g_geo_ahead != 0;
  // force buffers: substage k's IFX[k & 1], the first substage's IFX[2] when
  // the last step formed it
  const bool pre = ahead && k == 0 && c.pre_first;
  const int fb = pre ? 2 : (k & 1);
  double *ifx = ahead ? c.IFX[fb] : b.ifrcx, *ify = ahead ? c.IFY[fb] : b.ifrcy;
  bool force_side = false;  // this substage's force is running on the side stream (evF)
  if (ahead) {
    if (c.geo_ahead) {
      // geometry and force came ahead on the side stream; the bulk fluxes
      // follow them there, beside the listed faces
      cudaStreamWaitEvent(c.s, c.evp, 0);
      c.geo_ahead = false;
      cudaEventRecord(c.evf, c.s);
      cudaStreamWaitEvent(c.s2, c.evf, 0);
      launch_bulk_flux(c.s2, c.g, c.m, c.ph, b, ux, uy);
      cudaEventRecord(c.evx, c.s2);
    } else if (pre) {
      // the last step formed this substage's geometry and force: the bulk
      // fluxes here, beside decide_dt on the side stream
      launch_bulk_flux(c.s, c.g, c.m, c.ph, b, ux, uy);
    } else {
      // substage 0 (or a profiled step): the bulk fluxes first on the side
      // stream (after decide_dt, which waited for the state), the geometry
      // here, then the force on the side stream beside the listed faces and
      // the VOF update (which leaves vof^k in place).  A host-linked step
      // has its velocity last: the bulk fluxes then follow the listed faces
      // here, beside decide_dt, which waits for the same velocity
      if (par && !c.link) {
        cudaEventRecord(c.evf, c.s);
        cudaStreamWaitEvent(c.s2, c.evf, 0);
        launch_bulk_flux(c.s2, c.g, c.m, c.ph, b, ux, uy);
        cudaEventRecord(c.evx, c.s2);
      }
      timed(c, KC_PROPS, [&] { launch_props(c.s, c.g, c.m, c.ph, b, false, true, true, nullptr, scaled_vis()); });
      timed(c, KC_CURV_LIST, [&] { launch_geometry(c.s, c.g, c.m, b); });
      if (learned) timed(c, KC_MLP_CURV, [&] { launch_mlp_curv(c.s, c.g, b); });
      if (par) {
        cudaEventRecord(c.evf, c.s);
        cudaStreamWaitEvent(c.s2, c.evf, 0);
        launch_csf_force(c.s2, c.g, c.m, c.ph, b, den0, ifx, ify, learned);
        cudaEventRecord(c.evF, c.s2);
        force_side = true;
      } else {
        timed(c, KC_CSF_FORCE, [&] { launch_csf_force(c.s, c.g, c.m, c.ph, b, den0, ifx, ify, learned); });
      }
    }
    if (c.link && k == 0) cudaStreamWaitEvent(c.s, c.evh[1], 0);  // the velocity is in
    timed(c, KC_FACE_FLUX, [&] { launch_face_flux(c.s, c.g, b, ux, uy); });
    const bool bulk_here = !par || (k == 0 && c.link);
    if (par && !pre && !bulk_here) cudaStreamWaitEvent(c.s, c.evx, 0);
    if (bulk_here) timed(c, KC_BULK_FLUX, [&] { launch_bulk_flux(c.s, c.g, c.m, c.ph, b, ux, uy); });
    if (wait_dt) cudaStreamWaitEvent(c.s, c.evd, 0);
    timed(c, KC_VOF_ADVANCE,
          [&] { launch_vof_advance(c.s, c.g, c.m, c.ph, b, sc, k, sva, svb, true, ux, uy, den1, b.vof_alt); });
    std::swap(b.vof, b.vof_alt);  // vof^{k+1} is the current vof
  } else {
    if (c.props_ahead) {
      cudaStreamWaitEvent(c.s, c.evp, 0);
      c.props_ahead = false;
    } else {
      timed(c, KC_PROPS, [&] { launch_props(c.s, c.g, c.m, c.ph, b, false, true, true, nullptr, scaled_vis()); });
    }
    if (c.link && k == 0) cudaStreamWaitEvent(c.s, c.evh[1], 0);  // the velocity is in
    timed(c, KC_CURV_LIST, [&] { launch_interface_stage(c.s, c.g, c.m, c.ph, b, ux, uy, den0, 0); });
    if (learned) timed(c, KC_MLP_CURV, [&] { launch_mlp_curv(c.s, c.g, b); });
    if (par) {
      // the faces of single-phase upwind cells and the CSF force need only the
      // curvature: they run on the side stream beside the listed interface
      // faces (a few percent of the faces, a kernel that fills the GPU only
      // partly); the two write disjoint faces, and k_vof_advance waits for both
      cudaEventRecord(c.evf, c.s);
      cudaStreamWaitEvent(c.s2, c.evf, 0);
      launch_interface_stage(c.s2, c.g, c.m, c.ph, b, ux, uy, den0, learned ? 3 : 2);
      cudaEventRecord(c.evx, c.s2);
      launch_interface_stage(c.s, c.g, c.m, c.ph, b, ux, uy, den0, 1);
      cudaStreamWaitEvent(c.s, c.evx, 0);
    } else {
      timed(c, KC_INTERFACE, [&] { launch_interface_stage(c.s, c.g, c.m, c.ph, b, ux, uy, den0, 1); });
      timed(c, KC_FLUX_FORCE,
            [&] { launch_interface_stage(c.s, c.g, c.m, c.ph, b, ux, uy, den0, learned ? 3 : 2); });
    }
    if (wait_dt) cudaStreamWaitEvent(c.s, c.evd, 0);
    timed(c, KC_VOF_ADVANCE, [&] { launch_vof_advance(c.s, c.g, c.m, c.ph, b, sc, k, sva, svb, true, ux, uy, den1); });
  }
  if (c.link && k == 2) link_out(c, HL_VOF_OUT, L_VOF, b.vof);  // vof is final
  // the last substage leaves txy at the walls for the wall-stress log (all of
  // txx, txy, tyy when every array is synchronised), as the reference's
  // fluid_t holds the stress of its last predictor
  const int stress = k < 2 ? 0 : (g_sync_mode == SBFS_SYNC_ALL ? 2 : 1);
  timed(c, KC_MOMFLUX, [&] { launch_momflux(c.s, c.g, c.m, c.ph, b, ux, uy, stress, scaled_vis()); });
  if (par && (k < 2 || (ahead && c.make_next))) {
    // the next substage's viscosities and corner normals (and, ahead, its
    // geometry and force from the new vof and density) need only the new
    // vof: they run beside this substage's predictor, Poisson solve and
    // correction, none of which reads what they write.  After the last
    // substage of a device-resident step they are the next step's first
    // substage's (force into IFX[2]; the step joins them at its end)
    cudaEventRecord(c.evf, c.s);
    cudaStreamWaitEvent(c.s2, c.evf, 0);
    launch_props(c.s2, c.g, c.m, c.ph, b, false, true, true, nullptr, scaled_vis());
    if (ahead) {
      const int nb = k < 2 ? (k + 1) & 1 : 2;
      launch_geometry(c.s2, c.g, c.m, b);
      if (learned) launch_mlp_curv(c.s2, c.g, b);
      launch_csf_force(c.s2, c.g, c.m, c.ph, b, den1, c.IFX[nb], c.IFY[nb], learned);
      c.geo_ahead = k < 2;
    } else {
      c.props_ahead = true;
    }
    cudaEventRecord(c.evp, c.s2);
  }
  if (force_side) cudaStreamWaitEvent(c.s, c.evF, 0);
  if (c.link && k == 0) cudaStreamWaitEvent(c.s, c.evh[2], 0);  // p is in
  if (c.link && k == 0) cudaStreamWaitEvent(c.s, c.evh[3], 0);  // psi is in
  // the face sums of rho and the differences of psi_old come from the last
  // substage's predictor and correction: this step's, or for the first
  // substage the last device-resident step's (the same condition as its
  // geometry, pre_first)
  const bool cached = k > 0 || c.pre_first;
  timed(c, KC_PREDICT, [&] {
    launch_predict_mf(c.s, c.g, c.m, c.ph, b, sc, k, ux, uy, uxs, uys, den0, den1, psio, sxa, sxb, sya, syb, ifx,
                      ify, cached);
  });
  timed(c, KC_POISSON_FWD, [&] { launch_poisson_fwd_q(c.s, c.g, b, sc, k); });
  timed(c, KC_POISSON_TDM, [&] { launch_poisson_tdm(c.s, c.g, b); });
  timed(c, KC_POISSON_INV, [&] { launch_poisson_inv(c.s, c.g, b, psin); });
  // psi of substages 2 and 3 are final: the caller's psi[1] and psi[0] after the step
  if (c.link && k >= 1) link_out(c, k == 1 ? HL_PSI1_OUT : HL_PSI0_OUT, L_P, psin);
  timed(c, KC_CORRECT, [&] { launch_correct(c.s, c.g, c.m, b, sc, k, uxs, uys, psin, true, k < 2 || c.make_next); });
  c.iu ^= 1;
  c.ipsi ^= 1;
  c.iden ^= 1;
}

constexpr int kKernelsPerStep = 3 + 3 * 11;

void enqueue_step(Ctx &c) {
  // profiled steps keep every launch on the main stream (events per launch)
  const bool par = !g_prof.on;
  c.props_ahead = false;
  c.geo_ahead = false;
  if (c.link) link_in(c);
  if (par) {
    cudaEventRecord(c.evf, c.s);
    cudaStreamWaitEvent(c.s2, c.evf, 0);
    if (c.link) cudaStreamWaitEvent(c.s2, c.evh[1], 0);
    launch_decide_dt(c.s2, c.g, c.m, c.ph, c.b, c.U[c.iu], c.V[c.iu], c.dt_fixed, g_coef[0]);
    cudaEventRecord(c.evd, c.s2);
  } else {
    if (c.link) cudaStreamWaitEvent(c.s, c.evh[1], 0);
    timed(c, KC_DECIDE_DT,
          [&] { launch_decide_dt(c.s, c.g, c.m, c.ph, c.b, c.U[c.iu], c.V[c.iu], c.dt_fixed, g_coef[0]); });
  }
  for (int k = 0; k < 3; ++k) enqueue_substage(c, k, par, par && k == 0);
  // the next step's first-substage geometry (device-resident steps) joins here
  if (par && g_geo_ahead && c.make_next) cudaStreamWaitEvent(c.s, c.evp, 0);
  if (c.link) {
    // the velocity and p of the last correction, then the copy stream joins
    launch_host_rows(c.s, c.g, c.link_tab_dev, false, host_rows(c, HL_UX_OUT, L_UX, c.U[c.iu]),
                     host_rows(c, HL_UY_OUT, L_UY, c.V[c.iu]), 2, kLinkWide);
    launch_host_rows(c.s, c.g, c.link_tab_dev, false, host_rows(c, HL_P_OUT, L_P, c.b.p), HostRows{}, 1,
                     kLinkWide);
    cudaEventRecord(c.evh[4], c.s3);
    cudaStreamWaitEvent(c.s, c.evh[4], 0);
  }
}

// ---- autotuner of the launch shapes (block shape of each stencil kernel,
// columns per block of the Poisson transforms, wavenumbers per block of the
// tridiagonal solves).  On the first step of a context it times each
// candidate on the context's own state (saved before and put back after
// every trial): the block shapes by two eager steps per candidate (up to
// eight on small grids) with CUDA events around every launch, keeping the
// fastest per kernel class; then the
// two Poisson choices by the time of whole steps.  Results do not depend on
// the shapes.
int g_autotune = 0;

int autotune(Ctx &c) {
  c.pre_first = c.make_next = false;  // the trials form every substage's geometry themselves
  const size_t n = c.g.cs1 * c.nc;
  double *live[6] = {c.U[c.iu], c.V[c.iu], c.b.p, c.PSI[c.ipsi], c.b.vof, c.DEN[c.iden]};
  double *save[6] = {nullptr};
  for (int q = 0; q < 6; ++q) {
    CK(cudaMalloc(&save[q], n * sizeof(double)));
    CK(cudaMemcpyAsync(save[q], live[q], n * sizeof(double), cudaMemcpyDeviceToDevice, c.s));
  }
  const int iu = c.iu, ipsi = c.ipsi, iden = c.iden, isrc = c.isrc;
  double *const vof_cur = c.b.vof, *const vof_oth = c.b.vof_alt;
  auto restore = [&]() -> int {
    c.b.vof = vof_cur;
    c.b.vof_alt = vof_oth;
    c.iu = iu;
    c.ipsi = ipsi;
    c.iden = iden;
    c.isrc = isrc;
    for (int q = 0; q < 6; ++q)
      CK(cudaMemcpyAsync(live[q], save[q], n * sizeof(double), cudaMemcpyDeviceToDevice, c.s));
    return 0;
  };
  // 256-thread blocks (whose warps are 32 x 1 cells, 16 x 2, 8 x 4 or 4 x 8)
  // and smaller ones; an FP64 instruction costs a warp its issue slot however
  // few lanes take it, so where a branch follows the interface, warps of
  // compact patches are more often all in or all out of it
  const unsigned short shapes[][2] = {{32, 8}, {32, 4}, {64, 4}, {128, 2}, {32, 2}, {64, 2},
                                      {16, 16}, {256, 1}, {8, 32}, {4, 64}};
  const int nshape = sizeof(shapes) / sizeof(shapes[0]);
  std::vector<int> fws;
  std::vector<std::pair<int, int>> tdms;  // (wavenumbers per block, warps per system)
  for (int w : {2, 4, 8})
    if (fft_w_fits(c.ny, w)) fws.push_back(w);
  if (fws.empty()) fws.push_back(poisson_fft_cols(c.ny));
  const int G = c.b.tiles.tdm_g;  // fixed by the grid
  {
    Tiles cl = c.b.tiles;
    cl.tdm_cl = 1;
    if (tdm_uses_cluster(cl, c.nx)) tdms.push_back({0, G});  // 0: a cluster of four CTAs per pair
  }
  for (int mb : {1, 2, 4})
    if (G * mb <= 4 && poisson_tdm_smem(c.nx, mb, G) <= 200 * 1024) tdms.push_back({mb, G});
  if (tdms.empty()) tdms.push_back({1, G});  // one pair per block (staged in global memory above ~6900 rows)
  const int tk_of[KC_COUNT] = {TK_PROPS, TK_CURV_LIST, -1, TK_FLUX_FORCE, TK_VOF_ADVANCE, TK_MOMFLUX, TK_PREDICT,
                               -1, -1, -1, TK_CORRECT, -1, -1, TK_FORCE, -1, TK_FLUX_FORCE};
  Tiles best = c.b.tiles;
  float best_ms[TK_COUNT];
  for (int k = 0; k < TK_COUNT; ++k) best_ms[k] = 1e30f;
  const Tiles keep = c.b.tiles;
  // profiled steps per shape: 2, or up to 8 on grids below a million cells,
  // whose kernels last a few microseconds each
  const int nprof = (int)std::min(8., std::max(2., std::ceil(1e6 / ((double)c.nx * c.ny * c.nc))));
  int rc = 0;
  for (int t = 0; t < nshape && !rc; ++t) {
    Tiles cand = keep;
    for (int k = 0; k < TK_COUNT; ++k) {
      cand.bx[k] = shapes[t][0];
      cand.by[k] = shapes[t][1];
    }
    c.b.tiles = cand;
    if (restore()) {
      rc = 1;
      break;
    }
    enqueue_step(c);  // warm-up of this shape
    g_prof.on = true;
    g_prof.used = 0;
    g_prof.marks.clear();
    for (int r = 0; r < nprof; ++r) enqueue_step(c);
    g_prof.on = false;
    if (sync(c)) {
      rc = 1;
      break;
    }
    float ms[KC_COUNT] = {0.f};
    for (auto &mk : g_prof.marks) {
      float x = 0.f;
      cudaEventElapsedTime(&x, mk.second.first, mk.second.second);
      ms[mk.first] += x;
    }
    for (int kc = 0; kc < KC_COUNT; ++kc) {
      const int tk = tk_of[kc];
      if (tk >= 0 && ms[kc] < best_ms[tk]) {
        best_ms[tk] = ms[kc];
        best.bx[tk] = cand.bx[tk];
        best.by[tk] = cand.by[tk];
      }
    }
  }
  // second pass, on the chosen block shapes: the transform columns per block
  // and the wavenumber pairs per tridiagonal block set how many blocks a
  // Poisson launch has and so how its last wave fills the SMs, which events
  // around every launch misjudge (they also stop the launches overlapping);
  // the interface-branch compaction saves FP64 issue slots on large grids
  // but lengthens the kernels' critical path, which small grids feel.  Each
  // candidate is timed as whole steps launched as a step runs: three, or as
  // many as take about 8 M cell-steps on small grids (up to 40)
  if (!rc) {
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess) rc = 1;
    const double cells = (double)c.nx * c.ny * c.nc;
    const int nsteps = (int)std::min(40., std::max(3., std::ceil(8e6 / cells)));
    auto step_ms = [&](const Tiles &cand, float *out) -> int {
      c.b.tiles = cand;
      if (restore()) return 1;
      enqueue_step(c);  // warm-up
      cudaEventRecord(t0, c.s);
      for (int r = 0; r < nsteps; ++r) enqueue_step(c);
      cudaEventRecord(t1, c.s);
      if (sync(c)) return 1;
      return cudaEventElapsedTime(out, t0, t1) == cudaSuccess ? 0 : 1;
    };
    float bms = 1e30f;
    Tiles pick = best;
    for (size_t i = 0; i < fws.size() && !rc; ++i) {
      Tiles cand = best;
      cand.fft_w = fws[i];
      float ms = 0.f;
      if (step_ms(cand, &ms)) rc = 1;
      else if (ms < bms) {
        bms = ms;
        pick = cand;
      }
    }
    best = pick;
    bms = 1e30f;
    for (size_t i = 0; i < tdms.size() && !rc && tdms.size() > 1; ++i) {
      Tiles cand = best;
      cand.tdm_cl = tdms[i].first == 0 ? 1 : 0;
      cand.tdm_mb = tdms[i].first == 0 ? 1 : tdms[i].first;
      cand.tdm_g = tdms[i].second;
      float ms = 0.f;
      if (step_ms(cand, &ms)) rc = 1;
      else if (ms < bms) {
        bms = ms;
        pick = cand;
      }
    }
    best = pick;
    bms = 1e30f;
    for (int cm = 1; cm >= 0 && !rc; --cm) {
      Tiles cand = best;
      cand.compact = cm;
      float ms = 0.f;
      if (step_ms(cand, &ms)) rc = 1;
      else if (ms < bms) {
        bms = ms;
        pick = cand;
      }
    }
    best = pick;
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
  }
  c.b.tiles = rc ? keep : best;
  const int rr = restore();
  const cudaError_t e = cudaStreamSynchronize(c.s);
  for (int q = 0; q < 6; ++q) cudaFree(save[q]);
  for (auto &kv : c.graphs) cudaGraphExecDestroy(kv.second);
  c.graphs.clear();
  c.tuned = true;
  state_touched(c);
  if (rc || rr) return 1;
  if (e != cudaSuccess) return fail("autotune: %s", cudaGetErrorString(e));
  return 0;
}

int role_key(const Ctx &c) {
  return c.iu | (c.ipsi << 1) | (c.iden << 2) | (c.isrc << 3) | (g_curv_model << 4) | ((int)c.link << 5) |
         (g_pdl << 6) | ((g_compact + 1) << 7) | ((g_sync_mode == SBFS_SYNC_ALL) << 9) | (g_geo_ahead << 10) |
         ((c.b.vof != c.VOF0) << 11) | (g_stream_prio << 12) | ((int)c.pre_first << 13) | ((int)c.make_next << 14) | (g_tdm_cluster << 15);
}

int launch_step(Ctx &c) {
  if (g_autotune && !c.tuned && c.resident && !g_prof.on) {
    const bool link = c.link;  // the trials step the device state only
    c.link = false;
    const int rc = autotune(c);
    c.link = link;
    if (rc) return 1;
  }
  // the first substage's geometry from the last step (device-resident
  // steps in the same configuration), and this step's for the next one
  auto plan = [&c]() {
    const bool par = !g_prof.on;
    c.pre_first = par && g_geo_ahead && c.geo_next && !c.link && c.geo_next_cfg == geo_cfg();
    c.make_next = par && g_geo_ahead && g_sync_mode == SBFS_SYNC_NONE && !c.link;
  };
  auto planned = [&c]() {
    c.geo_next = c.make_next;
    if (c.make_next) c.geo_next_cfg = geo_cfg();
  };
  if (!g_use_graphs || g_prof.on) {
    plan();
    enqueue_step(c);
    planned();
    CK(cudaGetLastError());
    return 0;
  }
  {
    const Phys &p = c.ph;
    float klo, khi;  // the learned closure's range (a kernel argument when it runs)
    mlp_range(&klo, &khi);
    const std::vector<double> sig = {p.denr, p.visr,   p.refden,   p.den_lo,   p.den_hi,   p.vis_lo,
                                     p.vis_hi, p.grav, p.force_coef, p.irefden, p.nu,      c.dt_fixed,
                                     g_coef[0], g_coef[1], g_coef[2], klo, khi};
    std::vector<double> all(sig);
    for (const Phys &q : c.phys_host) {
      const double *w = reinterpret_cast<const double *>(&q);
      all.insert(all.end(), w, w + sizeof(Phys) / sizeof(double));
    }
    if (all.size() != c.graph_sig.size() ||
        memcmp(all.data(), c.graph_sig.data(), sizeof(double) * all.size()) != 0) {
      for (auto &kv : c.graphs) cudaGraphExecDestroy(kv.second);
      c.graphs.clear();
      c.graph_sig = all;
      state_touched(c);
    }
  }
  plan();
  const int key = role_key(c);
  auto it = c.graphs.find(key);
  // a host-linked graph holds copy-engine copies of the caller's arrays: it
  // is captured again when the arrays are others
  std::vector<const void *> hosts = c.link && c.nc == 1 ? c.link_host : std::vector<const void *>();
  if (!hosts.empty()) hosts.push_back(reinterpret_cast<const void *>(c.link_reg));
  if (it != c.graphs.end() && c.graph_hosts[key] != hosts) {
    cudaGraphExecDestroy(it->second);
    c.graphs.erase(it);
    it = c.graphs.end();
  }
  if (it == c.graphs.end()) {
    const int iu = c.iu, ipsi = c.ipsi, iden = c.iden, isrc = c.isrc;
    double *const vof = c.b.vof, *const vof_alt = c.b.vof_alt;
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(c.s, cudaStreamCaptureModeThreadLocal));
    enqueue_step(c);
    cudaError_t e = cudaStreamEndCapture(c.s, &graph);
    if (e != cudaSuccess) return fail("graph capture: %s", cudaGetErrorString(e));
    cudaGraphExec_t exec;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail("graph instantiate: %s", cudaGetErrorString(e));
    it = c.graphs.emplace(key, exec).first;
    c.graph_hosts[key] = hosts;
    // capturing advanced the roles; restore, the launch below advances them
    c.iu = iu;
    c.ipsi = ipsi;
    c.iden = iden;
    c.isrc = isrc;
    c.b.vof = vof;
    c.b.vof_alt = vof_alt;
  }
  CK(cudaGraphLaunch(it->second, c.s));
  // roles after one step (3 substages: velocity, potential and density flip
  // three times, the RK sources twice, the two vof buffers three times when
  // the geometry runs ahead)
  c.iu ^= 1;
  c.ipsi ^= 1;
  c.iden ^= 1;
  if (g_geo_ahead) std::swap(c.b.vof, c.b.vof_alt);
  planned();
  return 0;
}

int upload_fields(Ctx &c, const fluid_t *f, const interface_t *itf) {
  state_touched(c);
  return h2d(c, f->ux, L_UX, c.U[c.iu]) || h2d(c, f->uy, L_UY, c.V[c.iu]) || h2d(c, f->p, L_P, c.b.p) ||
         h2d(c, f->psi[0], L_P, c.PSI[c.ipsi]) || h2d(c, itf->vof, L_VOF, c.b.vof);
}

int upload_state(Ctx &c, const fluid_t *f, const interface_t *itf) {
  if (upload_fields(c, f, itf)) return 1;
  // rho^k of the current vof (src/fluid/density.c)
  launch_props(c.s, c.g, c.m, c.ph, c.b, true, false, false, c.DEN[c.iden]);
  c.resident = true;
  return 0;
}

int download_state(Ctx &c, fluid_t *f, interface_t *itf, bool all) {
  // the reference's psi pointers end a step swapped (three swaps)
  if (d2h(c, f->ux, L_UX, c.U[c.iu]) || d2h(c, f->uy, L_UY, c.V[c.iu]) || d2h(c, f->p, L_P, c.b.p) ||
      d2h(c, f->psi[0], L_P, c.PSI[c.ipsi]) || d2h(c, f->psi[1], L_P, c.PSI[c.ipsi ^ 1]) ||
      d2h(c, itf->vof, L_VOF, c.b.vof))
    return 1;
  if (all) {
    Bufs &b = c.b;
    if (d2h(c, f->den[0], L_DEN, c.DEN[c.iden ^ 1]) || d2h(c, f->den[1], L_DEN, c.DEN[c.iden]) ||
        d2h(c, f->visux, L_VISUX, b.visux) || d2h(c, f->visuy, L_VISUY, b.visuy) ||
        d2h(c, f->txx, L_TXX, b.txx) || d2h(c, f->txy, L_TXY, b.txy) || d2h(c, f->tyy, L_TYY, b.tyy) ||
        d2h(c, f->srcux[0], L_SRCUX, c.SX[c.isrc]) || d2h(c, f->srcux[1], L_SRCUX, c.SX[c.isrc ^ 1]) ||
        d2h(c, f->srcuy[0], L_SRCUY, c.SY[c.isrc]) || d2h(c, f->srcuy[1], L_SRCUY, c.SY[c.isrc ^ 1]) ||
        d2h(c, itf->ifrcx, L_IFRCX, b.ifrcx) || d2h(c, itf->ifrcy, L_IFRCY, b.ifrcy) ||
        d2h(c, itf->dvof, L_DVOF, b.dvof) || d2h(c, itf->normal, L_NORMAL, b.normal) ||
        d2h(c, itf->curv, L_CURV, b.curv) || d2h(c, itf->fluxx, L_FLUXX, b.mfluxx) ||
        d2h(c, itf->fluxy, L_FLUXY, b.mfluxy) || d2h(c, itf->src[0], L_SRC, c.SV[c.isrc]) ||
        d2h(c, itf->src[1], L_SRC, c.SV[c.isrc ^ 1]))
      return 1;
  }
  return 0;
}

int read_dt_status(Ctx &c, double *dt, int *status) {
  CK(cudaMemcpyAsync(c.small_host, c.b.scalars, sizeof(double) * (kScalars + 1), cudaMemcpyDeviceToHost, c.s));
  if (sync(c)) return 1;
  if (dt) *dt = c.small_host[0];
  if (status) memcpy(status, c.small_host + kScalars, sizeof(int));
  return 0;
}

// ---- batches of independent cases (sbfs_integrate_batch)
// Cases are grouped by grid; each group is one context whose fields hold its
// cases as consecutive slabs, and every kernel of the step runs all cases of
// the group in one launch (the case is blockIdx.z).  Groups run on their own
// streams.
struct Batch {
  std::vector<std::unique_ptr<Ctx>> groups;
  std::vector<int> group_of, slot_of;
  std::vector<const void *> ident;  // fluid and interface pointers of the cases
  std::vector<double> res;          // Re per case, to notice a change
};
std::unique_ptr<Batch> g_batch;

bool same_domain_grid(const domain_t *a, const domain_t *d) {
  return a->mysizes[0] == d->mysizes[0] && a->mysizes[1] == d->mysizes[1] && a->lengths[0] == d->lengths[0] &&
         a->lengths[1] == d->lengths[1] && a->hy == d->hy &&
         memcmp(a->hxxf, d->hxxf, sizeof(double) * (a->mysizes[0] + 1)) == 0;
}

bool same_grid_as(const Ctx &c, const domain_t *d) {
  return c.nx == (int)d->mysizes[0] && c.ny == (int)d->mysizes[1] && c.lx == d->lengths[0] &&
         c.ly == d->lengths[1] && c.g.hy == d->hy &&
         memcmp(c.hxxf.data(), d->hxxf, sizeof(double) * (c.nx + 1)) == 0;
}

Batch *prepare_batch(int n, const domain_t *const *d, fluid_t *const *f, interface_t *const *itf) {
  if (n <= 0 || !d || !f || !itf) {
    fail("empty batch");
    return nullptr;
  }
  if (load_coefs()) return nullptr;
  for (int i = 0; i < n; ++i) {
    if (!f[i] || !itf[i]) {
      fail("case %d: null fluid or interface", i);
      return nullptr;
    }
    if (check_domain(d[i])) return nullptr;
  }
  Batch *b = g_batch.get();
  bool same = b && (int)b->group_of.size() == n;
  for (int i = 0; same && i < n; ++i)
    same = b->ident[2 * i] == f[i] && b->ident[2 * i + 1] == itf[i] &&
           same_grid_as(*b->groups[b->group_of[i]], d[i]);
  if (!same) {
    g_batch.reset();
    auto nb = std::make_unique<Batch>();
    std::vector<int> first, count;  // first case and size of each group
    nb->group_of.resize(n);
    nb->slot_of.resize(n);
    for (int i = 0; i < n; ++i) {
      // cases per group: the face list holds 4 * cell + face of every case as
      // an int, and the case is blockIdx.z; a full group starts another one
      const long cells = (long)d[i]->mysizes[0] * (long)d[i]->mysizes[1];
      const int cap = (int)std::min(65535L, (1L << 29) / cells);
      int gi = -1;
      for (size_t q = 0; q < first.size() && gi < 0; ++q)
        if (count[q] < cap && same_domain_grid(d[first[q]], d[i])) gi = (int)q;
      if (gi < 0) {
        gi = (int)first.size();
        first.push_back(i);
        count.push_back(0);
      }
      nb->group_of[i] = gi;
      nb->slot_of[i] = count[gi]++;
      nb->ident.push_back(f[i]);
      nb->ident.push_back(itf[i]);
    }
    for (size_t q = 0; q < first.size(); ++q) {
      auto c = std::make_unique<Ctx>();
      if (build_ctx(c.get(), d[first[q]], count[q])) return nullptr;
      c->phys_host.resize(count[q]);
      nb->groups.push_back(std::move(c));
    }
    nb->res.assign(n, NAN);
    g_batch = std::move(nb);
    b = g_batch.get();
  }
  // physics and metrics per case (re-uploaded when they change)
  for (size_t q = 0; q < b->groups.size(); ++q) {
    Ctx &c = *b->groups[q];
    std::vector<Phys> ph(c.nc);
    std::vector<double> re(c.nc);
    const domain_t *dq = nullptr;
    bool re_changed = !c.met;
    for (int i = 0; i < n; ++i) {
      if (b->group_of[i] != (int)q) continue;
      const int k = b->slot_of[i];
      ph[k] = phys_of(f[i], itf[i]);
      finish_phys(ph[k], c.g);
      ph[k].dtfix = fixed_dt(c, d[i], f[i], itf[i]);
      re[k] = f[i]->Re;
      re_changed = re_changed || !(b->res[i] == f[i]->Re);
      b->res[i] = f[i]->Re;
      dq = d[i];
    }
    if (re_changed && upload_metrics(c, dq, re.data())) return nullptr;
    if (re_changed || memcmp(ph.data(), c.phys_host.data(), sizeof(Phys) * c.nc) != 0) {
      c.phys_host = ph;
      c.geo_next = false;  // other physics: a geometry formed ahead is stale
      // a group of one case has no table: its kernels take c.ph
      if (c.phys_dev && (cudaMemcpyAsync(c.phys_dev, c.phys_host.data(), sizeof(Phys) * c.nc,
                                         cudaMemcpyHostToDevice, c.s) != cudaSuccess ||
                         sync(c))) {
        fail("uploading the per-case physics");
        return nullptr;
      }
    }
    c.ph = ph[0];  // the kernels read the table; this is only their argument
    c.dt_fixed = ph[0].dtfix;
  }
  return b;
}

int batch_upload(Batch &b, int n, fluid_t *const *f, interface_t *const *itf) {
  for (int i = 0; i < n; ++i) {
    Ctx &c = *b.groups[b.group_of[i]];
    c.kcase = b.slot_of[i];
    const int rc = upload_fields(c, f[i], itf[i]);
    c.kcase = 0;
    if (rc) return 1;
  }
  for (auto &c : b.groups) {
    // rho^k of the current vof, every case of the group in one launch
    launch_props(c->s, c->g, c->m, c->ph, c->b, true, false, false, c->DEN[c->iden]);
    c->resident = true;
  }
  return 0;
}

int batch_download(Batch &b, int n, fluid_t *const *f, interface_t *const *itf, bool all) {
  for (int i = 0; i < n; ++i) {
    Ctx &c = *b.groups[b.group_of[i]];
    c.kcase = b.slot_of[i];
    const int rc = download_state(c, f[i], itf[i], all);
    c.kcase = 0;
    if (rc) return 1;
  }
  return 0;
}

// dt of every case after the last step; fails on a non-finite velocity
int batch_read_dt(Batch &b, int n, double *dts) {
  for (auto &c : b.groups) {
    const size_t bytes = sizeof(double) * (size_t)kScalars * c->nc + sizeof(int) * c->nc;
    CK(cudaMemcpyAsync(c->small_host, c->b.scalars, bytes, cudaMemcpyDeviceToHost, c->s));
  }
  for (auto &c : b.groups)
    if (sync(*c)) return 1;
  for (int i = 0; i < n; ++i) {
    const Ctx &c = *b.groups[b.group_of[i]];
    const int k = b.slot_of[i];
    int status = 0;
    memcpy(&status, reinterpret_cast<const char *>(c.small_host + (size_t)kScalars * c.nc) + sizeof(int) * k,
           sizeof(int));
    if (status & 1) return fail("case %d: non-finite velocity detected by decide_dt", i);
    if (dts) dts[i] = c.small_host[(size_t)k * kScalars];
  }
  return 0;
}

Ctx *prepare_step(const domain_t *d, fluid_t *f, interface_t *itf) {
  if (!f || !itf) {
    fail("null fluid or interface");
    return nullptr;
  }
  if (load_coefs()) return nullptr;
  Ctx *c = get_ctx(d, f, itf);
  if (!c) return nullptr;
  c->dt_fixed = fixed_dt(*c, d, f, itf);
  return c;
}

}  // namespace

// ===========================================================================
// exported entry points
// ===========================================================================
extern "C" {

const char *sbfs_last_error(void) { return g_err.c_str(); }

int sbfs_set_pdl(int on) {
  g_pdl = on ? 1 : 0;
  return 0;
}

int sbfs_set_compaction(int mode) {
  if (mode < -1 || mode > 1) return fail("bad compaction mode %d", mode);
  g_compact = mode;
  return 0;
}

int sbfs_set_tdm_cluster(int on) {
  g_tdm_cluster = on ? 1 : 0;
  return 0;
}

int sbfs_set_stream_priorities(int on) {
  g_stream_prio = on ? 1 : 0;
  return 0;
}

int sbfs_set_geometry_ahead(int on) {
  g_geo_ahead = on ? 1 : 0;
  return 0;
}

int sbfs_set_host_link(int on) {
  if (on < 0 || on > 2) return fail("bad host-link mode %d", on);
  g_host_link = on;
  return 0;
}

int sbfs_host_link_used(void) { return g_link_used ? 1 : 0; }

int sbfs_set_sync_mode(int mode) {
  if (mode < SBFS_SYNC_STATE || mode > SBFS_SYNC_NONE) return fail("bad sync mode %d", mode);
  g_sync_mode = mode;
  return 0;
}

int sbfs_set_use_graphs(int on) {
  g_use_graphs = on ? 1 : 0;
  return 0;
}

int sbfs_set_dt_coefs(double adv, double dif, double itf) {
  if (!(adv >= 0.) || !(dif >= 0.) || !(itf >= 0.)) return fail("dt safety factors must be non-negative");
  g_coef[0] = adv;
  g_coef[1] = dif;
  g_coef[2] = itf;
  return 0;
}

int sbfs_invalidate_device(void) {
  if (g_ctx) g_ctx->resident = false;
  if (g_ctx) state_touched(*g_ctx);
  ++g_reg_epoch;  // and look at the host arrays' registration again
  return 0;
}

int sbfs_kernels_per_step(void) { return kKernelsPerStep + (g_geo_ahead ? 3 : 0) + (g_curv_model ? 3 : 0); }

int sbfs_set_curvature_model(int model) {
  if (model != 0 && model != 1) return fail("bad curvature model %d", model);
  if (model == 1 && !mlp_ready()) return fail("learned curvature selected before its parameters were set");
  g_curv_model = model;
  return 0;
}

// the state the device holds, uploaded first when the host is the truth
static Ctx *diag_ctx(const domain_t *d, fluid_t *f, interface_t *itf) {
  Ctx *c = prepare_step(d, f, itf);
  if (!c) return nullptr;
  // the host is the truth unless the caller keeps the state on the device
  if (g_sync_mode != SBFS_SYNC_NONE || !c->resident) {
    if (upload_state(*c, f, itf)) return nullptr;
    // the wall-stress log reads the caller's txy, as the reference's does
    if (h2d(*c, f->txy, L_TXY, c->b.txy)) return nullptr;
  }
  return c;
}

// logging quantities of the reference (src/logging/), reduced on the GPU
int sbfs_diagnostics(const domain_t *d, fluid_t *f, interface_t *itf, sbfs_diagnostics_t *out) {
  Ctx *c = diag_ctx(d, f, itf);
  if (!c) return 1;
  if (!c->diag_part) {
    if (dalloc(*c, &c->diag_part, (size_t)diag_partial_blocks(c->g) * 16) || dalloc(*c, &c->diag_out, 16)) return 1;
  }
  launch_diagnostics(c->s, c->g, c->m, c->U[c->iu], c->V[c->iu], c->b.vof, c->DEN[c->iden], c->b.txy, c->ph.nu,
                     c->diag_part, c->diag_out);
  double h[16];
  CK(cudaMemcpyAsync(h, c->diag_out, sizeof(h), cudaMemcpyDeviceToHost, c->s));
  if (sync(*c)) return 1;
  out->divmax = h[0];
  out->vof_min = h[1];
  out->vof_max = h[2];
  out->vof_integral = h[3];
  out->volume = h[4];
  out->interface_area = h[5];
  out->momentum[0] = h[6];
  out->momentum[1] = h[7];
  out->energy[0] = h[8];
  out->energy[1] = h[9];
  out->umax[0] = h[10];
  out->umax[1] = h[11];
  out->wall_stress[0] = h[12];
  out->wall_stress[1] = h[13];
  return 0;
}

// the reference's monitor files (src/logging/main.c:90-108), appended to in
// dirname with the reference's line formats; the quantities come from the
// device reductions of sbfs_diagnostics
int sbfs_logging_output(const char dirname[], const domain_t *d, fluid_t *f, interface_t *itf, size_t step,
                        double time, double dt, double wtime) {
  sbfs_diagnostics_t q;
  if (sbfs_diagnostics(d, f, itf, &q)) return 1;
  const std::string dir = dirname ? std::string(dirname) : std::string(".");
  auto open = [&](const char *name) -> FILE * {
    const std::string path = dir + "/" + name;
    FILE *fp = fopen(path.c_str(), "a");
    if (!fp) fail("%s: cannot open for appending", path.c_str());
    return fp;
  };
  FILE *fp;
  if (!(fp = open("progress.dat"))) return 1;
  fprintf(fp, "step %10zu, time %.3f, dt %.3e, elapsed %.1f [sec]\n", step, time, dt, wtime);
  fprintf(stdout, "step %10zu, time %.3f, dt %.3e, elapsed %.1f [sec]\n", step, time, dt, wtime);
  fclose(fp);
  if (!(fp = open("divergence.dat"))) return 1;
  fprintf(fp, "%8.2f % .1e\n", time, q.divmax);
  fclose(fp);
  if (!(fp = open("momentum.dat"))) return 1;
  fprintf(fp, "%8.2f % 18.15e % 18.15e\n", time, q.momentum[0], q.momentum[1]);
  fclose(fp);
  if (!(fp = open("extrema.dat"))) return 1;
  fprintf(fp, "%8.2f % 18.15e % 18.15e\n", time, q.umax[0], q.umax[1]);
  fclose(fp);
  if (!(fp = open("energy.dat"))) return 1;
  fprintf(fp, "%8.2f % 18.15e % 18.15e\n", time, q.energy[0], q.energy[1]);
  fclose(fp);
  if (!(fp = open("stress.dat"))) return 1;
  fprintf(fp, "%8.2f % 18.15e % 18.15e\n", time, q.wall_stress[0], q.wall_stress[1]);
  fclose(fp);
  if (!(fp = open("vof.dat"))) return 1;
  fprintf(fp, "%8.2f % 18.15e % 18.15e % 18.15e % 18.15e\n", time, q.vof_min, q.vof_max,
          q.vof_integral / q.volume, q.interface_area);
  fclose(fp);
  fflush(stdout);
  return 0;
}

// running sums of src/statistics.c:99-166 kept on the GPU
int sbfs_statistics_collect(const domain_t *d, fluid_t *f, interface_t *itf) {
  Ctx *c = diag_ctx(d, f, itf);
  if (!c) return 1;
  if (!c->st_ux1) {
    const size_t n1 = (size_t)c->g.p1 * c->g.ny;
    if (dalloc(*c, &c->st_ux1, n1) || dalloc(*c, &c->st_uy1, n1) || dalloc(*c, &c->st_vof1, n1)) return 1;
    c->st_num = 0;
  }
  launch_stats_collect(c->s, c->g, c->U[c->iu], c->V[c->iu], c->b.vof, c->st_ux1, c->st_uy1, c->st_vof1);
  c->st_num += 1;
  return sync(*c);
}

int sbfs_statistics_reset(void) {
  Ctx *c = g_ctx.get();
  if (!c || !c->st_ux1) return 0;
  const size_t bytes = sizeof(double) * (size_t)c->g.p1 * c->g.ny;
  CK(cudaMemsetAsync(c->st_ux1, 0, bytes, c->s));
  CK(cudaMemsetAsync(c->st_uy1, 0, bytes, c->s));
  CK(cudaMemsetAsync(c->st_vof1, 0, bytes, c->s));
  c->st_num = 0;
  return sync(*c);
}

// sums in the reference's statistics layout: ux1 (ny, nx+1), uy1 and vof1 (ny, nx+2)
int sbfs_statistics_fetch(double *ux1, double *uy1, double *vof1, size_t *num) {
  Ctx *c = g_ctx.get();
  *num = (c && c->st_ux1) ? c->st_num : 0;
  if (!*num) return 0;
  const size_t p = sizeof(double) * c->g.p1;
  CK(cudaMemcpy2DAsync(ux1, sizeof(double) * (c->nx + 1), c->st_ux1, p, sizeof(double) * (c->nx + 1), c->ny,
                       cudaMemcpyDeviceToHost, c->s));
  CK(cudaMemcpy2DAsync(uy1, sizeof(double) * (c->nx + 2), c->st_uy1, p, sizeof(double) * (c->nx + 2), c->ny,
                       cudaMemcpyDeviceToHost, c->s));
  CK(cudaMemcpy2DAsync(vof1, sizeof(double) * (c->nx + 2), c->st_vof1, p, sizeof(double) * (c->nx + 2), c->ny,
                       cudaMemcpyDeviceToHost, c->s));
  return sync(*c);
}

int sbfs_measure_fp64_peak(double *gflops) {
  CK(measure_fp64_peak(gflops));
  return 0;
}

int sbfs_check_newton_raphson(const double *x, double *rcp, double *rsq, int n) {
  double *d = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * 3 * (size_t)n));
  cudaError_t e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = nr_check(d, d + n, d + 2 * (size_t)n, n);
  if (e == cudaSuccess) e = cudaMemcpy(rcp, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(rsq, d + 2 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail("newton-raphson check: %s", cudaGetErrorString(e));
  return 0;
}

int sbfs_set_device(int device) {
  g_ctx.reset();
  CK(cudaSetDevice(device));
  return 0;
}

int sbfs_pin_host_state(fluid_t *f, interface_t *itf) {
  void *ptrs[] = {f->ux.data, f->uy.data, f->p.data, f->psi[0].data, f->psi[1].data, itf->vof.data};
  size_t sizes[] = {f->ux.datasize, f->uy.datasize, f->p.datasize, f->psi[0].datasize, f->psi[1].datasize,
                    itf->vof.datasize};
  ++g_reg_epoch;
  for (int i = 0; i < 6; ++i) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, ptrs[i]) == cudaSuccess && at.type == cudaMemoryTypeHost) continue;
    cudaGetLastError();
    CK(cudaHostRegister(ptrs[i], sizes[i], cudaHostRegisterDefault));
  }
  return 0;
}

int sbfs_unpin_host_state(fluid_t *f, interface_t *itf) {
  void *ptrs[] = {f->ux.data, f->uy.data, f->p.data, f->psi[0].data, f->psi[1].data, itf->vof.data};
  ++g_reg_epoch;
  for (void *p : ptrs) {
    if (cudaHostUnregister(p) != cudaSuccess) cudaGetLastError();
  }
  return 0;
}

const char *sbfs_kernel_name(int cls) { return (cls >= 0 && cls < KC_COUNT) ? kKernelNames[cls] : ""; }
int sbfs_kernel_classes(void) { return KC_COUNT; }

int sbfs_profile_steps(const domain_t *d, fluid_t *f, interface_t *itf, int nsteps, float *ms_per_class,
                       int *launches_per_class) {
  Ctx *c = prepare_step(d, f, itf);
  if (!c) return 1;
  if (!c->resident) {
    if (upload_state(*c, f, itf)) return 1;
  }
  g_prof.on = true;
  g_prof.used = 0;
  g_prof.marks.clear();
  int rc = 0;
  for (int n = 0; n < nsteps && !rc; ++n) rc = launch_step(*c);
  g_prof.on = false;
  if (rc) return 1;
  if (sync(*c)) return 1;
  for (int k = 0; k < KC_COUNT; ++k) {
    ms_per_class[k] = 0.f;
    launches_per_class[k] = 0;
  }
  for (auto &mk : g_prof.marks) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, mk.second.first, mk.second.second));
    ms_per_class[mk.first] += ms;
    launches_per_class[mk.first] += 1;
  }
  int status = 0;
  if (read_dt_status(*c, nullptr, &status)) return 1;
  return (status & 1) ? fail("non-finite velocity detected by decide_dt") : 0;
}

int sbfs_release(void) {
  g_ctx.reset();
  return 0;
}

int sbfs_device_status(int *status) {
  if (!g_ctx) {
    *status = 0;
    return 0;
  }
  return read_dt_status(*g_ctx, nullptr, status);
}

int sbfs_sync_to_host(const domain_t *d, fluid_t *f, interface_t *itf) {
  Ctx *c = g_ctx.get();
  if (!c || !c->resident) return 0;
  (void)d;
  if (download_state(*c, f, itf, g_sync_mode == SBFS_SYNC_ALL)) return 1;
  return sync(*c);
}

// host memory the GPU can address: any on a system whose GPU reads pageable
// memory through the host page tables, else memory registered with CUDA
int g_pageable = -1, g_pageable_dev = -1;  // the attribute of device g_pageable_dev
bool host_addressable(void *p, double **dev) {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (d != g_pageable_dev) {
    int v = 0;
    g_pageable = cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, d) == cudaSuccess && v == 1;
    g_pageable_dev = d;
    cudaGetLastError();
  }
  if (g_pageable && g_host_link == 1) {
    *dev = static_cast<double *>(p);
    return true;
  }
  // registered (or cudaHostAlloc'd) memory and its device address
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return false;
  *dev = static_cast<double *>(at.devicePointer);
  return true;
}

// fills the link table of case k for a strict-mode step, or says the step
// cannot be host-linked (then the state goes through cudaMemcpy as before)
bool link_tab_fill(Ctx &c, int k, fluid_t *f, interface_t *itf) {
  if (!g_host_link || g_prof.on || g_sync_mode != SBFS_SYNC_STATE) return false;
  const array_t *arr[HL_COUNT] = {&f->ux, &f->uy, &f->p, &f->psi[0], &itf->vof, &f->ux, &f->uy, &f->p,
                                  &f->psi[1], &f->psi[0], &itf->vof};
  const Layout *lay[HL_COUNT] = {&L_UX, &L_UY, &L_P, &L_P, &L_VOF, &L_UX, &L_UY, &L_P, &L_P, &L_P, &L_VOF};
  if (c.nc == 1) c.link_host.assign(HL_COUNT, nullptr);
  for (int q = 0; q < HL_COUNT; ++q) {
    if (!layout_ok(*arr[q], *lay[q]) || !host_addressable(arr[q]->data, &c.link_tab[(size_t)k * kLinkSlots + q]))
      return false;
    if (c.nc == 1) c.link_host[q] = arr[q]->data;
  }
  if (c.nc == 1 && (c.link_host != c.link_prev || c.link_epoch != g_reg_epoch)) {
    // page-locked or pageable: the copy engines move them differently, and a
    // captured copy keeps the way it was captured with
    c.link_reg = 0;
    for (int q = 0; q < HL_COUNT; ++q) {
      cudaPointerAttributes at;
      if (cudaPointerGetAttributes(&at, c.link_host[q]) == cudaSuccess && at.type == cudaMemoryTypeHost)
        c.link_reg |= (uintptr_t)1 << q;
      cudaGetLastError();
    }
    c.link_prev = c.link_host;
    c.link_epoch = g_reg_epoch;
  }
  return true;
}

// reference src/integrate.c:11-70
int integrate(const domain_t *d, fluid_t *f, interface_t *itf, double *dt) {
  Ctx *c = prepare_step(d, f, itf);
  if (!c) return 1;
  g_link_used = link_tab_fill(*c, 0, f, itf);
  if (g_link_used) {
    // the step reads the caller's arrays and writes them back itself; the
    // reference's psi pointers end a step swapped (three swaps)
    c->link = true;
    const int rc = launch_step(*c);
    c->link = false;
    if (rc) return 1;
    c->resident = true;
    swap_data(f->psi[0], f->psi[1]);
    int status = 0;
    if (read_dt_status(*c, dt, &status)) return 1;
    if (status & 1) return fail("non-finite velocity detected by decide_dt");
    return 0;
  }
  if (g_sync_mode != SBFS_SYNC_NONE || !c->resident) {
    if (upload_state(*c, f, itf)) return 1;
  }
  if (launch_step(*c)) return 1;
  if (g_sync_mode != SBFS_SYNC_NONE) {
    swap_data(f->psi[0], f->psi[1]);
    if (download_state(*c, f, itf, g_sync_mode == SBFS_SYNC_ALL)) return 1;
  }
  int status = 0;
  if (read_dt_status(*c, dt, &status)) return 1;
  if (status & 1) return fail("non-finite velocity detected by decide_dt");
  return 0;
}

int sbfs_integrate_batch(int n, const domain_t *const *domains, fluid_t *const *fluids,
                         interface_t *const *interfaces, double *dts) {
  Batch *b = prepare_batch(n, domains, fluids, interfaces);
  if (!b) return 1;
  bool link = true;
  for (int i = 0; i < n && link; ++i)
    link = link_tab_fill(*b->groups[b->group_of[i]], b->slot_of[i], fluids[i], interfaces[i]);
  g_link_used = link;
  if (link) {
    // every group's step copies its cases in and out itself (see integrate)
    for (auto &c : b->groups) {
      c->link = true;
      const int rc = launch_step(*c);
      c->link = false;
      if (rc) return 1;
      c->resident = true;
    }
    for (int i = 0; i < n; ++i) swap_data(fluids[i]->psi[0], fluids[i]->psi[1]);
    return batch_read_dt(*b, n, dts);
  }
  bool upload = g_sync_mode != SBFS_SYNC_NONE;
  for (auto &c : b->groups) upload = upload || !c->resident;
  if (upload && batch_upload(*b, n, fluids, interfaces)) return 1;
  for (auto &c : b->groups)
    if (launch_step(*c)) return 1;
  if (g_sync_mode != SBFS_SYNC_NONE) {
    for (int i = 0; i < n; ++i) swap_data(fluids[i]->psi[0], fluids[i]->psi[1]);
    if (batch_download(*b, n, fluids, interfaces, g_sync_mode == SBFS_SYNC_ALL)) return 1;
  }
  return batch_read_dt(*b, n, dts);
}

int sbfs_run_batch_steps_timed(int nsteps, float *ms) {
  Batch *b = g_batch.get();
  if (!b) return fail("no batch on the device: call sbfs_integrate_batch first");
  for (auto &c : b->groups)
    if (!c->resident) return fail("the batch's state is not on the device");
  Ctx &c0 = *b->groups[0];
  CK(cudaEventRecord(c0.e0, c0.s));
  for (size_t q = 1; q < b->groups.size(); ++q) CK(cudaStreamWaitEvent(b->groups[q]->s, c0.e0, 0));
  for (int k = 0; k < nsteps; ++k)
    for (auto &c : b->groups)
      if (launch_step(*c)) return 1;
  for (size_t q = 1; q < b->groups.size(); ++q) {
    CK(cudaEventRecord(b->groups[q]->e1, b->groups[q]->s));
    CK(cudaStreamWaitEvent(c0.s, b->groups[q]->e1, 0));
  }
  CK(cudaEventRecord(c0.e1, c0.s));
  for (auto &c : b->groups)
    if (sync(*c)) return 1;
  CK(cudaEventElapsedTime(ms, c0.e0, c0.e1));
  return batch_read_dt(*b, (int)b->group_of.size(), nullptr);
}

int sbfs_batch_sync_to_host(int n, const domain_t *const *domains, fluid_t *const *fluids,
                            interface_t *const *interfaces) {
  (void)domains;
  Batch *b = g_batch.get();
  if (!b || (int)b->group_of.size() != n) return fail("no batch of %d cases on the device", n);
  for (int i = 0; i < n; ++i)
    if (b->ident[2 * i] != fluids[i] || b->ident[2 * i + 1] != interfaces[i])
      return fail("case %d is not the one the batch holds", i);
  if (batch_download(*b, n, fluids, interfaces, g_sync_mode == SBFS_SYNC_ALL)) return 1;
  for (auto &c : b->groups)
    if (sync(*c)) return 1;
  return 0;
}

// per-kernel-class device time of nsteps eager steps of the resident batch
int sbfs_profile_batch_steps(int nsteps, float *ms_per_class, int *launches_per_class) {
  Batch *b = g_batch.get();
  if (!b) return fail("no batch on the device: call sbfs_integrate_batch first");
  for (auto &c : b->groups)
    if (!c->resident) return fail("the batch's state is not on the device");
  g_prof.on = true;
  g_prof.used = 0;
  g_prof.marks.clear();
  int rc = 0;
  for (int k = 0; k < nsteps && !rc; ++k)
    for (auto &c : b->groups)
      if (!rc) rc = launch_step(*c);
  g_prof.on = false;
  if (rc) return 1;
  for (auto &c : b->groups)
    if (sync(*c)) return 1;
  for (int k = 0; k < KC_COUNT; ++k) {
    ms_per_class[k] = 0.f;
    launches_per_class[k] = 0;
  }
  for (auto &mk : g_prof.marks) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, mk.second.first, mk.second.second));
    ms_per_class[mk.first] += ms;
    launches_per_class[mk.first] += 1;
  }
  return batch_read_dt(*b, (int)b->group_of.size(), nullptr);
}

int sbfs_set_autotune(int on) {
  g_autotune = on ? 1 : 0;
  return 0;
}

// launch shapes in use: group -1 = the single-case context, else batch group
int sbfs_tiles(int group, int *bx, int *by, int *fft_w, int *tdm_mb, int *tdm_warps, int *compact) {
  Ctx *c = nullptr;
  if (group < 0)
    c = g_ctx.get();
  else if (g_batch && group < (int)g_batch->groups.size())
    c = g_batch->groups[group].get();
  if (!c) return fail("no such context");
  for (int k = 0; k < TK_COUNT; ++k) {
    bx[k] = c->b.tiles.bx[k];
    by[k] = c->b.tiles.by[k];
  }
  *fft_w = c->b.tiles.fft_w;
  *tdm_mb = tdm_uses_cluster(c->b.tiles, c->nx) ? 0 : tdm_modes_per_block(c->b.tiles, c->nx);
  *tdm_warps = c->b.tiles.tdm_g > 0 ? c->b.tiles.tdm_g : 1;
  if (compact) *compact = c->b.tiles.compact;
  return 0;
}

int sbfs_batch_groups(int *ngroups, int *cases) {
  Batch *b = g_batch.get();
  *ngroups = b ? (int)b->groups.size() : 0;
  if (b && cases)
    for (size_t q = 0; q < b->groups.size(); ++q) cases[q] = b->groups[q]->nc;
  return 0;
}

int sbfs_batch_release(void) {
  g_batch.reset();
  return 0;
}

int sbfs_run_steps_timed(const domain_t *d, fluid_t *f, interface_t *itf, int nsteps, float *ms, double *dt_last) {
  Ctx *c = prepare_step(d, f, itf);
  if (!c) return 1;
  if (!c->resident) {
    if (upload_state(*c, f, itf)) return 1;
  }
  CK(cudaEventRecord(c->e0, c->s));
  for (int n = 0; n < nsteps; ++n)
    if (launch_step(*c)) return 1;
  CK(cudaEventRecord(c->e1, c->s));
  if (sync(*c)) return 1;
  CK(cudaEventElapsedTime(ms, c->e0, c->e1));
  int status = 0;
  if (read_dt_status(*c, dt_last, &status)) return 1;
  if (status & 1) return fail("non-finite velocity detected by decide_dt");
  return 0;
}

// reference src/decide_dt.c:140-169
int decide_dt(const domain_t *d, const fluid_t *f, const interface_t *itf, double *dt) {
  Ctx *c = prepare_step(d, const_cast<fluid_t *>(f), const_cast<interface_t *>(itf));
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  if (h2d(*c, f->ux, L_UX, c->b.ux) || h2d(*c, f->uy, L_UY, c->b.uy)) return 1;
  launch_decide_dt(c->s, c->g, c->m, c->ph, c->b, c->b.ux, c->b.uy, c->dt_fixed, g_coef[0]);
  int status = 0;
  if (read_dt_status(*c, dt, &status)) return 1;
  if (status & 1) {
    CK(cudaMemsetAsync(c->b.status, 0, sizeof(int), c->s));
    return fail("non-finite velocity detected by decide_dt");
  }
  return 0;
}

// reference src/fluid/density.c:9-31
int fluid_compute_density(const domain_t *d, fluid_t *f, const interface_t *itf, const size_t index) {
  if (index > 1) return fail("density index %zu out of range", index);
  Ctx *c = get_ctx(d, f, itf);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  if (h2d(*c, itf->vof, L_VOF, c->b.vof)) return 1;
  launch_props(c->s, c->g, c->m, c->ph, c->b, true, false, false, c->b.den0);
  if (d2h(*c, f->den[index], L_DEN, c->b.den0)) return 1;
  return sync(*c);
}

// reference src/fluid/viscosity.c:93-108
int fluid_compute_viscosity(const domain_t *d, fluid_t *f, const interface_t *itf) {
  Ctx *c = get_ctx(d, f, itf);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  if (h2d(*c, itf->vof, L_VOF, c->b.vof)) return 1;
  launch_props(c->s, c->g, c->m, c->ph, c->b, false, true, false, nullptr);
  if (d2h(*c, f->visux, L_VISUX, c->b.visux) || d2h(*c, f->visuy, L_VISUY, c->b.visuy)) return 1;
  return sync(*c);
}

// reference src/interface/curvature_tensor.c:137-145
int interface_compute_curvature_tensor(const domain_t *d, interface_t *itf) {
  Ctx *c = get_ctx(d, nullptr, itf);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  // cells outside the interface band keep their previous normal, as in the reference
  if (h2d(*c, itf->vof, L_VOF, c->b.vof) || h2d(*c, itf->normal, L_NORMAL, c->b.normal)) return 1;
  launch_props(c->s, c->g, c->m, c->ph, c->b, false, false, true, nullptr);
  launch_normal_curv(c->s, c->g, c->m, c->b, true, true, false);
  if (d2h(*c, itf->dvof, L_DVOF, c->b.dvof) || d2h(*c, itf->normal, L_NORMAL, c->b.normal) ||
      d2h(*c, itf->curv, L_CURV, c->b.curv))
    return 1;
  return sync(*c);
}

// reference src/interface/force.c:90-98
int interface_compute_force(const domain_t *d, const fluid_t *f, interface_t *itf) {
  Ctx *c = get_ctx(d, f, itf);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  if (h2d(*c, f->den[0], L_DEN, c->b.den0) || h2d(*c, itf->vof, L_VOF, c->b.vof) ||
      h2d(*c, itf->curv, L_CURV, c->b.curv))
    return 1;
  launch_flux_force(c->s, c->g, c->m, c->ph, c->b, c->b.ux, c->b.uy, c->b.den0, false, true, false);
  if (d2h(*c, itf->ifrcx, L_IFRCX, c->b.ifrcx) || d2h(*c, itf->ifrcy, L_IFRCY, c->b.ifrcy)) return 1;
  return sync(*c);
}

// reference src/interface/update/main.c:122-136
int interface_update_vof(const domain_t *d, const size_t rkstep, const double dt, const fluid_t *f,
                         interface_t *itf) {
  if (rkstep > 2) return fail("rkstep %zu out of range", rkstep);
  Ctx *c = get_ctx(d, f, itf);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  if (rkstep != 0) swap_data(itf->src[0], itf->src[1]);
  Bufs &b = c->b;
  if (h2d(*c, f->ux, L_UX, b.ux) || h2d(*c, f->uy, L_UY, b.uy) || h2d(*c, itf->vof, L_VOF, b.vof) ||
      h2d(*c, itf->normal, L_NORMAL, b.normal) || h2d(*c, itf->src[1], L_SRC, b.srcvof[1]))
    return 1;
  if (put_scalars(*c, dt, (int)rkstep, 0., 0.)) return 1;
  launch_flux_force(c->s, c->g, c->m, c->ph, b, b.ux, b.uy, b.den0, true, false, false);
  launch_vof_advance(c->s, c->g, c->m, c->ph, b, b.scalars, (int)rkstep, b.srcvof[0], b.srcvof[1], false, b.ux,
                     b.uy, nullptr);
  if (d2h(*c, itf->fluxx, L_FLUXX, b.fluxx) || d2h(*c, itf->fluxy, L_FLUXY, b.fluxy) ||
      d2h(*c, itf->src[0], L_SRC, b.srcvof[0]) || d2h(*c, itf->vof, L_VOF, b.vof))
    return 1;
  return sync(*c);
}

// reference src/interface/mass_flux.c:48-58
int interface_compute_mass_flux(const domain_t *d, const fluid_t *f, interface_t *itf) {
  Ctx *c = get_ctx(d, f, itf);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  Bufs &b = c->b;
  if (h2d(*c, f->ux, L_UX, b.ux) || h2d(*c, f->uy, L_UY, b.uy) || h2d(*c, itf->fluxx, L_FLUXX, b.fluxx) ||
      h2d(*c, itf->fluxy, L_FLUXY, b.fluxy))
    return 1;
  launch_mass_flux_inplace(c->s, c->g, c->ph, b, b.ux, b.uy);
  if (d2h(*c, itf->fluxx, L_FLUXX, b.fluxx) || d2h(*c, itf->fluxy, L_FLUXY, b.fluxy)) return 1;
  return sync(*c);
}

// reference src/fluid/predict/main.c:60-80
int fluid_predict_field(const domain_t *d, const size_t rkstep, const double dt, fluid_t *f,
                        const interface_t *itf) {
  if (rkstep > 2) return fail("rkstep %zu out of range", rkstep);
  Ctx *c = get_ctx(d, f, itf);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  if (rkstep != 0) {
    swap_data(f->srcux[0], f->srcux[1]);
    swap_data(f->srcuy[0], f->srcuy[1]);
  }
  Bufs &b = c->b;
  if (h2d(*c, f->ux, L_UX, b.ux) || h2d(*c, f->uy, L_UY, b.uy) || h2d(*c, f->visux, L_VISUX, b.visux) ||
      h2d(*c, f->visuy, L_VISUY, b.visuy) || h2d(*c, itf->fluxx, L_FLUXX, b.mfluxx) ||
      h2d(*c, itf->fluxy, L_FLUXY, b.mfluxy) || h2d(*c, f->p, L_P, b.p) || h2d(*c, itf->ifrcx, L_IFRCX, b.ifrcx) ||
      h2d(*c, itf->ifrcy, L_IFRCY, b.ifrcy) || h2d(*c, f->den[0], L_DEN, b.den0) ||
      h2d(*c, f->den[1], L_DEN, b.den1) || h2d(*c, f->srcux[1], L_SRCUX, b.srcux[1]) ||
      h2d(*c, f->srcuy[1], L_SRCUY, b.srcuy[1]))
    return 1;
  if (put_scalars(*c, dt, (int)rkstep, 0., 0.)) return 1;
  launch_stress(c->s, c->g, c->m, b, b.ux, b.uy);
  launch_predict(c->s, c->g, c->m, c->ph, b, b.scalars, (int)rkstep, b.ux, b.uy, b.ux_star, b.uy_star, b.mfluxx,
                 b.mfluxy, b.den0, b.den1, b.srcux[0], b.srcux[1], b.srcux[2], b.srcuy[0], b.srcuy[1], b.srcuy[2]);
  if (d2h(*c, f->txx, L_TXX, b.txx) || d2h(*c, f->txy, L_TXY, b.txy) || d2h(*c, f->tyy, L_TYY, b.tyy) ||
      d2h(*c, f->srcux[0], L_SRCUX, b.srcux[0]) || d2h(*c, f->srcux[2], L_SRCUX, b.srcux[2]) ||
      d2h(*c, f->srcuy[0], L_SRCUY, b.srcuy[0]) || d2h(*c, f->srcuy[2], L_SRCUY, b.srcuy[2]) ||
      d2h(*c, f->ux, L_UX, b.ux_star) || d2h(*c, f->uy, L_UY, b.uy_star))
    return 1;
  return sync(*c);
}

// reference src/fluid/compute_potential.c:421-469
int fluid_compute_potential(const domain_t *d, const double dt_old, const double dt_new, fluid_t *f) {
  Ctx *c = get_ctx(d, f, nullptr);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  Bufs &b = c->b;
  if (h2d(*c, f->ux, L_UX, b.ux) || h2d(*c, f->uy, L_UY, b.uy) || h2d(*c, f->psi[0], L_P, b.psi0) ||
      h2d(*c, f->den[1], L_DEN, b.den1))
    return 1;
  if (put_scalars(*c, 0., -1, dt_old, dt_new)) return 1;
  launch_face_factor(c->s, c->g, c->ph, b, b.den1, b.psi0);
  launch_poisson(c->s, c->g, b, b.scalars, 0, b.ux, b.uy, b.psi1);
  if (d2h(*c, f->psi[1], L_P, b.psi1)) return 1;
  return sync(*c);
}

// reference src/fluid/correct_velocity/main.c:14-28
int fluid_correct_velocity(const domain_t *d, const double dt_old, const double dt_new, fluid_t *f) {
  Ctx *c = get_ctx(d, f, nullptr);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  Bufs &b = c->b;
  if (h2d(*c, f->ux, L_UX, b.ux) || h2d(*c, f->uy, L_UY, b.uy) || h2d(*c, f->psi[0], L_P, b.psi0) ||
      h2d(*c, f->psi[1], L_P, b.psi1) || h2d(*c, f->den[1], L_DEN, b.den1))
    return 1;
  if (put_scalars(*c, 0., -1, dt_old, dt_new)) return 1;
  launch_face_factor(c->s, c->g, c->ph, b, b.den1, b.psi0);
  launch_correct(c->s, c->g, c->m, b, b.scalars, 0, b.ux, b.uy, b.psi1, false, false);
  if (d2h(*c, f->ux, L_UX, b.ux) || d2h(*c, f->uy, L_UY, b.uy)) return 1;
  return sync(*c);
}

// reference src/fluid/update_pressure.c:43-53
int fluid_update_pressure(const domain_t *d, fluid_t *f) {
  Ctx *c = get_ctx(d, f, nullptr);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  if (h2d(*c, f->p, L_P, c->b.p) || h2d(*c, f->psi[1], L_P, c->b.psi1)) return 1;
  launch_pressure(c->s, c->g, c->b, c->b.psi1);
  if (d2h(*c, f->p, L_P, c->b.p)) return 1;
  if (sync(*c)) return 1;
  swap_data(f->psi[0], f->psi[1]);
  return 0;
}

static int bc_call(const domain_t *d, array_t *a, const Layout &l, int kind) {
  Ctx *c = get_ctx(d, nullptr, nullptr);
  if (!c) return 1;
  c->resident = false;
  state_touched(*c);
  double *buf = c->b.txy;  // scratch
  if (h2d(*c, *a, l, buf)) return 1;
  if (kind == 0) launch_bc_ux(c->s, c->g, buf);
  else if (kind == 1) launch_bc_uy(c->s, c->g, buf);
  else if (kind == 2) launch_bc_neumann(c->s, c->g, buf);
  else launch_bc_vof(c->s, c->g, buf);
  if (d2h(*c, *a, l, buf)) return 1;
  return sync(*c);
}

// reference src/fluid/boundary/{ux,uy,p,psi}.c, src/interface/boundary.c
int fluid_update_boundaries_ux(const domain_t *d, array_t *a) { return bc_call(d, a, L_UX, 0); }
int fluid_update_boundaries_uy(const domain_t *d, array_t *a) { return bc_call(d, a, L_UY, 1); }
int fluid_update_boundaries_p(const domain_t *d, array_t *a) { return bc_call(d, a, L_P, 2); }
int fluid_update_boundaries_psi(const domain_t *d, array_t *a) { return bc_call(d, a, L_P, 2); }
int interface_update_boundaries_vof(const domain_t *d, array_t *a) { return bc_call(d, a, L_VOF, 3); }

}  // extern "C"
