/*
 * CPU oracle for the 2-D two-phase time step of SimpleBubblyFlowSolver.
 *
 * TEST INFRASTRUCTURE ONLY (see sbfs_oracle.h): the checker for the CUDA
 * library and the timed CPU baseline, never part of the product path.
 *
 * Each operator restates the discretisation of the reference function cited
 * in its comment (paths relative to the reference project root).  The
 * arithmetic is written in the same evaluation order as the reference so that
 * this restatement agrees bit-for-bit with the reference's own sources built
 * with the same compiler flags; that agreement is what pins the oracle.
 * Loops over rows are parallelised with OpenMP; every cell is independent,
 * so results do not depend on the thread count.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "dct.h"
#include "sbfs_oracle.h"

/* ------------------------------------------------------------------------ */
/* constants                                                                */
/* ------------------------------------------------------------------------ */

/* three-stage low-storage RK (src/runge_kutta.c:8-15): alpha, beta, gamma */
static const double rk_alpha[3] = {32. / 60., 25. / 60., 45. / 60.};
static const double rk_beta[3] = {0. / 60., -17. / 60., -25. / 60.};
static double rk_gamma(int k) { return rk_alpha[k] + rk_beta[k]; }

/* THINC constants (src/interface/common.c:4-14) */
static const double thinc_gauss_pt[2] = {-0.2886751345948129, +0.2886751345948129};
static const double thinc_gauss_wt[2] = {+0.5, +0.5};
static const double thinc_beta = 1.;
static const double thinc_vofmin = 1.e-8;

/* wall tangential velocities (src/param/boundary-condition.c:3-4) */
static const double wall_uy_xm = 0.;
static const double wall_uy_xp = 0.;

static double dt_coef_adv = -1., dt_coef_dif = -1., dt_coef_int = -1.;
static int n_threads = 0;

void orc_set_threads(int nthreads) { n_threads = nthreads; }
int orc_get_threads(void) {
#ifdef _OPENMP
  return n_threads > 0 ? n_threads : omp_get_max_threads();
#else
  return 1;
#endif
}
#define OMP_FOR _Pragma("omp parallel for schedule(static) num_threads(orc_get_threads())")

/* ------------------------------------------------------------------------ */
/* field views                                                              */
/* ------------------------------------------------------------------------ */

/* element (I, J[, c]) of an array_t using its own ghost widths */
typedef struct {
  double *d;
  long ox, oy, pitch;
  int nc;
} fview;

static fview view_of(const domain_t *dom, const array_t *a, int ncomp) {
  fview v;
  v.d = (double *)a->data;
  v.ox = a->nadds[0][0] - 1;
  v.oy = a->nadds[1][0] - 1;
  v.pitch = (long)dom->mysizes[0] + a->nadds[0][0] + a->nadds[0][1];
  v.nc = ncomp;
  return v;
}
#define F(v, I, J) ((v).d[((long)(I) + (v).ox) + (v).pitch * ((long)(J) + (v).oy)])
#define FC(v, I, J, c) ((v).d[(((long)(I) + (v).ox) + (v).pitch * ((long)(J) + (v).oy)) * (v).nc + (c)])

/* metric arrays: HXXF/JDXF at faces I = 1..nx+1, HXXC/JDXC at centres 1..nx */
#define HXXF(I) (dom->hxxf[(I)-1])
#define HXXC(I) (dom->hxxc[(I)-1])
#define JDXF(I) (dom->jdxf[(I)-1])
#define JDXC(I) (dom->jdxc[(I)-1])

/* periodic y ghost rows: whole rows, x ghosts included (src/halo.c:18-76) */
static int fill_y_ghosts(const domain_t *dom, array_t *a) {
  const int ng = a->nadds[1][0];
  if (ng != a->nadds[1][1]) return 1;
  const long ny = (long)dom->mysizes[1];
  const long rowlen = ((long)dom->mysizes[0] + a->nadds[0][0] + a->nadds[0][1]) * (long)(a->size / sizeof(double));
  double *d = (double *)a->data;
  /* memory row r holds J = r + 1 - ng */
  for (int g = 0; g < ng; g++) {
    /* lower ghost J = 1 - ng + g  <-  J + ny */
    memcpy(d + rowlen * g, d + rowlen * (g + ny), sizeof(double) * rowlen);
    /* upper ghost J = ny + 1 + g  <-  J - ny */
    memcpy(d + rowlen * (ng + ny + g), d + rowlen * (ng + g), sizeof(double) * rowlen);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* boundary conditions (src/fluid/boundary/{ux,uy,p,psi}.c, src/interface/boundary.c)    */
/* ------------------------------------------------------------------------ */

int orc_fluid_update_boundaries_ux(const domain_t *dom, array_t *arr) {
  /* impermeable walls: ux = 0 on both wall faces (src/fluid/boundary/ux.c:27-33) */
  fview ux = view_of(dom, arr, 1);
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  for (int j = 1; j <= ny; j++) {
    F(ux, 1, j) = 0.;
    F(ux, nx + 1, j) = 0.;
  }
  return fill_y_ghosts(dom, arr);
}

int orc_fluid_update_boundaries_uy(const domain_t *dom, array_t *arr) {
  /* prescribed wall tangential velocity in the x ghost cells (src/fluid/boundary/uy.c:28-34) */
  fview uy = view_of(dom, arr, 1);
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  for (int j = 1; j <= ny; j++) {
    F(uy, 0, j) = wall_uy_xm;
    F(uy, nx + 1, j) = wall_uy_xp;
  }
  return fill_y_ghosts(dom, arr);
}

static int neumann_x(const domain_t *dom, array_t *arr) {
  fview f = view_of(dom, arr, 1);
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  for (int j = 1; j <= ny; j++) {
    F(f, 0, j) = F(f, 1, j);
    F(f, nx + 1, j) = F(f, nx, j);
  }
  return fill_y_ghosts(dom, arr);
}

/* src/fluid/boundary/p.c:17-44 and psi.c:17-44: zero normal gradient at walls */
int orc_fluid_update_boundaries_p(const domain_t *dom, array_t *arr) { return neumann_x(dom, arr); }
int orc_fluid_update_boundaries_psi(const domain_t *dom, array_t *arr) { return neumann_x(dom, arr); }

int orc_interface_update_boundaries_vof(const domain_t *dom, array_t *arr) {
  /* vof = 0 in the wall ghost cells, two periodic ghost rows (src/interface/boundary.c:15-42) */
  fview vof = view_of(dom, arr, 1);
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  for (int j = 1; j <= ny; j++) {
    F(vof, 0, j) = 0.;
    F(vof, nx + 1, j) = 0.;
  }
  return fill_y_ghosts(dom, arr);
}

/* ------------------------------------------------------------------------ */
/* material properties                                                      */
/* ------------------------------------------------------------------------ */

/* src/fluid/density.c:9-31: clipped linear mixture over all cells incl. ghosts */
int orc_fluid_compute_density(const domain_t *dom, fluid_t *fl, const interface_t *itf, size_t index) {
  if (index > 1) return 1;
  fview den = view_of(dom, &fl->den[index], 1);
  fview vof = view_of(dom, &itf->vof, 1);
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double r = fl->denr;
  const double lo = fmin(1., r), hi = fmax(1., r);
  OMP_FOR
  for (int j = 0; j <= ny + 1; j++) {
    for (int i = 0; i <= nx + 1; i++) {
      double v = 1. + (r - 1.) * F(vof, i, j);
      v = fmax(lo, v);
      v = fmin(hi, v);
      F(den, i, j) = v;
    }
  }
  return 0;
}

static double mix_clip(double ratio, double lo, double hi, double phi) {
  double v = 1. + (ratio - 1.) * phi;
  v = fmax(lo, v);
  return fmin(hi, v);
}

/* src/fluid/viscosity.c:23-108: face-averaged vof -> clipped viscosity */
int orc_fluid_compute_viscosity(const domain_t *dom, fluid_t *fl, const interface_t *itf) {
  fview vof = view_of(dom, &itf->vof, 1);
  fview vx = view_of(dom, &fl->visux, 1);
  fview vy = view_of(dom, &fl->visuy, 1);
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double r = fl->visr;
  const double lo = fmin(1., r), hi = fmax(1., r);
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    /* wall faces take the ghost-cell vof */
    F(vx, 1, j) = mix_clip(r, lo, hi, F(vof, 0, j));
    for (int i = 2; i <= nx; i++)
      F(vx, i, j) = mix_clip(r, lo, hi, +0.5 * F(vof, i - 1, j) + 0.5 * F(vof, i, j));
    F(vx, nx + 1, j) = mix_clip(r, lo, hi, F(vof, nx + 1, j));
  }
  if (fill_y_ghosts(dom, &fl->visux)) return 1;
  OMP_FOR
  for (int j = 1; j <= ny; j++)
    for (int i = 0; i <= nx + 1; i++)
      F(vy, i, j) = mix_clip(r, lo, hi, +0.5 * F(vof, i, j - 1) + 0.5 * F(vof, i, j));
  return fill_y_ghosts(dom, &fl->visuy);
}

/* ------------------------------------------------------------------------ */
/* interface geometry (src/interface/curvature_tensor.c)                    */
/* ------------------------------------------------------------------------ */

int orc_interface_compute_curvature_tensor(const domain_t *dom, interface_t *itf) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  fview vof = view_of(dom, &itf->vof, 1);
  fview dv = view_of(dom, &itf->dvof, 2);
  fview nrm = view_of(dom, &itf->normal, 3);
  fview curv = view_of(dom, &itf->curv, 1);
  /* :16-49 normalised vof gradient at cell corners (faces i, j-1/2) */
  OMP_FOR
  for (int j = 0; j <= ny + 2; j++) {
    for (int i = 1; i <= nx + 1; i++) {
      const double gx = 1. / HXXF(i) * (-F(vof, i - 1, j - 1) + F(vof, i, j - 1) - F(vof, i - 1, j) + F(vof, i, j));
      const double gy = 1. / hy * (-F(vof, i - 1, j - 1) - F(vof, i, j - 1) + F(vof, i - 1, j) + F(vof, i, j));
      const double mag = sqrt(pow(gx, 2.) + pow(gy, 2.));
      const double inv = 1. / fmax(mag, DBL_EPSILON);
      FC(dv, i, j, 0) = gx * inv;
      FC(dv, i, j, 1) = gy * inv;
    }
  }
  /* :51-97 cell-centred normal and THINC intercept, interface cells only */
  OMP_FOR
  for (int j = 0; j <= ny + 1; j++) {
    for (int i = 1; i <= nx; i++) {
      const double phi = F(vof, i, j);
      if (phi < thinc_vofmin || 1. - thinc_vofmin < phi) continue;
      double mx = (FC(dv, i, j, 0) + FC(dv, i + 1, j, 0) + FC(dv, i, j + 1, 0) + FC(dv, i + 1, j + 1, 0));
      double my = (FC(dv, i, j, 1) + FC(dv, i + 1, j, 1) + FC(dv, i, j + 1, 1) + FC(dv, i + 1, j + 1, 1));
      mx /= HXXC(i);
      my /= hy;
      const double mag = sqrt(pow(mx, 2.) + pow(my, 2.));
      const double inv = 1. / fmax(mag, DBL_EPSILON);
      mx *= inv;
      my *= inv;
      FC(nrm, i, j, 0) = mx;
      FC(nrm, i, j, 1) = my;
      FC(nrm, i, j, 2) = -0.5 / thinc_beta * log(1. / phi - 1.);
    }
  }
  /* :100-135 curvature = -div(corner normals) */
  OMP_FOR
  for (int j = 0; j <= ny + 1; j++) {
    for (int i = 1; i <= nx; i++) {
      const double hxm = HXXF(i), hxp = HXXF(i + 1);
      const double jdm = JDXF(i), jd0 = JDXC(i), jdp = JDXF(i + 1);
      const double nxm = +0.5 * FC(dv, i, j, 0) + 0.5 * FC(dv, i, j + 1, 0);
      const double nxp = +0.5 * FC(dv, i + 1, j, 0) + 0.5 * FC(dv, i + 1, j + 1, 0);
      const double nym = +0.5 * FC(dv, i, j, 1) + 0.5 * FC(dv, i + 1, j, 1);
      const double nyp = +0.5 * FC(dv, i, j + 1, 1) + 0.5 * FC(dv, i + 1, j + 1, 1);
      const double div = 1. / jd0 * (-jdm / hxm * nxm + jdp / hxp * nxp - jd0 / hy * nym + jd0 / hy * nyp);
      F(curv, i, j) = -1. * div;
    }
  }
  return 0;
}

/* src/interface/force.c:14-98: CSF force at ux and uy faces */
int orc_interface_compute_force(const domain_t *dom, const fluid_t *fl, interface_t *itf) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  const double tension = 1. / itf->We;
  const double dscale = 2. / (1. + fl->denr);
  fview den = view_of(dom, &fl->den[0], 1);
  fview vof = view_of(dom, &itf->vof, 1);
  fview curv = view_of(dom, &itf->curv, 1);
  fview fx = view_of(dom, &itf->ifrcx, 1);
  fview fy = view_of(dom, &itf->ifrcy, 1);
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 2; i <= nx; i++) {
      const double rho = (+0.5 * F(den, i - 1, j) + 0.5 * F(den, i, j));
      const double kap = (+0.5 * F(curv, i - 1, j) + 0.5 * F(curv, i, j));
      const double dlt = 1. / HXXF(i) * (-F(vof, i - 1, j) + F(vof, i, j));
      F(fx, i, j) = rho * dscale * tension * kap * dlt;
    }
  }
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double rho = (+0.5 * F(den, i, j - 1) + 0.5 * F(den, i, j));
      const double kap = (+0.5 * F(curv, i, j - 1) + 0.5 * F(curv, i, j));
      const double dlt = 1. / hy * (-F(vof, i, j - 1) + F(vof, i, j));
      F(fy, i, j) = rho * dscale * tension * kap * dlt;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* VOF transport (src/interface/update/{main,fluxx,fluxy}.c)                             */
/* ------------------------------------------------------------------------ */

/* smoothed indicator 0.5 (1 + tanh(beta (n . x + d))) (update/main.c:18-35) */
static double thinc_indicator(const double *n, double x, double y) {
  const double s = n[0] * x + n[1] * y + n[2];
  return 0.5 * (1. + tanh(thinc_beta * s));
}

static void swap_data(array_t *a, array_t *b) {
  void *t = a->data;
  a->data = b->data;
  b->data = t;
}

int orc_interface_update_vof(const domain_t *dom, size_t rkstep, double dt, const fluid_t *fl, interface_t *itf) {
  if (rkstep > 2) return 1;
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  /* keep the previous stage's source: pointer swap (update/main.c:37-52) */
  if (rkstep != 0) swap_data(&itf->src[0], &itf->src[1]);
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  fview vof = view_of(dom, &itf->vof, 1);
  fview nrm = view_of(dom, &itf->normal, 3);
  fview fxv = view_of(dom, &itf->fluxx, 1);
  fview fyv = view_of(dom, &itf->fluxy, 1);
  /* x faces: upwind-cell THINC flux (update/fluxx.c:39-73) */
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 2; i <= nx; i++) {
      const double vel = F(ux, i, j);
      const int iu = vel < 0. ? i : i - 1;
      const double xq = vel < 0. ? -0.5 : +0.5;
      const double phi = F(vof, iu, j);
      if (phi < thinc_vofmin || 1. - thinc_vofmin < phi) {
        F(fxv, i, j) = vel * phi;
        continue;
      }
      const double n[3] = {FC(nrm, iu, j, 0), FC(nrm, iu, j, 1), FC(nrm, iu, j, 2)};
      double acc = 0.;
      for (int q = 0; q < 2; q++) acc += thinc_gauss_wt[q] * thinc_indicator(n, xq, thinc_gauss_pt[q]);
      F(fxv, i, j) = vel * acc;
    }
  }
  for (int j = 1; j <= ny; j++) {
    F(fxv, 1, j) = 0.;
    F(fxv, nx + 1, j) = 0.;
  }
  if (fill_y_ghosts(dom, &itf->fluxx)) return 1;
  /* y faces (update/fluxy.c:39-73) */
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double vel = F(uy, i, j);
      const int ju = vel < 0. ? j : j - 1;
      const double yq = vel < 0. ? -0.5 : +0.5;
      const double phi = F(vof, i, ju);
      if (phi < thinc_vofmin || 1. - thinc_vofmin < phi) {
        F(fyv, i, j) = vel * phi;
        continue;
      }
      const double n[3] = {FC(nrm, i, ju, 0), FC(nrm, i, ju, 1), FC(nrm, i, ju, 2)};
      double acc = 0.;
      for (int q = 0; q < 2; q++) acc += thinc_gauss_wt[q] * thinc_indicator(n, thinc_gauss_pt[q], yq);
      F(fyv, i, j) = vel * acc;
    }
  }
  for (int j = 1; j <= ny; j++) {
    F(fyv, 0, j) = 0.;
    F(fyv, nx + 1, j) = 0.;
  }
  if (fill_y_ghosts(dom, &itf->fluxy)) return 1;
  /* flux divergence (update/main.c:54-88) */
  fview sa = view_of(dom, &itf->src[0], 1);
  fview sb = view_of(dom, &itf->src[1], 1);
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double hxm = HXXF(i), hxp = HXXF(i + 1);
      const double jdm = JDXF(i), jd0 = JDXC(i), jdp = JDXF(i + 1);
      F(sa, i, j) = 1. / jd0 * (+jdm / hxm * F(fxv, i, j) - jdp / hxp * F(fxv, i + 1, j)
                                + jd0 / hy * F(fyv, i, j) - jd0 / hy * F(fyv, i, j + 1));
    }
  }
  /* RK update, alpha then beta contribution (update/main.c:90-120) */
  {
    const double c = rk_alpha[rkstep];
    OMP_FOR
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) F(vof, i, j) += dt * c * F(sa, i, j);
  }
  if (rkstep != 0) {
    const double c = rk_beta[rkstep];
    OMP_FOR
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) F(vof, i, j) += dt * c * F(sb, i, j);
  }
  return orc_interface_update_boundaries_vof(dom, &itf->vof);
}

/* src/interface/mass_flux.c:10-58: vof flux -> mass flux u + (rho_r - 1) flux, ghosts included */
int orc_interface_compute_mass_flux(const domain_t *dom, const fluid_t *fl, interface_t *itf) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double r = fl->denr;
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  fview fxv = view_of(dom, &itf->fluxx, 1);
  fview fyv = view_of(dom, &itf->fluxy, 1);
  OMP_FOR
  for (int j = 0; j <= ny + 1; j++)
    for (int i = 1; i <= nx + 1; i++) F(fxv, i, j) = F(ux, i, j) + (r - 1.) * F(fxv, i, j);
  OMP_FOR
  for (int j = 0; j <= ny + 1; j++)
    for (int i = 0; i <= nx + 1; i++) F(fyv, i, j) = F(uy, i, j) + (r - 1.) * F(fyv, i, j);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* momentum predictor (src/fluid/predict/{main,txx,txy,tyy,ux,uy}.c)                            */
/* ------------------------------------------------------------------------ */

static int stress_tensor(const domain_t *dom, fluid_t *fl) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  fview vx = view_of(dom, &fl->visux, 1);
  fview vy = view_of(dom, &fl->visuy, 1);
  fview txx = view_of(dom, &fl->txx, 1);
  fview txy = view_of(dom, &fl->txy, 1);
  fview tyy = view_of(dom, &fl->tyy, 1);
  /* txx at centres (txx.c:11-40) */
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double mu = +0.5 * F(vx, i, j) + 0.5 * F(vx, i + 1, j);
      const double du = -F(ux, i, j) + F(ux, i + 1, j);
      const double l = 1. / HXXC(i) * du;
      F(txx, i, j) = mu * l + mu * l;
    }
  }
  if (fill_y_ghosts(dom, &fl->txx)) return 1;
  /* txy at corners (txy.c:13-50) */
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx + 1; i++) {
      const double mux = +0.5 * F(vx, i, j - 1) + 0.5 * F(vx, i, j);
      const double muy = +0.5 * F(vy, i - 1, j) + 0.5 * F(vy, i, j);
      const double du = -F(ux, i, j - 1) + F(ux, i, j);
      const double dv = -F(uy, i - 1, j) + F(uy, i, j);
      const double lxy = 1. / hy * du;
      const double lyx = 1. / HXXF(i) * dv;
      F(txy, i, j) = mux * lxy + muy * lyx;
    }
  }
  if (fill_y_ghosts(dom, &fl->txy)) return 1;
  /* tyy at centres (tyy.c:10-38) */
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double mu = +0.5 * F(vy, i, j) + 0.5 * F(vy, i, j + 1);
      const double dv = -F(uy, i, j) + F(uy, i, j + 1);
      const double l = 1. / hy * dv;
      F(tyy, i, j) = mu * l + mu * l;
    }
  }
  return fill_y_ghosts(dom, &fl->tyy);
}

/* explicit terms of the ux equation at faces i = 2..nx (predict/ux.c:29-226).
 * The reference accumulates each term in its own sweep; per cell the order of
 * accumulation is the same here. */
static void rhs_ux(const domain_t *dom, const fluid_t *fl, const interface_t *itf) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  const double nu = 1. / fl->Re;
  const double grav = -1. / fl->Fr / fl->Fr;
  fview ux = view_of(dom, &fl->ux, 1);
  fview p = view_of(dom, &fl->p, 1);
  fview txx = view_of(dom, &fl->txx, 1);
  fview txy = view_of(dom, &fl->txy, 1);
  fview den = view_of(dom, &fl->den[0], 1);
  fview fxv = view_of(dom, &itf->fluxx, 1);
  fview fyv = view_of(dom, &itf->fluxy, 1);
  fview frc = view_of(dom, &itf->ifrcx, 1);
  fview sa = view_of(dom, &fl->srcux[0], 1);
  fview sg = view_of(dom, &fl->srcux[2], 1);
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 2; i <= nx; i++) {
      double a = F(sa, i, j);
      {
        /* advection in x (:29-61) */
        const double hm = HXXF(i - 1), h0 = HXXF(i), hp = HXXF(i + 1);
        const double jm = JDXF(i - 1), j0 = JDXF(i), jp = JDXF(i + 1);
        const double mm = +0.5 * jm / hm * F(fxv, i - 1, j) + 0.5 * j0 / h0 * F(fxv, i, j);
        const double mp = +0.5 * j0 / h0 * F(fxv, i, j) + 0.5 * jp / hp * F(fxv, i + 1, j);
        const double um = +0.5 * F(ux, i - 1, j) + 0.5 * F(ux, i, j);
        const double up = +0.5 * F(ux, i, j) + 0.5 * F(ux, i + 1, j);
        a -= 1. / j0 * (-mm * um + mp * up);
      }
      {
        /* advection in y (:63-93) */
        const double jm = JDXC(i - 1), j0 = JDXF(i), jp = JDXC(i);
        const double mm = +0.5 * jm / hy * F(fyv, i - 1, j) + 0.5 * jp / hy * F(fyv, i, j);
        const double mp = +0.5 * jm / hy * F(fyv, i - 1, j + 1) + 0.5 * jp / hy * F(fyv, i, j + 1);
        const double um = +0.5 * F(ux, i, j - 1) + 0.5 * F(ux, i, j);
        const double up = +0.5 * F(ux, i, j) + 0.5 * F(ux, i, j + 1);
        a -= 1. / j0 * (-mm * um + mp * up);
      }
      {
        /* diffusion in x (:95-121) */
        const double hm = HXXC(i - 1), hp = HXXC(i);
        const double jm = JDXC(i - 1), j0 = JDXF(i), jp = JDXC(i);
        a += nu / j0 * (-jm / hm * F(txx, i - 1, j) + jp / hp * F(txx, i, j));
      }
      {
        /* diffusion in y (:123-144) */
        const double jd = JDXF(i);
        a += nu / jd * (-jd / hy * F(txy, i, j) + jd / hy * F(txy, i, j + 1));
      }
      /* pressure gradient into the gamma source (:146-162) */
      F(sg, i, j) -= 1. / HXXF(i) * (-F(p, i - 1, j) + F(p, i, j));
      /* surface tension and gravity (:164-192) */
      a += F(frc, i, j);
      a += grav * (+0.5 * F(den, i - 1, j) + 0.5 * F(den, i, j));
      F(sa, i, j) = a;
    }
  }
}

/* explicit terms of the uy equation at faces j = 1..ny (predict/uy.c:29-204) */
static void rhs_uy(const domain_t *dom, const fluid_t *fl, const interface_t *itf) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  const double nu = 1. / fl->Re;
  fview uy = view_of(dom, &fl->uy, 1);
  fview p = view_of(dom, &fl->p, 1);
  fview txy = view_of(dom, &fl->txy, 1);
  fview tyy = view_of(dom, &fl->tyy, 1);
  fview fxv = view_of(dom, &itf->fluxx, 1);
  fview fyv = view_of(dom, &itf->fluxy, 1);
  fview frc = view_of(dom, &itf->ifrcy, 1);
  fview sa = view_of(dom, &fl->srcuy[0], 1);
  fview sg = view_of(dom, &fl->srcuy[2], 1);
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      double a = F(sa, i, j);
      {
        /* advection in x (:29-64) */
        const double hm = HXXF(i), hp = HXXF(i + 1);
        const double jm = JDXF(i), j0 = JDXC(i), jp = JDXF(i + 1);
        const double mm = +0.5 * jm / hm * F(fxv, i, j - 1) + 0.5 * jm / hm * F(fxv, i, j);
        const double mp = +0.5 * jp / hp * F(fxv, i + 1, j - 1) + 0.5 * jp / hp * F(fxv, i + 1, j);
        const double um = +0.5 * F(uy, i - 1, j) + 0.5 * F(uy, i, j);
        const double up = +0.5 * F(uy, i, j) + 0.5 * F(uy, i + 1, j);
        a -= 1. / j0 * (-mm * um + mp * up);
      }
      {
        /* advection in y (:66-93) */
        const double jd = JDXC(i);
        const double mm = +0.5 * jd / hy * F(fyv, i, j - 1) + 0.5 * jd / hy * F(fyv, i, j);
        const double mp = +0.5 * jd / hy * F(fyv, i, j) + 0.5 * jd / hy * F(fyv, i, j + 1);
        const double um = +0.5 * F(uy, i, j - 1) + 0.5 * F(uy, i, j);
        const double up = +0.5 * F(uy, i, j) + 0.5 * F(uy, i, j + 1);
        a -= 1. / jd * (-mm * um + mp * up);
      }
      {
        /* diffusion in x (:95-122) */
        const double hm = HXXF(i), hp = HXXF(i + 1);
        const double jm = JDXF(i), j0 = JDXC(i), jp = JDXF(i + 1);
        a += nu / j0 * (-jm / hm * F(txy, i, j) + jp / hp * F(txy, i + 1, j));
      }
      {
        /* diffusion in y (:124-144) */
        const double jd = JDXC(i);
        a += nu / jd * (-jd / hy * F(tyy, i, j - 1) + jd / hy * F(tyy, i, j));
      }
      F(sg, i, j) -= 1. / hy * (-F(p, i, j - 1) + F(p, i, j));
      a += F(frc, i, j);
      F(sa, i, j) = a;
    }
  }
}

int orc_fluid_predict_field(const domain_t *dom, size_t rkstep, double dt, fluid_t *fl, const interface_t *itf) {
  if (rkstep > 2) return 1;
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  /* stash the previous stage's sources, clear the new ones (predict/main.c:9-29) */
  if (rkstep != 0) {
    swap_data(&fl->srcux[0], &fl->srcux[1]);
    swap_data(&fl->srcuy[0], &fl->srcuy[1]);
  }
  memset(fl->srcux[0].data, 0, fl->srcux[0].datasize);
  memset(fl->srcux[2].data, 0, fl->srcux[2].datasize);
  memset(fl->srcuy[0].data, 0, fl->srcuy[0].datasize);
  memset(fl->srcuy[2].data, 0, fl->srcuy[2].datasize);
  if (stress_tensor(dom, fl)) return 1;
  rhs_ux(dom, fl, itf);
  rhs_uy(dom, fl, itf);
  const double ca = rk_alpha[rkstep], cb = rk_beta[rkstep], cg = rk_gamma((int)rkstep);
  fview d0 = view_of(dom, &fl->den[0], 1);
  fview d1 = view_of(dom, &fl->den[1], 1);
  {
    /* predict_ux (ux.c:236-273): rho^k u + dt sum, then divide by rho^{k+1} */
    fview u = view_of(dom, &fl->ux, 1);
    fview sa = view_of(dom, &fl->srcux[0], 1);
    fview sb = view_of(dom, &fl->srcux[1], 1);
    fview sg = view_of(dom, &fl->srcux[2], 1);
    OMP_FOR
    for (int j = 1; j <= ny; j++) {
      for (int i = 2; i <= nx; i++) {
        const double r0 = +0.5 * F(d0, i - 1, j) + 0.5 * F(d0, i, j);
        double v = +r0 * F(u, i, j) + ca * dt * F(sa, i, j) + cb * dt * F(sb, i, j) + cg * dt * F(sg, i, j);
        const double r1 = +0.5 * F(d1, i - 1, j) + 0.5 * F(d1, i, j);
        v /= r1;
        F(u, i, j) = v;
      }
    }
    if (orc_fluid_update_boundaries_ux(dom, &fl->ux)) return 1;
  }
  {
    /* predict_uy (uy.c:214-251) */
    fview u = view_of(dom, &fl->uy, 1);
    fview sa = view_of(dom, &fl->srcuy[0], 1);
    fview sb = view_of(dom, &fl->srcuy[1], 1);
    fview sg = view_of(dom, &fl->srcuy[2], 1);
    OMP_FOR
    for (int j = 1; j <= ny; j++) {
      for (int i = 1; i <= nx; i++) {
        const double r0 = +0.5 * F(d0, i, j - 1) + 0.5 * F(d0, i, j);
        double v = +r0 * F(u, i, j) + ca * dt * F(sa, i, j) + cb * dt * F(sb, i, j) + cg * dt * F(sg, i, j);
        const double r1 = +0.5 * F(d1, i, j - 1) + 0.5 * F(d1, i, j);
        v /= r1;
        F(u, i, j) = v;
      }
    }
    if (orc_fluid_update_boundaries_uy(dom, &fl->uy)) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* pressure-potential Poisson solve (src/fluid/compute_potential.c)         */
/* ------------------------------------------------------------------------ */

/* Thomas algorithm on n rows with a zero-pivot guard on the last row
 * (src/tdm.c:17-50); v is scratch */
static void thomas(int n, double l, const double *c, double u, double *v, double *q) {
  v[0] = u / c[0];
  q[0] = q[0] / c[0];
  for (int i = 1; i < n - 1; i++) {
    const double w = 1. / (c[i] - l * v[i - 1]);
    v[i] = w * (u);
    q[i] = w * (q[i] - l * q[i - 1]);
  }
  const double w = c[n - 1] - l * v[n - 2];
  if (fabs(w) > DBL_EPSILON) q[n - 1] = 1. / w * (q[n - 1] - l * q[n - 2]);
  else q[n - 1] = 0.;
  for (int i = n - 2; i >= 0; i--) q[i] -= v[i] * q[i + 1];
}

/* cyclic tridiagonal system by Sherman-Morrison (src/tdm.c:66-106) with
 * constant off-diagonals l, u; q1, v scratch of n entries */
static void thomas_periodic(int n, double l, const double *c, double u, double *v, double *q1, double *q0) {
  for (int i = 0; i < n - 1; i++) q1[i] = i == 0 ? -l : i == n - 2 ? -u : 0.;
  thomas(n - 1, l, c, u, v, q1);
  thomas(n - 1, l, c, u, v, q0);
  const double num = q0[n - 1] - u * q0[0] - l * q0[n - 2];
  const double den = c[n - 1] + u * q1[0] + l * q1[n - 2];
  q0[n - 1] = fabs(den) < DBL_EPSILON ? 0. : num / den;
  for (int i = 0; i < n - 1; i++) q0[i] = q0[i] + q0[n - 1] * q1[i];
}

typedef struct {
  int nx, ny;
  double lx, hy;
  sbfs_dct_plan *dct;
  double *eig;   /* x eigenvalues of the DCT-diagonalised operator */
  double *rhs;   /* nx*ny, x-fastest */
  double *spec;  /* nx*ny, y-fastest (one periodic y line per x wavenumber) */
} poisson_cache;

static poisson_cache pcache;

static int poisson_prepare(const domain_t *dom) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  if (pcache.dct && pcache.nx == nx && pcache.ny == ny && pcache.lx == dom->lengths[0] && pcache.hy == dom->hy)
    return 0;
  sbfs_dct_plan_destroy(pcache.dct);
  free(pcache.eig);
  free(pcache.rhs);
  free(pcache.spec);
  memset(&pcache, 0, sizeof(pcache));
  pcache.nx = nx; pcache.ny = ny; pcache.lx = dom->lengths[0]; pcache.hy = dom->hy;
  pcache.dct = sbfs_dct_plan_create(nx);
  pcache.eig = malloc(sizeof(double) * nx);
  pcache.rhs = malloc(sizeof(double) * (size_t)nx * ny);
  pcache.spec = malloc(sizeof(double) * (size_t)nx * ny);
  if (!pcache.dct || !pcache.eig || !pcache.rhs || !pcache.spec) return 1;
  /* compute_potential.c:233-261 */
  const double pi = 3.14159265358979324;
  const double dx = dom->lengths[0] / nx;
  for (int k = 0; k < nx; k++)
    pcache.eig[k] = -4. / pow(dx, 2.) * pow(sin(pi * k / (2. * nx)), 2.);
  return 0;
}

int orc_fluid_compute_potential(const domain_t *dom, double dt_old, double dt_new, fluid_t *fl) {
  if (poisson_prepare(dom)) return 1;
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  const double rref = fl->refden;
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  fview psi = view_of(dom, &fl->psi[0], 1);
  fview den = view_of(dom, &fl->den[1], 1);
  double *rhs = pcache.rhs, *spec = pcache.spec;
  /* right-hand side, pre-scaled by 1/(2 nx) for the DCT pair (:285-363) */
  const double norm = 2. * nx;
  const double c_div = 1. / norm / dt_new * rref;
  const double c_add = 1. / norm * -1. / dt_new * dt_old;
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double hxm = HXXF(i), hxp = HXXF(i + 1);
      const double jdm = JDXF(i), jd0 = JDXC(i), jdp = JDXF(i + 1);
      const double div = 1. / jd0 * (-jdm / hxm * F(ux, i, j) + jdp / hxp * F(ux, i + 1, j)
                                     - jd0 / hy * F(uy, i, j) + jd0 / hy * F(uy, i, j + 1));
      const double rxm = +0.5 * F(den, i - 1, j) + 0.5 * F(den, i, j);
      const double rxp = +0.5 * F(den, i, j) + 0.5 * F(den, i + 1, j);
      const double rym = +0.5 * F(den, i, j - 1) + 0.5 * F(den, i, j);
      const double ryp = +0.5 * F(den, i, j) + 0.5 * F(den, i, j + 1);
      const double dxm = -F(psi, i - 1, j) + F(psi, i, j);
      const double dxp = -F(psi, i, j) + F(psi, i + 1, j);
      const double dym = -F(psi, i, j - 1) + F(psi, i, j);
      const double dyp = -F(psi, i, j) + F(psi, i, j + 1);
      const double gxm = (rref / rxm - 1.) * dxm / hxm;
      const double gxp = (rref / rxp - 1.) * dxp / hxp;
      const double gym = (rref / rym - 1.) * dym / hy;
      const double gyp = (rref / ryp - 1.) * dyp / hy;
      const double add = 1. / jd0 * (-jdm / hxm * gxm + jdp / hxp * gxp - jd0 / hy * gym + jd0 / hy * gyp);
      rhs[(size_t)(j - 1) * nx + (i - 1)] = (+c_div * div + c_add * add);
    }
  }
  /* DCT-II along x, then one periodic y system per x wavenumber (:382-410),
   * then DCT-III back; the row <-> column reorderings stand in for the
   * pencil transposes */
  OMP_FOR
  for (int j = 0; j < ny; j++) {
    double *work = malloc(sizeof(double) * 4 * (size_t)nx);
    double *line = rhs + (size_t)j * nx;
    sbfs_dct2(pcache.dct, line, line, work);
    free(work);
  }
  OMP_FOR
  for (int k = 0; k < nx; k++)
    for (int j = 0; j < ny; j++) spec[(size_t)k * ny + j] = rhs[(size_t)j * nx + k];
  const double l = 1. / hy / hy, u = 1. / hy / hy;
  OMP_FOR
  for (int k = 0; k < nx; k++) {
    double *c = malloc(sizeof(double) * 3 * (size_t)ny);
    double *v = c + ny, *q1 = c + 2 * ny;
    for (int n = 0; n < ny; n++) c[n] = -l - u + pcache.eig[k];
    thomas_periodic(ny, l, c, u, v, q1, spec + (size_t)k * ny);
    free(c);
  }
  OMP_FOR
  for (int j = 0; j < ny; j++)
    for (int k = 0; k < nx; k++) rhs[(size_t)j * nx + k] = spec[(size_t)k * ny + j];
  OMP_FOR
  for (int j = 0; j < ny; j++) {
    double *work = malloc(sizeof(double) * 4 * (size_t)nx);
    double *line = rhs + (size_t)j * nx;
    sbfs_dct3(pcache.dct, line, line, work);
    free(work);
  }
  /* psi[1] and its wall / periodic ghosts (:365-380) */
  fview out = view_of(dom, &fl->psi[1], 1);
  OMP_FOR
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) F(out, i, j) = rhs[(size_t)(j - 1) * nx + (i - 1)];
  return orc_fluid_update_boundaries_psi(dom, &fl->psi[1]);
}

/* src/fluid/correct_velocity/ux.c:18-66, uy.c:17-64 */
int orc_fluid_correct_velocity(const domain_t *dom, double dt_old, double dt_new, fluid_t *fl) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  const double rref = fl->refden;
  const double coef = -1. / dt_new * dt_old;
  fview p1 = view_of(dom, &fl->psi[1], 1);
  fview p0 = view_of(dom, &fl->psi[0], 1);
  fview den = view_of(dom, &fl->den[1], 1);
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 2; i <= nx; i++) {
      const double hx = HXXF(i);
      double v = F(ux, i, j);
      v -= dt_new / rref / hx * (-F(p1, i - 1, j) + F(p1, i, j));
      const double r = +0.5 * F(den, i - 1, j) + 0.5 * F(den, i, j);
      v += dt_new * coef * (1. / r - 1. / rref) / hx * (-F(p0, i - 1, j) + F(p0, i, j));
      F(ux, i, j) = v;
    }
  }
  if (orc_fluid_update_boundaries_ux(dom, &fl->ux)) return 1;
  OMP_FOR
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      double v = F(uy, i, j);
      v -= dt_new / rref / hy * (-F(p1, i, j - 1) + F(p1, i, j));
      const double r = +0.5 * F(den, i, j - 1) + 0.5 * F(den, i, j);
      v += dt_new * coef * (1. / r - 1. / rref) / hy * (-F(p0, i, j - 1) + F(p0, i, j));
      F(uy, i, j) = v;
    }
  }
  return orc_fluid_update_boundaries_uy(dom, &fl->uy);
}

/* src/fluid/update_pressure.c:7-53: p += psi_new, Neumann walls, swap psi */
int orc_fluid_update_pressure(const domain_t *dom, fluid_t *fl) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  fview p = view_of(dom, &fl->p, 1);
  fview ps = view_of(dom, &fl->psi[1], 1);
  OMP_FOR
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) F(p, i, j) += F(ps, i, j);
  if (orc_fluid_update_boundaries_p(dom, &fl->p)) return 1;
  swap_data(&fl->psi[0], &fl->psi[1]);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* time step size and the RK3 driver                                        */
/* ------------------------------------------------------------------------ */

void orc_set_dt_coefs(double adv, double dif, double itf) {
  dt_coef_adv = adv;
  dt_coef_dif = dif;
  dt_coef_int = itf;
}

static int load_dt_coefs(void) {
  if (dt_coef_adv >= 0. && dt_coef_dif >= 0. && dt_coef_int >= 0.) return 0;
  const char *keys[3] = {"coef_dt_adv", "coef_dt_dif", "coef_dt_int"};
  double vals[3];
  for (int k = 0; k < 3; k++) {
    const char *s = getenv(keys[k]);
    if (!s) return 1;
    vals[k] = strtod(s, NULL);
  }
  orc_set_dt_coefs(vals[0], vals[1], vals[2]);
  return 0;
}

/* src/decide_dt.c:34-169 */
int orc_decide_dt(const domain_t *dom, const fluid_t *fl, const interface_t *itf, double *dt) {
  if (load_dt_coefs()) return 1;
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  const double small = 1.e-8;
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  double adv = 1.;
#pragma omp parallel for reduction(min : adv) num_threads(orc_get_threads())
  for (int j = 1; j <= ny; j++) {
    for (int i = 2; i <= nx; i++) adv = fmin(adv, HXXF(i) / (fabs(F(ux, i, j)) + small));
    for (int i = 1; i <= nx; i++) adv = fmin(adv, hy / (fabs(F(uy, i, j)) + small));
  }
  adv *= dt_coef_adv;
  double hxmin = DBL_MAX;
  for (int i = 2; i <= nx; i++) hxmin = fmin(hxmin, HXXF(i));
  const double h[2] = {hxmin, hy};
  const double diffusivity = 1. / fl->Re;
  const double tension = 1. / itf->We;
  const double pi = 3.1415926535897932384626433832;
  double out = adv;
  for (int d = 0; d < 2; d++) {
    double dif = fmin(1., fl->denr / fl->visr) / diffusivity * 0.5 / 2 * pow(h[d], 2.);
    dif *= dt_coef_dif;
    out = fmin(out, dif);
  }
  double cap = 1.;
  for (int d = 0; d < 2; d++) cap = fmin(cap, sqrt(1. / tension / 4. / pi * pow(h[d], 3.)));
  cap *= dt_coef_int;
  out = fmin(out, cap);
  *dt = out;
  return 0;
}

/* src/integrate.c:11-70 */
int orc_integrate(const domain_t *dom, fluid_t *fl, interface_t *itf, double *dt) {
  if (orc_decide_dt(dom, fl, itf, dt)) return 1;
  for (int k = 0; k < 3; k++) {
    if (orc_fluid_compute_density(dom, fl, itf, 0)) return 1;
    if (orc_fluid_compute_viscosity(dom, fl, itf)) return 1;
    if (orc_interface_compute_curvature_tensor(dom, itf)) return 1;
    if (orc_interface_compute_force(dom, fl, itf)) return 1;
    if (orc_interface_update_vof(dom, (size_t)k, *dt, fl, itf)) return 1;
    if (orc_fluid_compute_density(dom, fl, itf, 1)) return 1;
    if (orc_interface_compute_mass_flux(dom, fl, itf)) return 1;
    if (orc_fluid_predict_field(dom, (size_t)k, *dt, fl, itf)) return 1;
    const double dt_old = rk_gamma((k + 2) % 3) * (*dt);
    const double dt_new = rk_gamma(k) * (*dt);
    if (orc_fluid_compute_potential(dom, dt_old, dt_new, fl)) return 1;
    if (orc_fluid_correct_velocity(dom, dt_old, dt_new, fl)) return 1;
    if (orc_fluid_update_pressure(dom, fl)) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* diagnostics                                                              */
/* ------------------------------------------------------------------------ */

int orc_max_divergence(const domain_t *dom, const fluid_t *fl, double *divmax) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  double m = 0.;
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double hxm = HXXF(i), hxp = HXXF(i + 1);
      const double jdm = JDXF(i), jd0 = JDXC(i), jdp = JDXF(i + 1);
      const double div = 1. / jd0 * (-jdm / hxm * F(ux, i, j) + jdp / hxp * F(ux, i + 1, j)
                                     - jd0 / hy * F(uy, i, j) + jd0 / hy * F(uy, i, j + 1));
      m = fmax(m, fabs(div));
    }
  }
  *divmax = m;
  return 0;
}

int orc_vof_stats(const domain_t *dom, const interface_t *itf, double out[4]) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  fview vof = view_of(dom, &itf->vof, 1);
  double lo = 1., hi = 0., s0 = 0., s1 = 0.;
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double ds = JDXC(i);
      const double v = F(vof, i, j);
      lo = fmin(lo, v);
      hi = fmax(hi, v);
      s0 += v * ds;
      s1 += ds;
    }
  }
  out[0] = lo; out[1] = hi; out[2] = s0; out[3] = s1;
  return 0;
}

/* all logging quantities of src/logging/{divergence,interface,momentum,energy,extrema,stress}.c
 * in the order of sbfs_diagnostics:
 * divmax, vof min, max, sum vof J, sum J, interface area, momentum x, y,
 * energy x, y, max |ux|, max |uy|, wall stress at x = 0, lx */
int orc_diagnostics(const domain_t *dom, const fluid_t *fl, const interface_t *itf, double out[16]) {
  const int nx = (int)dom->mysizes[0], ny = (int)dom->mysizes[1];
  const double hy = dom->hy;
  double st[4];
  for (int k = 0; k < 16; k++) out[k] = 0.;
  orc_max_divergence(dom, fl, &out[0]);
  orc_vof_stats(dom, itf, st);
  out[1] = st[0]; out[2] = st[1]; out[3] = st[2]; out[4] = st[3];
  fview vof = view_of(dom, &itf->vof, 1);
  fview den = view_of(dom, &fl->den[1], 1);
  fview ux = view_of(dom, &fl->ux, 1);
  fview uy = view_of(dom, &fl->uy, 1);
  fview txy = view_of(dom, &fl->txy, 1);
  /* interface area (src/logging/interface.c:47-62) */
  double area = 0.;
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx + 1; i++) area += fabs(F(vof, i, j) - F(vof, i - 1, j)) * (JDXF(i) / HXXF(i));
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) area += fabs(F(vof, i, j) - F(vof, i, j - 1)) * (JDXC(i) / hy);
  out[5] = area;
  /* momentum, energy, extrema (momentum.c:40-56, energy.c:42-58, extrema.c:25-38) */
  double mx = 0., my = 0., ex = 0., ey = 0., umax = 0., vmax = 0.;
  for (int j = 1; j <= ny; j++) {
    for (int i = 2; i <= nx; i++) {
      const double ds = JDXF(i);
      const double r = 0.5 * F(den, i - 1, j) + 0.5 * F(den, i, j);
      const double u = F(ux, i, j);
      mx += r * u * ds;
      ex += 0.5 * r * pow(u, 2.) * ds;
      umax = fmax(umax, fabs(u));
    }
  }
  for (int j = 1; j <= ny; j++) {
    for (int i = 1; i <= nx; i++) {
      const double ds = JDXC(i);
      const double r = 0.5 * F(den, i, j - 1) + 0.5 * F(den, i, j);
      const double v = F(uy, i, j);
      my += r * v * ds;
      ey += 0.5 * r * pow(v, 2.) * ds;
      vmax = fmax(vmax, fabs(v));
    }
  }
  out[6] = mx; out[7] = my; out[8] = ex; out[9] = ey; out[10] = umax; out[11] = vmax;
  /* wall shear stress (stress.c:29-35) */
  const double nu = 1. / fl->Re;
  for (int j = 1; j <= ny; j++) {
    out[12] += nu * JDXF(1) / HXXF(1) * F(txy, 1, j);
    out[13] += nu * JDXF(nx + 1) / HXXF(nx + 1) * F(txy, nx + 1, j);
  }
  return 0;
}
