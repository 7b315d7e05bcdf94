// sm_103a kernels of the 2-D two-phase (VOF) time step.
//
// All arithmetic is FP64.  On GB300 the FP64 pipe (about 0.5 T fused
// multiply-adds per second, measured) is the bound of this solver, not HBM,
// so the kernels are written to minimise FP64 instructions:
//   * every per-column metric factor of the reference's stencils (1/HXXF,
//     JDXF/HXXF, 0.5 JDXF/HXXF, ...) is precomputed once with the reference's
//     own expression (struct Metrics);
//   * each reciprocal the reference forms with "1. / x" uses the correctly
//     rounded reciprocal __drcp_rn (same value, cheaper than a division);
//   * divisions by a face density are replaced by one reciprocal per face per
//     substage, shared by the predictor, the Poisson right-hand side and the
//     velocity correction (irhox / irhoy);
//   * threshold tests (vofmin, upwind sign, clipping of the mixture rules)
//     run on the integer pattern of the double;
//   * cells where all inputs of a stencil are bitwise equal (single-phase
//     bulk) take the exact short cut (zero gradient, zero force).
// Index conventions follow sbfs_device.cuh; the reference file:line each
// kernel follows is cited at the kernel.
#include <cfloat>

#include "sbfs_kernels.cuh"

namespace sbfs {

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ size_t ix(const Grid &g, int row, int col) { return (size_t)row * g.p1 + col; }
__device__ __forceinline__ double half_sum(double a, double b) { return 0.5 * (a + b); }
__device__ __forceinline__ bool same(double a, double b) { return dbits(a) == dbits(b); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

dim3 grid2d(int ni, int nj) { return dim3((ni + BX - 1) / BX, (nj + BY - 1) / BY); }

// ---------------------------------------------------------------------------
// density, viscosity, corner gradients of vof
//   den:   src/fluid/density.c:9-31
//   visux: src/fluid/viscosity.c:23-61, visuy: :63-91
//   dvof:  src/interface/curvature_tensor.c:16-49
// thread (I, J): I = 0..nx+1
// ---------------------------------------------------------------------------
template <bool DEN, bool VIS, bool GRAD>
__global__ void __launch_bounds__(BX *BY) k_props(Grid g, Metrics m, Phys ph, const double *__restrict__ vof,
                                                  double *__restrict__ den, double *__restrict__ visux,
                                                  double *__restrict__ visuy, double *__restrict__ dvof) {
  const int I = blockIdx.x * BX + threadIdx.x;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int r = J - 1, rm = wrap(J - 1, g.ny);
  const double v = vof[ix(g, r, I)];
  if (DEN) den[ix(g, r, I)] = clip_pos(fma(ph.denr - 1., v, 1.), ph.den_lo, ph.den_hi);
  if (VIS) {
    const double c = ph.visr - 1.;
    if (I >= 1) {
      double phi;
      if (I == 1) phi = vof[ix(g, r, 0)];
      else if (I == g.nx + 1) phi = v;
      else phi = half_sum(vof[ix(g, r, I - 1)], v);
      visux[ix(g, r, I - 1)] = clip_pos(fma(c, phi, 1.), ph.vis_lo, ph.vis_hi);
    }
    const double phy = half_sum(vof[ix(g, rm, I)], v);
    visuy[ix(g, r, I)] = clip_pos(fma(c, phy, 1.), ph.vis_lo, ph.vis_hi);
  }
  if (GRAD && I >= 1) {
    // corner at x face I between rows J-1 and J
    const double a = vof[ix(g, rm, I - 1)], b = vof[ix(g, rm, I)];
    const double c = vof[ix(g, r, I - 1)], d = v;
    double2 out = make_double2(0., 0.);
    if (!(same(a, b) && same(b, c) && same(c, d))) {
      const double gx = m.ihxxf[I] * (((-a + b) - c) + d);
      const double gy = g.ihy * (((-a - b) + c) + d);
      const double nrm = sqrt(fma(gx, gx, gy * gy));
      const double inv = __drcp_rn(lt_pos(nrm, DBL_EPSILON) ? DBL_EPSILON : nrm);
      out = make_double2(gx * inv, gy * inv);
    }
    reinterpret_cast<double2 *>(dvof)[(size_t)r * (g.p2 / 2) + (I - 1)] = out;
  }
}

// ---------------------------------------------------------------------------
// cell normal + THINC intercept (interface cells) and curvature
//   normal:    src/interface/curvature_tensor.c:51-97
//   curvature: src/interface/curvature_tensor.c:100-135
// thread (I, J): I = 1..nx
// ---------------------------------------------------------------------------
template <bool NORMAL, bool CURV>
__global__ void __launch_bounds__(BX *BY) k_normal_curv(Grid g, Metrics m, const double *__restrict__ vof,
                                                        const double *__restrict__ dvof, double *__restrict__ normal,
                                                        double *__restrict__ curv) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int r = J - 1, rp = wrap(J + 1, g.ny);
  const double2 *dv = reinterpret_cast<const double2 *>(dvof);
  const size_t q = g.p2 / 2;
  const double2 d00 = dv[(size_t)r * q + (I - 1)], d10 = dv[(size_t)r * q + I];
  const double2 d01 = dv[(size_t)rp * q + (I - 1)], d11 = dv[(size_t)rp * q + I];
  if (CURV) {
    const long long any = dbits(d00.x) | dbits(d00.y) | dbits(d10.x) | dbits(d10.y) | dbits(d01.x) | dbits(d01.y) |
                          dbits(d11.x) | dbits(d11.y);
    double k = -0.;
    if ((any << 1) != 0) {  // some corner normal is not +-0
      const double nxm = half_sum(d00.x, d01.x), nxp = half_sum(d10.x, d11.x);
      const double nym = half_sum(d00.y, d10.y), nyp = half_sum(d01.y, d11.y);
      const double div = m.ijdxc[I] * (((-m.qf[I] * nxm + m.qf[I + 1] * nxp) - m.qc_hy[I] * nym) + m.qc_hy[I] * nyp);
      k = -div;
    }
    curv[ix(g, r, I)] = k;
  }
  if (NORMAL) {
    const double phi = vof[ix(g, r, I)];
    if (!single_phase(phi)) {
      double mx = ((d00.x + d10.x) + d01.x) + d11.x;
      double my = ((d00.y + d10.y) + d01.y) + d11.y;
      mx *= m.ihxxc[I];
      my *= g.ihy;
      const double nrm = sqrt(fma(mx, mx, my * my));
      const double inv = __drcp_rn(lt_pos(nrm, DBL_EPSILON) ? DBL_EPSILON : nrm);
      double *o = normal + (size_t)r * g.p3 + (size_t)(I - 1) * 3;
      o[0] = mx * inv;
      o[1] = my * inv;
      o[2] = -0.5 * log(__drcp_rn(phi) - 1.);
    }
  }
}

// smoothed-indicator face average of a THINC cell: sum over the two Gauss
// points of 0.5 * (1 + tanh(n . x + d)) with weight 0.5 each
// (src/interface/update/main.c:18-35, fluxx.c:62-68)
__device__ __forceinline__ double thinc_face(const double *n, double x0, double y0, double x1, double y1) {
  const double i0 = 0.5 * (1. + tanh(fma(n[1], y0, n[0] * x0) + n[2]));
  const double i1 = 0.5 * (1. + tanh(fma(n[1], y1, n[0] * x1) + n[2]));
  return fma(0.5, i1, 0.5 * i0);
}

// ---------------------------------------------------------------------------
// THINC vof fluxes and CSF surface-tension force
//   fluxes: src/interface/update/fluxx.c:14-73, fluxy.c:14-73
//   force:  src/interface/force.c:20-88
// thread (I, J): I = 1..nx handles x face I (I >= 2) and y face (I, J - 1/2)
// ---------------------------------------------------------------------------
template <bool FLUX, bool FORCE>
__global__ void __launch_bounds__(BX *BY)
    k_flux_force(Grid g, Metrics m, Phys ph, const double *__restrict__ ux, const double *__restrict__ uy,
                 const double *__restrict__ vof, const double *__restrict__ normal, const double *__restrict__ den0,
                 const double *__restrict__ curv, double *__restrict__ fluxx, double *__restrict__ fluxy,
                 double *__restrict__ ifrcx, double *__restrict__ ifrcy) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int r = J - 1, rm = wrap(J - 1, g.ny);
  const double v0 = vof[ix(g, r, I)];
  const double vxm = vof[ix(g, r, I - 1)];
  const double vym = vof[ix(g, rm, I)];
  if (FLUX) {
    if (I >= 2) {
      const double vel = ux[ix(g, r, I - 1)];
      const bool n = neg(vel);
      const int iu = n ? I : I - 1;
      const double phi = n ? v0 : vxm;
      double f;
      if (single_phase(phi)) {
        f = vel * phi;
      } else {
        const double xq = n ? -0.5 : 0.5;
        const double *nv = normal + (size_t)r * g.p3 + (size_t)(iu - 1) * 3;
        f = vel * thinc_face(nv, xq, -kGaussPt, xq, kGaussPt);
      }
      fluxx[ix(g, r, I - 1)] = f;
    }
    {
      const double vel = uy[ix(g, r, I)];
      const bool n = neg(vel);
      const int ru = n ? r : rm;
      const double phi = n ? v0 : vym;
      double f;
      if (single_phase(phi)) {
        f = vel * phi;
      } else {
        const double yq = n ? -0.5 : 0.5;
        const double *nv = normal + (size_t)ru * g.p3 + (size_t)(I - 1) * 3;
        f = vel * thinc_face(nv, -kGaussPt, yq, kGaussPt, yq);
      }
      fluxy[ix(g, r, I)] = f;
    }
    // impermeable walls / dummy ghost faces
    if (I == 1) {
      fluxx[ix(g, r, 0)] = 0.;
      fluxy[ix(g, r, 0)] = 0.;
    }
    if (I == g.nx) {
      fluxx[ix(g, r, g.nx)] = 0.;
      fluxy[ix(g, r, g.nx + 1)] = 0.;
    }
  }
  if (FORCE) {
    if (I >= 2) {
      double f = 0.;
      if (!same(vxm, v0)) {
        const double rho = half_sum(den0[ix(g, r, I - 1)], den0[ix(g, r, I)]);
        const double kap = half_sum(curv[ix(g, r, I - 1)], curv[ix(g, r, I)]);
        const double dl = m.ihxxf[I] * (v0 - vxm);
        f = ((rho * ph.force_coef) * kap) * dl;
      }
      ifrcx[ix(g, r, I - 2)] = f;
    }
    double f = 0.;
    if (!same(vym, v0)) {
      const double rho = half_sum(den0[ix(g, rm, I)], den0[ix(g, r, I)]);
      const double kap = half_sum(curv[ix(g, rm, I)], curv[ix(g, r, I)]);
      const double dl = g.ihy * (v0 - vym);
      f = ((rho * ph.force_coef) * kap) * dl;
    }
    ifrcy[ix(g, r, I - 1)] = f;
  }
}

// ---------------------------------------------------------------------------
// vof source (flux divergence), RK update and vof boundaries
//   src/interface/update/main.c:54-136, src/interface/boundary.c:15-42
// FUSED additionally writes rho^{k+1} (src/fluid/density.c) and the mass
// fluxes u + (rho_r - 1) flux into separate buffers
// (src/interface/mass_flux.c:10-58).
// thread (I, J): I = 1..nx
// ---------------------------------------------------------------------------
template <bool FUSED>
__global__ void __launch_bounds__(BX *BY)
    k_vof_advance(Grid g, Metrics m, Phys ph, const double *__restrict__ sc, int k, double *__restrict__ vof,
                  const double *__restrict__ fluxx, const double *__restrict__ fluxy, double *__restrict__ src_a,
                  const double *__restrict__ src_b, const double *__restrict__ ux, const double *__restrict__ uy,
                  double *__restrict__ mfx, double *__restrict__ mfy, double *__restrict__ den1) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int r = J - 1, rp = wrap(J + 1, g.ny);
  const double fxm = fluxx[ix(g, r, I - 1)], fxp = fluxx[ix(g, r, I)];
  const double fym = fluxy[ix(g, r, I)], fyp = fluxy[ix(g, rp, I)];
  const double s = m.ijdxc[I] * (((m.qf[I] * fxm - m.qf[I + 1] * fxp) + m.qc_hy[I] * fym) - m.qc_hy[I] * fyp);
  src_a[ix(g, r, I - 1)] = s;
  double v = vof[ix(g, r, I)];
  v = fma(sc[sc_adt(k)], s, v);
  if (k != 0) v = fma(sc[sc_bdt(k)], src_b[ix(g, r, I - 1)], v);
  vof[ix(g, r, I)] = v;
  if (I == 1) vof[ix(g, r, 0)] = 0.;
  if (I == g.nx) vof[ix(g, r, g.nx + 1)] = 0.;
  if (FUSED) {
    const double c = ph.denr - 1.;
    den1[ix(g, r, I)] = clip_pos(fma(c, v, 1.), ph.den_lo, ph.den_hi);
    mfx[ix(g, r, I - 1)] = fma(c, fxm, ux[ix(g, r, I - 1)]);
    mfy[ix(g, r, I)] = fma(c, fym, uy[ix(g, r, I)]);
    if (I == 1) {
      den1[ix(g, r, 0)] = clip_pos(1., ph.den_lo, ph.den_hi);
      mfy[ix(g, r, 0)] = fma(c, fluxy[ix(g, r, 0)], uy[ix(g, r, 0)]);
    }
    if (I == g.nx) {
      den1[ix(g, r, g.nx + 1)] = clip_pos(1., ph.den_lo, ph.den_hi);
      mfx[ix(g, r, g.nx)] = fma(c, fxp, ux[ix(g, r, g.nx)]);
      mfy[ix(g, r, g.nx + 1)] = fma(c, fluxy[ix(g, r, g.nx + 1)], uy[ix(g, r, g.nx + 1)]);
    }
  }
}

// vof flux -> mass flux in place (src/interface/mass_flux.c:10-58); I = 0..nx+1
__global__ void k_mass_flux(Grid g, Phys ph, const double *__restrict__ ux, const double *__restrict__ uy,
                            double *__restrict__ fluxx, double *__restrict__ fluxy) {
  const int I = blockIdx.x * BX + threadIdx.x;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int r = J - 1;
  const double c = ph.denr - 1.;
  if (I >= 1) fluxx[ix(g, r, I - 1)] = fma(c, fluxx[ix(g, r, I - 1)], ux[ix(g, r, I - 1)]);
  fluxy[ix(g, r, I)] = fma(c, fluxy[ix(g, r, I)], uy[ix(g, r, I)]);
}

// ---------------------------------------------------------------------------
// viscous stress tensor: txx, tyy at centres, txy at corners
//   src/fluid/predict/txx.c:11-40, txy.c:13-50, tyy.c:10-38
// thread (I, J): I = 1..nx+1
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BX *BY)
    k_stress(Grid g, Metrics m, const double *__restrict__ ux, const double *__restrict__ uy,
             const double *__restrict__ visux, const double *__restrict__ visuy, double *__restrict__ txx,
             double *__restrict__ txy, double *__restrict__ tyy) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int r = J - 1, rm = wrap(J - 1, g.ny), rp = wrap(J + 1, g.ny);
  const double u0 = ux[ix(g, r, I - 1)];
  const double vx0 = visux[ix(g, r, I - 1)];
  const double w0 = uy[ix(g, r, I)];
  const double vy0 = visuy[ix(g, r, I)];
  if (I <= g.nx) {
    const double mu = half_sum(vx0, visux[ix(g, r, I)]);
    const double l = m.ihxxc[I] * (ux[ix(g, r, I)] - u0);
    const double t = __dmul_rn(mu, l);
    txx[ix(g, r, I - 1)] = __dadd_rn(t, t);
    const double muy = half_sum(vy0, visuy[ix(g, rp, I)]);
    const double ly = g.ihy * (uy[ix(g, rp, I)] - w0);
    const double ty = __dmul_rn(muy, ly);
    tyy[ix(g, r, I - 1)] = __dadd_rn(ty, ty);
  }
  const double mux = half_sum(visux[ix(g, rm, I - 1)], vx0);
  const double muy = half_sum(visuy[ix(g, r, I - 1)], vy0);
  const double lxy = g.ihy * (u0 - ux[ix(g, rm, I - 1)]);
  const double lyx = m.ihxxf[I] * (w0 - uy[ix(g, r, I - 1)]);
  txy[ix(g, r, I - 1)] = fma(mux, lxy, muy * lyx);
}

// ---------------------------------------------------------------------------
// momentum right-hand sides and the RK predictor
//   ux: src/fluid/predict/ux.c:29-273, uy: src/fluid/predict/uy.c:29-251,
//   src/fluid/predict/main.c:9-80, walls: src/fluid/boundary/ux.c, uy.c
// thread (I, J): I = 1..nx handles the ux face I (I >= 2) and the uy face
// (I, J - 1/2); also stores 1 / rho^{k+1} at both faces
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BX *BY)
    k_predict(Grid g, Metrics m, Phys ph, const double *__restrict__ sc, int k, const double *__restrict__ ux,
              const double *__restrict__ uy, double *__restrict__ ux_out, double *__restrict__ uy_out,
              const double *__restrict__ mfx, const double *__restrict__ mfy, const double *__restrict__ txx,
              const double *__restrict__ txy, const double *__restrict__ tyy, const double *__restrict__ p,
              const double *__restrict__ ifrcx, const double *__restrict__ ifrcy, const double *__restrict__ den0,
              const double *__restrict__ den1, double *__restrict__ sxa, const double *__restrict__ sxb,
              double *__restrict__ sxg, double *__restrict__ sya, const double *__restrict__ syb,
              double *__restrict__ syg, double *__restrict__ irhox, double *__restrict__ irhoy) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int r = J - 1, rm = wrap(J - 1, g.ny), rp = wrap(J + 1, g.ny);
  const double adt = sc[sc_adt(k)], bdt = sc[sc_bdt(k)], gdt = sc[sc_gdt(k)];
  // ---- ux at face I
  if (I >= 2) {
    const double fxm = mfx[ix(g, r, I - 2)], fx0 = mfx[ix(g, r, I - 1)], fxp = mfx[ix(g, r, I)];
    const double um1 = ux[ix(g, r, I - 2)], u0 = ux[ix(g, r, I - 1)], up1 = ux[ix(g, r, I)];
    double a;
    {
      const double mm = fma(m.hqf[I - 1], fxm, m.hqf[I] * fx0);
      const double mp = fma(m.hqf[I], fx0, m.hqf[I + 1] * fxp);
      const double um = half_sum(um1, u0), up = half_sum(u0, up1);
      a = -(m.ijdxf[I] * fma(mp, up, -mm * um));
    }
    {
      const double mm = fma(m.hqc_hy[I - 1], mfy[ix(g, r, I - 1)], m.hqc_hy[I] * mfy[ix(g, r, I)]);
      const double mp = fma(m.hqc_hy[I - 1], mfy[ix(g, rp, I - 1)], m.hqc_hy[I] * mfy[ix(g, rp, I)]);
      const double um = half_sum(ux[ix(g, rm, I - 1)], u0), up = half_sum(u0, ux[ix(g, rp, I - 1)]);
      a -= m.ijdxf[I] * fma(mp, up, -mm * um);
    }
    a = fma(m.nu_ijdxf[I], fma(m.qc[I], txx[ix(g, r, I - 1)], -m.qc[I - 1] * txx[ix(g, r, I - 2)]), a);
    a = fma(m.nu_ijdxf[I], m.qf_hy[I] * (txy[ix(g, rp, I - 1)] - txy[ix(g, r, I - 1)]), a);
    const double gs = -(m.ihxxf[I] * (p[ix(g, r, I)] - p[ix(g, r, I - 1)]));
    a += ifrcx[ix(g, r, I - 2)];
    const double rho0 = half_sum(den0[ix(g, r, I - 1)], den0[ix(g, r, I)]);
    a = fma(ph.grav, rho0, a);
    const double irho = __drcp_rn(half_sum(den1[ix(g, r, I - 1)], den1[ix(g, r, I)]));
    double u = fma(adt, a, rho0 * u0);
    if (k != 0) u = fma(bdt, sxb[ix(g, r, I - 2)], u);
    u = fma(gdt, gs, u);
    ux_out[ix(g, r, I - 1)] = u * irho;
    sxa[ix(g, r, I - 2)] = a;
    if (sxg) sxg[ix(g, r, I - 2)] = gs;
    irhox[ix(g, r, I - 1)] = irho;
  }
  // ---- uy at face (I, J - 1/2)
  {
    const double w0 = uy[ix(g, r, I)];
    double a;
    {
      const double mm = m.hqf[I] * (mfx[ix(g, rm, I - 1)] + mfx[ix(g, r, I - 1)]);
      const double mp = m.hqf[I + 1] * (mfx[ix(g, rm, I)] + mfx[ix(g, r, I)]);
      const double um = half_sum(uy[ix(g, r, I - 1)], w0), up = half_sum(w0, uy[ix(g, r, I + 1)]);
      a = -(m.ijdxc[I] * fma(mp, up, -mm * um));
    }
    {
      const double f0 = mfy[ix(g, r, I)];
      const double mm = m.hqc_hy[I] * (mfy[ix(g, rm, I)] + f0);
      const double mp = m.hqc_hy[I] * (f0 + mfy[ix(g, rp, I)]);
      const double um = half_sum(uy[ix(g, rm, I)], w0), up = half_sum(w0, uy[ix(g, rp, I)]);
      a -= m.ijdxc[I] * fma(mp, up, -mm * um);
    }
    a = fma(m.nu_ijdxc[I], fma(m.qf[I + 1], txy[ix(g, r, I)], -m.qf[I] * txy[ix(g, r, I - 1)]), a);
    a = fma(m.nu_ijdxc[I], m.qc_hy[I] * (tyy[ix(g, r, I - 1)] - tyy[ix(g, rm, I - 1)]), a);
    const double gs = -(g.ihy * (p[ix(g, r, I)] - p[ix(g, rm, I)]));
    a += ifrcy[ix(g, r, I - 1)];
    const double rho0 = half_sum(den0[ix(g, rm, I)], den0[ix(g, r, I)]);
    const double irho = __drcp_rn(half_sum(den1[ix(g, rm, I)], den1[ix(g, r, I)]));
    double u = fma(adt, a, rho0 * w0);
    if (k != 0) u = fma(bdt, syb[ix(g, r, I - 1)], u);
    u = fma(gdt, gs, u);
    uy_out[ix(g, r, I)] = u * irho;
    sya[ix(g, r, I - 1)] = a;
    if (syg) syg[ix(g, r, I - 1)] = gs;
    irhoy[ix(g, r, I)] = irho;
  }
  // walls: impermeable, no-slip; wall-face densities for the Poisson operator
  if (I == 1) {
    ux_out[ix(g, r, 0)] = 0.;
    uy_out[ix(g, r, 0)] = 0.;
    irhox[ix(g, r, 0)] = __drcp_rn(half_sum(den1[ix(g, r, 0)], den1[ix(g, r, 1)]));
  }
  if (I == g.nx) {
    ux_out[ix(g, r, g.nx)] = 0.;
    uy_out[ix(g, r, g.nx + 1)] = 0.;
    irhox[ix(g, r, g.nx)] = __drcp_rn(half_sum(den1[ix(g, r, g.nx)], den1[ix(g, r, g.nx + 1)]));
  }
}

// ---------------------------------------------------------------------------
// Poisson solve for the scalar potential (src/fluid/compute_potential.c)
//
// The reference diagonalises the constant-coefficient operator with a DCT
// along x and solves one periodic tridiagonal system along y per x
// wavenumber.  Here the same discrete operator is diagonalised by a real DFT
// along the periodic y direction and one (non-periodic, Neumann-ended)
// tridiagonal system along x is solved per y wavenumber.
//   1. k_poisson_fwd: right-hand side of src/fluid/compute_potential.c:
//      285-363 for a tile of W columns, packed two reals per complex, a
//      radix-2 Stockham FFT of length ny/2 in shared memory and the
//      real-to-complex split; spectrum [I][m], m = 0..ny/2
//   2. k_poisson_tdm: Thomas sweeps along x with precomputed pivots; the
//      singular m = 0 mode is pinned to zero mean
//   3. k_poisson_inv: inverse of step 1, psi and its Neumann ghosts
// ---------------------------------------------------------------------------

// radix-2 Stockham FFT of W rows of length M in shared memory; tw[e] =
// exp(-2 pi i e / (2M)), so W_M^e = tw[2e].  Returns the buffer holding the
// result (x or y).
template <int W>
__device__ double2 *fft_rows(double2 *x, double2 *y, int M, const double2 *__restrict__ tw, bool inverse) {
  const int half = M >> 1;
  for (int Ns = 1; Ns < M; Ns <<= 1) {
    for (int t = threadIdx.x; t < W * half; t += blockDim.x) {
      const int c = t / half, j = t - c * half;
      const double2 *xr = x + c * M;
      double2 *yr = y + c * M;
      const int kk = j & (Ns - 1);
      const double2 v0 = xr[j];
      double2 v1 = xr[j + half];
      if (Ns > 1) {
        double2 w = tw[kk * (M / Ns)];
        if (inverse) w.y = -w.y;
        v1 = cmul(v1, w);
      }
      const int d = ((j - kk) << 1) + kk;
      yr[d] = cadd(v0, v1);
      yr[d + Ns] = csub(v0, v1);
    }
    __syncthreads();
    double2 *tmp = x;
    x = y;
    y = tmp;
  }
  return x;
}

template <int W>
__global__ void __launch_bounds__(256)
    k_poisson_fwd(Grid g, Metrics m, Phys ph, const double *__restrict__ sc, int k, const double *__restrict__ ux,
                  const double *__restrict__ uy, const double *__restrict__ psi, const double *__restrict__ irhox,
                  const double *__restrict__ irhoy, const double2 *__restrict__ tw, double2 *__restrict__ spec) {
  extern __shared__ double2 smem[];
  const int ny = g.ny, M = ny >> 1;
  double2 *A = smem, *B = smem + W * M;
  double *Ad = reinterpret_cast<double *>(A);
  const int I0 = blockIdx.x * W + 1;
  const double pdiv = sc[sc_pdiv(k)], padd = sc[sc_padd(k)];
  const double rref = ph.refden;
  for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
    const int c = t % W, r = t / W;
    const int I = I0 + c;
    double val = 0.;
    if (I <= g.nx) {
      const int rm = r == 0 ? ny - 1 : r - 1, rp = r == ny - 1 ? 0 : r + 1;
      const double div = m.ijdxc[I] * (((-m.qf[I] * ux[ix(g, r, I - 1)] + m.qf[I + 1] * ux[ix(g, r, I)]) -
                                        m.qc_hy[I] * uy[ix(g, r, I)]) +
                                       m.qc_hy[I] * uy[ix(g, rp, I)]);
      const double ps = psi[ix(g, r, I)];
      const double gxm = fma(rref, irhox[ix(g, r, I - 1)], -1.) * (ps - psi[ix(g, r, I - 1)]) * m.ihxxf[I];
      const double gxp = fma(rref, irhox[ix(g, r, I)], -1.) * (psi[ix(g, r, I + 1)] - ps) * m.ihxxf[I + 1];
      const double gym = fma(rref, irhoy[ix(g, r, I)], -1.) * (ps - psi[ix(g, rm, I)]) * g.ihy;
      const double gyp = fma(rref, irhoy[ix(g, rp, I)], -1.) * (psi[ix(g, rp, I)] - ps) * g.ihy;
      const double add = m.ijdxc[I] * (((-m.qf[I] * gxm + m.qf[I + 1] * gxp) - m.qc_hy[I] * gym) + m.qc_hy[I] * gyp);
      val = fma(pdiv, div, padd * add);
    }
    Ad[c * ny + r] = val;
  }
  __syncthreads();
  double2 *Z = fft_rows<W>(A, B, M, tw, false);
  // real-to-complex split: X_m = E_m + exp(-2 pi i m / ny) O_m
  const int M1 = M + 1;
  for (int t = threadIdx.x; t < W * M1; t += blockDim.x) {
    const int c = t / M1, mm = t - c * M1;
    const int I = I0 + c;
    if (I > g.nx) continue;
    const double2 zm = Z[c * M + (mm == M ? 0 : mm)];
    const double2 zr = Z[c * M + (mm == 0 ? 0 : M - mm)];
    const double2 zc = make_double2(zr.x, -zr.y);
    const double2 E = make_double2(0.5 * (zm.x + zc.x), 0.5 * (zm.y + zc.y));
    const double2 dd = csub(zm, zc);
    const double2 O = make_double2(0.5 * dd.y, -0.5 * dd.x);
    spec[(size_t)(I - 1) * M1 + mm] = cadd(E, cmul(tw[mm], O));
  }
}

template <int W>
__global__ void __launch_bounds__(256)
    k_poisson_inv(Grid g, const double2 *__restrict__ tw, const double2 *__restrict__ spec, double *__restrict__ psi) {
  extern __shared__ double2 smem[];
  const int ny = g.ny, M = ny >> 1, M1 = M + 1;
  double2 *A = smem, *B = smem + W * M;
  const int I0 = blockIdx.x * W + 1;
  for (int t = threadIdx.x; t < W * M; t += blockDim.x) {
    const int c = t / M, mm = t - c * M;
    const int I = I0 + c;
    double2 z = make_double2(0., 0.);
    if (I <= g.nx) {
      const double2 xm = spec[(size_t)(I - 1) * M1 + mm];
      const double2 xr = spec[(size_t)(I - 1) * M1 + (M - mm)];
      const double2 xc = make_double2(xr.x, -xr.y);
      const double2 E = cadd(xm, xc);
      const double2 w = make_double2(tw[mm].x, -tw[mm].y);
      const double2 O = cmul(csub(xm, xc), w);
      z = make_double2(E.x - O.y, E.y + O.x);
    }
    A[c * M + mm] = z;
  }
  __syncthreads();
  const double2 *zr = fft_rows<W>(A, B, M, tw, true);
  const double *xd = reinterpret_cast<const double *>(zr);
  for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
    const int c = t % W, r = t / W;
    const int I = I0 + c;
    if (I > g.nx) continue;
    const double v = xd[c * ny + r];
    psi[ix(g, r, I)] = v;
    if (I == 1) psi[ix(g, r, 0)] = v;
    if (I == g.nx) psi[ix(g, r, g.nx + 1)] = v;
  }
}

// Thomas sweeps along x for MB consecutive y wavenumbers held in shared
// memory as [I][mode] complex; fac[I][m] = (1 / pivot_I, off / pivot_I)
__global__ void __launch_bounds__(256)
    k_poisson_tdm(Grid g, int MB, const double2 *__restrict__ fac, double2 *__restrict__ spec) {
  extern __shared__ double2 s[];
  __shared__ double red[256];
  const int nx = g.nx, M1 = g.ny / 2 + 1;
  const int m0 = blockIdx.x * MB;
  const int nm = min(MB, M1 - m0);
  for (int t = threadIdx.x; t < nx * nm; t += blockDim.x) {
    const int i = t / nm, q = t - i * nm;
    s[i * MB + q] = spec[(size_t)i * M1 + m0 + q];
  }
  __syncthreads();
  if (threadIdx.x < 2 * nm) {
    const int q = threadIdx.x >> 1, comp = threadIdx.x & 1;
    double *sd = reinterpret_cast<double *>(s) + 2 * q + comp;
    const double2 *f = fac + m0 + q;
    double y = 0.;
#pragma unroll 8
    for (int i = 0; i < nx; ++i) {
      const double2 wv = f[(size_t)i * M1];
      y = fma(-wv.y, y, wv.x * sd[2 * MB * i]);
      sd[2 * MB * i] = y;
    }
    double x = y;
#pragma unroll 8
    for (int i = nx - 2; i >= 0; --i) {
      const double2 wv = f[(size_t)i * M1];
      x = fma(-wv.y, x, sd[2 * MB * i]);
      sd[2 * MB * i] = x;
    }
  }
  __syncthreads();
  if (m0 == 0) {
    // gauge of the singular mode: zero mean over x
    double acc = 0.;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) acc += s[i * MB].x;
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    const double mean = red[0] / nx;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
      s[i * MB].x -= mean;
      s[i * MB].y = 0.;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < nx * nm; t += blockDim.x) {
    const int i = t / nm, q = t - i * nm;
    spec[(size_t)i * M1 + m0 + q] = s[i * MB + q];
  }
}

// ---------------------------------------------------------------------------
// velocity correction (+ pressure update)
//   src/fluid/correct_velocity/ux.c:18-66, uy.c:17-64
//   src/fluid/update_pressure.c:7-53
// thread (I, J): I = 1..nx
// ---------------------------------------------------------------------------
template <bool PRES>
__global__ void __launch_bounds__(BX *BY)
    k_correct(Grid g, Metrics m, Phys ph, const double *__restrict__ sc, int k, double *__restrict__ ux,
              double *__restrict__ uy, const double *__restrict__ psin, const double *__restrict__ psio,
              const double *__restrict__ irhox, const double *__restrict__ irhoy, double *__restrict__ p) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int r = J - 1, rm = wrap(J - 1, g.ny);
  const double cnew = sc[sc_cnew(k)], cold = sc[sc_cold(k)];
  const double pn0 = psin[ix(g, r, I)], po0 = psio[ix(g, r, I)];
  if (I >= 2) {
    const double ih = m.ihxxf[I];
    double u = ux[ix(g, r, I - 1)];
    u = fma(-(cnew * ih), pn0 - psin[ix(g, r, I - 1)], u);
    u = fma(cold * (irhox[ix(g, r, I - 1)] - ph.irefden) * ih, po0 - psio[ix(g, r, I - 1)], u);
    ux[ix(g, r, I - 1)] = u;
  }
  {
    double u = uy[ix(g, r, I)];
    u = fma(-(cnew * g.ihy), pn0 - psin[ix(g, rm, I)], u);
    u = fma(cold * (irhoy[ix(g, r, I)] - ph.irefden) * g.ihy, po0 - psio[ix(g, rm, I)], u);
    uy[ix(g, r, I)] = u;
  }
  if (I == 1) {
    ux[ix(g, r, 0)] = 0.;
    uy[ix(g, r, 0)] = 0.;
  }
  if (I == g.nx) {
    ux[ix(g, r, g.nx)] = 0.;
    uy[ix(g, r, g.nx + 1)] = 0.;
  }
  if (PRES) {
    const double pv = p[ix(g, r, I)] + pn0;
    p[ix(g, r, I)] = pv;
    if (I == 1) p[ix(g, r, 0)] = pv;
    if (I == g.nx) p[ix(g, r, g.nx + 1)] = pv;
  }
}

// pressure update alone (fine-grained entry point); I = 1..nx
__global__ void k_pressure(Grid g, const double *__restrict__ psin, double *__restrict__ p) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int r = J - 1;
  const double pv = p[ix(g, r, I)] + psin[ix(g, r, I)];
  p[ix(g, r, I)] = pv;
  if (I == 1) p[ix(g, r, 0)] = pv;
  if (I == g.nx) p[ix(g, r, g.nx + 1)] = pv;
}

// ---------------------------------------------------------------------------
// time step size (src/decide_dt.c:34-169)
// min over faces of h / (|u| + 1e-8) equals h / (max |u| + 1e-8) for a
// fixed h because both roundings are monotone; so the kernel reduces max |u|
// per x column (ux) and over the domain (uy) on the integer patterns of the
// non-negative doubles, and one block finishes with nx + 1 divisions.  A
// non-finite velocity sets bit 0 of the status word.
// ---------------------------------------------------------------------------
constexpr unsigned long long kAbsMask = 0x7fffffffffffffffULL;
constexpr unsigned long long kInfBits = 0x7ff0000000000000ULL;

__global__ void __launch_bounds__(BX *BY)
    k_decide_dt(Grid g, Metrics m, Phys ph, const double *__restrict__ ux, const double *__restrict__ uy,
                unsigned long long *__restrict__ acc, double *__restrict__ sc, int *__restrict__ status,
                double dt_fixed, double coef_adv, double r_a0, double r_a1, double r_a2, double r_b0, double r_b1,
                double r_b2) {
  __shared__ unsigned long long colmax[BY][BX];
  __shared__ unsigned long long ymax[BY * BX];
  __shared__ bool last;
  const int I = blockIdx.x * BX + threadIdx.x + 1;  // 1..nx+1
  unsigned long long mx = 0ULL, my = 0ULL;
  if (I <= g.nx) {
    for (int J = blockIdx.y * BY + threadIdx.y + 1; J <= g.ny; J += gridDim.y * BY) {
      const int r = J - 1;
      if (I >= 2) {
        const unsigned long long b = (unsigned long long)dbits(ux[ix(g, r, I - 1)]) & kAbsMask;
        mx = b > mx ? b : mx;
      }
      const unsigned long long c = (unsigned long long)dbits(uy[ix(g, r, I)]) & kAbsMask;
      my = c > my ? c : my;
    }
  }
  colmax[threadIdx.y][threadIdx.x] = mx;
  const int tid = threadIdx.y * BX + threadIdx.x;
  ymax[tid] = my;
  __syncthreads();
  if (threadIdx.y == 0) {
    unsigned long long v = 0ULL;
    for (int k = 0; k < BY; ++k) v = colmax[k][threadIdx.x] > v ? colmax[k][threadIdx.x] : v;
    if (I <= g.nx && v) atomicMax(acc + I, v);
    __threadfence();
  }
  for (int w = BX * BY / 2; w > 0; w >>= 1) {
    if (tid < w) ymax[tid] = ymax[tid + w] > ymax[tid] ? ymax[tid + w] : ymax[tid];
    __syncthreads();
  }
  if (tid == 0) {
    if (ymax[0]) atomicMax(acc + g.nx + 2, ymax[0]);
    __threadfence();
    const unsigned int nb = gridDim.x * gridDim.y;
    const unsigned int done = atomicAdd(reinterpret_cast<unsigned int *>(acc + g.nx + 3), 1u);
    last = (done == nb - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // finishing block: dt_adv = coef * min(1, min_i hx_i / (max|ux|_i + small), hy / (max|uy| + small))
  __shared__ double dmin[BY * BX];
  __shared__ unsigned long long bad[BY * BX];
  const double small = 1.e-8;
  double d = 1.;
  unsigned long long nb = 0ULL;
  for (int i = tid + 2; i <= g.nx; i += BX * BY) {
    const unsigned long long b = atomicAdd(acc + i, 0ULL);
    nb |= (b >= kInfBits) ? 1ULL : 0ULL;
    d = fmin(d, m.hxxf[i] / (__longlong_as_double((long long)b) + small));
  }
  dmin[tid] = d;
  bad[tid] = nb;
  __syncthreads();
  for (int w = BX * BY / 2; w > 0; w >>= 1) {
    if (tid < w) {
      dmin[tid] = fmin(dmin[tid], dmin[tid + w]);
      bad[tid] |= bad[tid + w];
    }
    __syncthreads();
  }
  if (tid == 0) {
    const unsigned long long by = atomicAdd(acc + g.nx + 2, 0ULL);
    double dt = fmin(dmin[0], g.hy / (__longlong_as_double((long long)by) + small));
    dt *= coef_adv;
    dt = fmin(dt, dt_fixed);
    if (bad[0] || by >= kInfBits) atomicOr(status, 1);
    const double al[3] = {r_a0, r_a1, r_a2}, be[3] = {r_b0, r_b1, r_b2};
    sc[0] = dt;
    for (int k = 0; k < 3; ++k) {
      const double gk = al[k] + be[k];
      const int ko = (k + 2) % 3;
      const double go = al[ko] + be[ko];
      const double dtold = go * dt, dtnew = gk * dt;
      sc[sc_adt(k)] = al[k] * dt;
      sc[sc_bdt(k)] = be[k] * dt;
      sc[sc_gdt(k)] = gk * dt;
      sc[sc_dtold(k)] = dtold;
      sc[sc_dtnew(k)] = dtnew;
      sc[sc_pdiv(k)] = ph.refden / dtnew / g.ny;
      sc[sc_padd(k)] = -(dtold / dtnew) / g.ny;
      sc[sc_cnew(k)] = dtnew / ph.refden;
      sc[sc_cold(k)] = -dtold;
    }
  }
  __syncthreads();
  // reset the accumulators for the next launch
  for (int i = tid; i <= g.nx + 3; i += BX * BY) acc[i] = 0ULL;
}

// 1 / rho at ux faces (I = 1..nx+1) and uy faces (I = 1..nx) from a density
// field, as k_predict stores them (fine-grained entry points); I = 1..nx+1
__global__ void k_inv_face_density(Grid g, const double *__restrict__ den, double *__restrict__ irhox,
                                   double *__restrict__ irhoy) {
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int r = J - 1, rm = wrap(J - 1, g.ny);
  irhox[ix(g, r, I - 1)] = __drcp_rn(half_sum(den[ix(g, r, I - 1)], den[ix(g, r, I)]));
  if (I <= g.nx) irhoy[ix(g, r, I)] = __drcp_rn(half_sum(den[ix(g, rm, I)], den[ix(g, r, I)]));
}

// ---- boundary kernels of the fine-grained entry points (one thread per row)
__global__ void k_bc_ux(Grid g, double *ux) {
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  ux[ix(g, J - 1, 0)] = 0.;
  ux[ix(g, J - 1, g.nx)] = 0.;
}
__global__ void k_bc_uy(Grid g, double *uy) {
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  uy[ix(g, J - 1, 0)] = 0.;
  uy[ix(g, J - 1, g.nx + 1)] = 0.;
}
__global__ void k_bc_neumann(Grid g, double *f) {
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  f[ix(g, J - 1, 0)] = f[ix(g, J - 1, 1)];
  f[ix(g, J - 1, g.nx + 1)] = f[ix(g, J - 1, g.nx)];
}
__global__ void k_bc_vof(Grid g, double *vof) {
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  vof[ix(g, J - 1, 0)] = 0.;
  vof[ix(g, J - 1, g.nx + 1)] = 0.;
}

constexpr int kFftCols = 4;

}  // namespace

// ===========================================================================
// launch helpers
// ===========================================================================

int poisson_fft_cols(int) { return kFftCols; }
size_t poisson_fft_smem(int ny) { return sizeof(double2) * 2 * kFftCols * (size_t)(ny / 2); }
int poisson_tdm_modes(int nx) {
  int mb = 8;
  while (mb > 1 && sizeof(double2) * (size_t)nx * mb > 200 * 1024) mb >>= 1;
  return mb;
}
size_t poisson_tdm_smem(int nx) { return sizeof(double2) * (size_t)nx * poisson_tdm_modes(nx); }

cudaError_t configure_kernels() {
  cudaError_t e;
  const int big = 227 * 1024;
  e = cudaFuncSetAttribute(k_poisson_fwd<kFftCols>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_inv<kFftCols>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_tdm, cudaFuncAttributeMaxDynamicSharedMemorySize, big - 4096);
  return e;
}

void launch_props(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b, bool den, bool vis,
                  bool grad, double *den_out) {
  const dim3 gr = grid2d(g.nx + 2, g.ny), bl(BX, BY);
  if (den && vis && grad)
    k_props<true, true, true><<<gr, bl, 0, s>>>(g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof);
  else if (vis && grad)
    k_props<false, true, true><<<gr, bl, 0, s>>>(g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof);
  else if (den)
    k_props<true, false, false><<<gr, bl, 0, s>>>(g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof);
  else if (vis)
    k_props<false, true, false><<<gr, bl, 0, s>>>(g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof);
  else if (grad)
    k_props<false, false, true><<<gr, bl, 0, s>>>(g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof);
}

void launch_normal_curv(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, bool normal, bool curv) {
  const dim3 gr = grid2d(g.nx, g.ny), bl(BX, BY);
  if (normal && curv) k_normal_curv<true, true><<<gr, bl, 0, s>>>(g, m, b.vof, b.dvof, b.normal, b.curv);
  else if (normal) k_normal_curv<true, false><<<gr, bl, 0, s>>>(g, m, b.vof, b.dvof, b.normal, b.curv);
  else if (curv) k_normal_curv<false, true><<<gr, bl, 0, s>>>(g, m, b.vof, b.dvof, b.normal, b.curv);
}

void launch_flux_force(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                       const double *ux, const double *uy, const double *den0, bool flux, bool force) {
  const dim3 gr = grid2d(g.nx, g.ny), bl(BX, BY);
  if (flux && force)
    k_flux_force<true, true><<<gr, bl, 0, s>>>(g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx, b.fluxy,
                                               b.ifrcx, b.ifrcy);
  else if (flux)
    k_flux_force<true, false><<<gr, bl, 0, s>>>(g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx, b.fluxy,
                                                b.ifrcx, b.ifrcy);
  else if (force)
    k_flux_force<false, true><<<gr, bl, 0, s>>>(g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx, b.fluxy,
                                                b.ifrcx, b.ifrcy);
}

void launch_vof_advance(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                        const double *sc, int k, double *src_a, const double *src_b, bool fused, const double *ux,
                        const double *uy, double *den1) {
  const dim3 gr = grid2d(g.nx, g.ny), bl(BX, BY);
  if (fused)
    k_vof_advance<true><<<gr, bl, 0, s>>>(g, m, ph, sc, k, b.vof, b.fluxx, b.fluxy, src_a, src_b, ux, uy, b.mfluxx,
                                          b.mfluxy, den1);
  else
    k_vof_advance<false><<<gr, bl, 0, s>>>(g, m, ph, sc, k, b.vof, b.fluxx, b.fluxy, src_a, src_b, ux, uy, nullptr,
                                           nullptr, nullptr);
}

void launch_mass_flux_inplace(cudaStream_t s, const Grid &g, const Phys &ph, const Bufs &b, const double *ux,
                              const double *uy) {
  k_mass_flux<<<grid2d(g.nx + 2, g.ny), dim3(BX, BY), 0, s>>>(g, ph, ux, uy, b.fluxx, b.fluxy);
}

void launch_stress(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, const double *ux,
                   const double *uy) {
  k_stress<<<grid2d(g.nx + 1, g.ny), dim3(BX, BY), 0, s>>>(g, m, ux, uy, b.visux, b.visuy, b.txx, b.txy, b.tyy);
}

void launch_predict(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b, const double *sc,
                    int k, const double *ux, const double *uy, double *ux_out, double *uy_out, const double *mfx,
                    const double *mfy, const double *den0, const double *den1, double *srcux_a,
                    const double *srcux_b, double *srcux_g, double *srcuy_a, const double *srcuy_b,
                    double *srcuy_g) {
  k_predict<<<grid2d(g.nx, g.ny), dim3(BX, BY), 0, s>>>(g, m, ph, sc, k, ux, uy, ux_out, uy_out, mfx, mfy, b.txx,
                                                        b.txy, b.tyy, b.p, b.ifrcx, b.ifrcy, den0, den1, srcux_a,
                                                        srcux_b, srcux_g, srcuy_a, srcuy_b, srcuy_g, b.irhox,
                                                        b.irhoy);
}

void launch_poisson_fwd(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                        const double *sc, int k, const double *ux, const double *uy, const double *psi_old) {
  const int nb = (g.nx + kFftCols - 1) / kFftCols;
  k_poisson_fwd<kFftCols><<<nb, 256, poisson_fft_smem(g.ny), s>>>(g, m, ph, sc, k, ux, uy, psi_old, b.irhox,
                                                                  b.irhoy, b.twiddle, b.spec);
}

void launch_poisson_tdm(cudaStream_t s, const Grid &g, const Bufs &b) {
  const int mb = poisson_tdm_modes(g.nx);
  const int M1 = g.ny / 2 + 1;
  k_poisson_tdm<<<(M1 + mb - 1) / mb, 256, poisson_tdm_smem(g.nx), s>>>(g, mb, b.tdm_fac, b.spec);
}

void launch_poisson_inv(cudaStream_t s, const Grid &g, const Bufs &b, double *psi_new) {
  const int nb = (g.nx + kFftCols - 1) / kFftCols;
  k_poisson_inv<kFftCols><<<nb, 256, poisson_fft_smem(g.ny), s>>>(g, b.twiddle, b.spec, psi_new);
}

void launch_poisson(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b, const double *sc,
                    int k, const double *ux, const double *uy, const double *psi_old, double *psi_new) {
  launch_poisson_fwd(s, g, m, ph, b, sc, k, ux, uy, psi_old);
  launch_poisson_tdm(s, g, b);
  launch_poisson_inv(s, g, b, psi_new);
}

void launch_correct(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b, const double *sc,
                    int k, double *ux, double *uy, const double *psi_new, const double *psi_old, bool pressure) {
  const dim3 gr = grid2d(g.nx, g.ny), bl(BX, BY);
  if (pressure)
    k_correct<true><<<gr, bl, 0, s>>>(g, m, ph, sc, k, ux, uy, psi_new, psi_old, b.irhox, b.irhoy, b.p);
  else
    k_correct<false><<<gr, bl, 0, s>>>(g, m, ph, sc, k, ux, uy, psi_new, psi_old, b.irhox, b.irhoy, b.p);
}

void launch_pressure(cudaStream_t s, const Grid &g, const Bufs &b, const double *psi_new) {
  k_pressure<<<grid2d(g.nx, g.ny), dim3(BX, BY), 0, s>>>(g, psi_new, b.p);
}

void launch_decide_dt(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                      const double *ux, const double *uy, double dt_fixed, double coef_adv) {
  // RK3 coefficients (reference src/runge_kutta.c:8-15)
  const double a0 = 32. / 60., b0 = 0. / 60.;
  const double a1 = 25. / 60., b1 = -17. / 60.;
  const double a2 = 45. / 60., b2 = -25. / 60.;
  int gy = (g.ny + BY - 1) / BY;
  const int gx = (g.nx + BX) / BX;
  while (gy > 1 && gx * gy > 4 * 152) gy = (gy + 1) / 2;
  k_decide_dt<<<dim3(gx, gy), dim3(BX, BY), 0, s>>>(g, m, ph, ux, uy, b.dt_acc, b.scalars, b.status, dt_fixed,
                                                    coef_adv, a0, a1, a2, b0, b1, b2);
}

void launch_inv_face_density(cudaStream_t s, const Grid &g, const double *den, double *irhox, double *irhoy) {
  k_inv_face_density<<<grid2d(g.nx + 1, g.ny), dim3(BX, BY), 0, s>>>(g, den, irhox, irhoy);
}

void launch_bc_ux(cudaStream_t s, const Grid &g, double *ux) { k_bc_ux<<<(g.ny + 127) / 128, 128, 0, s>>>(g, ux); }
void launch_bc_uy(cudaStream_t s, const Grid &g, double *uy) { k_bc_uy<<<(g.ny + 127) / 128, 128, 0, s>>>(g, uy); }
void launch_bc_neumann(cudaStream_t s, const Grid &g, double *f) {
  k_bc_neumann<<<(g.ny + 127) / 128, 128, 0, s>>>(g, f);
}
void launch_bc_vof(cudaStream_t s, const Grid &g, double *vof) {
  k_bc_vof<<<(g.ny + 127) / 128, 128, 0, s>>>(g, vof);
}

}  // namespace sbfs
