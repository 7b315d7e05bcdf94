// sm_103a kernels of the 2-D two-phase (VOF) time step.
//
// All arithmetic is FP64.  On GB300 the FP64 pipe (about 0.5 T fused
// multiply-adds per second, measured) bounds this solver, not HBM (a first
// version of the momentum kernel ran its FP64 pipe at 86% of peak with DRAM
// at 9%), so every kernel is written to spend as few FP64 instructions per
// cell as the discretisation allows:
//   * the reference's metric factors are folded into one coefficient per
//     column or per grid (see sbfs_device.cuh), and constant factors such
//     as the 0.5 of face averages are folded into those coefficients;
//   * reciprocals and inverse square roots are Newton-Raphson refinements of
//     the hardware seeds (rcp_nr, rsqrt_nr);
//   * 1 / rho^{k+1} is formed once per face and substage, and stored as
//     e = rho_ref / rho - 1, the factor the Poisson right-hand side and the
//     velocity correction both need;
//   * the THINC indicator 0.5 (1 + tanh(n . x + d)) with the intercept
//     d = -ln(1/phi - 1) / 2 equals 1 / (1 + K exp(-2 n . x)), K = 1/phi - 1:
//     one exponential per Gauss point and no logarithm;
//   * threshold tests (vofmin, upwind sign, clipping) run on the integer
//     pattern of the double; cells whose stencil inputs are bitwise equal
//     (single-phase bulk) take the exact short cut.
// The reference file:line each kernel follows is cited at the kernel.
#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>

#include "sbfs_kernels.cuh"

namespace sbfs {

int g_pdl = 1;  // step kernels launched with programmatic stream serialisation
int g_stream_prio = 1;
int g_compact = -1;

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ size_t ix(const Grid &g, int row, int col) { return (size_t)row * g.p1 + col; }
__device__ __forceinline__ bool same(double a, double b) { return dbits(a) == dbits(b); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// Interface-branch compaction.  An FP64 instruction costs its warp an issue
// slot however few of its lanes run it (measured: eight FMA chains on 1 to
// 32 lanes of every warp all took the same time), and the cells that need
// the FP64 work of an interface branch lie along the interface and its THINC
// tails, often a few to a warp.  block_compact lists the block's threads
// whose flag is set in list[0 .. n) in thread order (a ballot per warp, a
// prefix over the warp counts in shared memory) and returns n, so that
// threads 0 .. n-1 can each take one listed cell and fill whole warps.
// Every thread of the block must call it (two barriers).
__device__ __forceinline__ int block_compact(bool flag, int tid, int *cnt, int *list) {
  const int lane = tid & 31, warp = tid >> 5, nwarp = (blockDim.x * blockDim.y + 31) >> 5;
  const unsigned mask = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) cnt[warp] = __popc(mask);
  __syncthreads();
  int off = 0, n = 0;
  for (int w = 0; w < nwarp; ++w) {
    const int c = cnt[w];
    off += w < warp ? c : 0;
    n += c;
  }
  if (flag) list[off + __popc(mask & ((1u << lane) - 1u))] = tid;
  __syncthreads();
  return n;
}

dim3 grid2d(int ni, int nj, int nz = 1) { return dim3((ni + BX - 1) / BX, (nj + BY - 1) / BY, nz); }
// grid of the block shape of kernel k
dim3 tile_block(const Tiles &t, int k) { return dim3(t.bx[k], t.by[k]); }
dim3 tile_grid(const Tiles &t, int k, int ni, int nj, int nz) {
  return dim3((ni + t.bx[k] - 1) / t.bx[k], (nj + t.by[k] - 1) / t.by[k], nz);
}

// ---------------------------------------------------------------------------
// density, viscosity, corner gradients of vof
//   den:   src/fluid/density.c:9-31
//   visux: src/fluid/viscosity.c:23-61, visuy: :63-91
//   dvof:  src/interface/curvature_tensor.c:16-49
// thread (I, J): I = 0..nx+1
// ---------------------------------------------------------------------------
// unit normal of the vof gradient at the corner between columns I-1, I and
// rows J-1, J of a case (curvature_tensor.c:16-49)
__device__ __forceinline__ void corner_normal(const Grid &g, const Metrics &m, const double *__restrict__ vof,
                                              double *__restrict__ dvof, int zr, int I, int J) {
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr;
  const double a = vof[ix(g, rm, I - 1)], b = vof[ix(g, rm, I)];
  const double c = vof[ix(g, r, I - 1)], d = vof[ix(g, r, I)];
  // the reference's summation order, kept on purpose: in the THINC tails the
  // four values differ by ~1e-16 and the reference's sum is rounding noise
  // that the normalisation below (by max(|g|, eps)) scales up to O(1);
  // another order gives O(1) different corner normals
  const double gx = m.ihxxf[I] * (((-a + b) - c) + d);
  const double gy = g.ihy * (((-a - b) + c) + d);
  const double inv = inv_norm(fma(gx, gx, gy * gy));
  reinterpret_cast<double2 *>(dvof)[(size_t)r * (g.p2 / 2) + (I - 1)] = make_double2(gx * inv, gy * inv);
}

// compact: the corners with a gradient are handed to the block's first
// threads (see the interface-branch compaction below); otherwise each thread
// does its own.  The same arithmetic either way.  SCALED: the fused step's
// viscosities, visux times 2 nu / hy and visuy times 4 nu / hy (the factors
// k_momflux would otherwise apply per cell), formed with the constants and
// clip bounds scaled alike: the same two FP64 operations per face
template <bool DEN, bool VIS, bool GRAD, bool SCALED = false>
__global__ void __launch_bounds__(BX *BY) k_props(Grid g, Metrics m, Phys ph0, const double *__restrict__ vof,
                                                  double *__restrict__ den, double *__restrict__ visux,
                                                  double *__restrict__ visuy, double *__restrict__ dvof,
                                                  int compact) {
  pdl_entry();
  const Phys ph = zphys(g, ph0);
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const bool in = I <= g.nx + 1 && J <= g.ny;
  const bool cmp = GRAD && compact;  // uniform over the block
  if (!cmp && !in) return;  // when compacting, every thread meets the barriers below
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr;
  bool need = false;  // the corner gradient is not identically zero
  if (in) {
    const double v = vof[ix(g, r, I)];
    if (DEN) den[ix(g, r, I)] = clip_pos(fma(ph.dm1, v, 1.), ph.den_lo, ph.den_hi);
    if (VIS) {
      // 1 + (visr - 1) 0.5 (a + b) = 1 + c2 (a + b), c2 = (visr - 1) / 2
      const double c = SCALED ? ph.vsx_c : ph.vm1, c2 = SCALED ? ph.vsx_c2 : ph.hvm1, one = SCALED ? ph.vsx_1 : 1.;
      if (I >= 1) {
        double vis;
        if (I == 1) vis = fma(c, vof[ix(g, r, 0)], one);
        else if (I == g.nx + 1) vis = fma(c, v, one);
        else vis = fma(c2, vof[ix(g, r, I - 1)] + v, one);
        visux[ix(g, r, I - 1)] = SCALED ? clip_pos(vis, ph.vsx_lo, ph.vsx_hi) : clip_pos(vis, ph.vis_lo, ph.vis_hi);
      }
      const double vy = SCALED ? fma(ph.vsy_c2, vof[ix(g, rm, I)] + v, ph.vsy_1) : fma(c2, vof[ix(g, rm, I)] + v, 1.);
      visuy[ix(g, r, I)] = SCALED ? clip_pos(vy, ph.vsy_lo, ph.vsy_hi) : clip_pos(vy, ph.vis_lo, ph.vis_hi);
    }
    if (GRAD && I >= 1) {
      // zero where the four values are bitwise equal (single-phase bulk)
      const double a = vof[ix(g, rm, I - 1)], b = vof[ix(g, rm, I)], c = vof[ix(g, r, I - 1)];
      need = !(same(a, b) && same(b, c) && same(c, v));
      if (!need) reinterpret_cast<double2 *>(dvof)[(size_t)r * (g.p2 / 2) + (I - 1)] = make_double2(0., 0.);
      else if (!cmp) corner_normal(g, m, vof, dvof, zr, I, J);
    }
  }
  if (cmp) {
    __shared__ int cnt[BX * BY / 32];
    __shared__ int list[BX * BY];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int n = block_compact(need, tid, cnt, list);
    if (tid < n) {
      const int sy = list[tid] / blockDim.x, sx = list[tid] - sy * blockDim.x;
      corner_normal(g, m, vof, dvof, zr, blockIdx.x * blockDim.x + sx, blockIdx.y * blockDim.y + sy + 1);
    }
  }
}

// ---------------------------------------------------------------------------
// cell normal + THINC parameter (interface cells) and curvature
//   normal:    src/interface/curvature_tensor.c:51-97
//   curvature: src/interface/curvature_tensor.c:100-135
//     kappa = -[(nx_xp - nx_xm) / HXXC + (ny_yp - ny_ym) / hy]
// STORE_K: the third component is K = 1/phi - 1 (used by the fused step);
// otherwise the reference's intercept d = -ln(1/phi - 1) / 2.
// thread (I, J): I = 1..nx
// ---------------------------------------------------------------------------
template <bool NORMAL, bool CURV, bool STORE_K>
__global__ void __launch_bounds__(BX *BY) k_normal_curv(Grid g, Metrics m, const double *__restrict__ vof,
                                                        const double *__restrict__ dvof, double *__restrict__ normal,
                                                        double *__restrict__ curv) {
  pdl_entry();
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
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
      const double ddx = (d10.x + d11.x) - (d00.x + d01.x);
      const double ddy = (d01.y + d11.y) - (d00.y + d10.y);
      k = -fma(m.hihxxc[I], ddx, g.hihy * ddy);
    }
    curv[ix(g, r, I)] = k;
  }
  if (NORMAL) {
    const double phi = vof[ix(g, r, I)];
    if (!single_phase(phi)) {
      const double mx = (((d00.x + d10.x) + d01.x) + d11.x) * m.ihxxc[I];
      const double my = (((d00.y + d10.y) + d01.y) + d11.y) * g.ihy;
      const double inv = inv_norm(fma(mx, mx, my * my));
      double *o = normal + (size_t)r * g.p3 + (size_t)(I - 1) * 3;
      o[0] = mx * inv;
      o[1] = my * inv;
      o[2] = STORE_K ? rcp_nr(phi) - 1. : -0.5 * log(__drcp_rn(phi) - 1.);
    }
  }
}

// THINC flux factor of one face (src/interface/update/main.c:18-35,
// fluxx.c:62-68): the mean of the indicator over the two Gauss points
// t = +-g of the face, 0.5 sum 1 / (1 + K exp(-2 (n_a s + n_b t))), where s
// is the face position along its normal (+-1/2) and n_a, n_b the normal
// components along and across it.  With a = K exp(-2 n_a s) and
// b = exp(-2 n_b g) the two terms are 1 / (1 + a b) and b / (b + a).
// The caller passes -2 n_a s, which for s = -+1/2 is exactly +-n_a.
__device__ __forceinline__ double thinc_ab(double a, double b) {
  const double p = fma(a, b, 1.);
  const double q = b + a;
  // b p + q >= b >= exp(-2 g) > 1/2: positive and normal
  return half_pos_normal(fma(b, p, q)) * rcp_nr(p * q);
}
// a is rounded on its own (never fused into q = b + a), so that a factor
// formed ahead of time (k_curv_list<false>) gives the same flux
__device__ __forceinline__ double thinc_face(double m2nas, double nb, double K) {
  return thinc_ab(__dmul_rn(K, exp(m2nas)), exp(-2. * kGaussPt * nb));
}

// ---------------------------------------------------------------------------
// THINC vof fluxes and CSF surface-tension force
//   fluxes: src/interface/update/fluxx.c:14-73, fluxy.c:14-73
//   force:  src/interface/force.c:20-88
// HAVE_K: normal[2] holds K = 1/phi - 1 (fused step) instead of the
// reference's intercept d (then K = exp(-2 d)).
// thread (I, J): I = 1..nx handles x face I (I >= 2) and y face (I, J - 1/2)
// ---------------------------------------------------------------------------
// ITF_KAPPA (learned curvature mode): the face curvature comes from the
// interface side alone when only one of the two cells is an interface cell
// (the -div n of a single-phase cell next to the interface is not a
// curvature of anything); otherwise the mean, as in the reference.
__device__ __forceinline__ double face_kappa_sum(double pl, double pr, double kl, double kr) {
  const bool il = !single_phase(pl), ir = !single_phase(pr);
  return il == ir ? kl + kr : (il ? 2. * kl : 2. * kr);
}

template <bool FLUX, bool FORCE, bool HAVE_K, bool BULK_ONLY, bool ITF_KAPPA>
__device__ __forceinline__ void flux_force_body(const Grid &g, const Metrics &m, const Phys &ph0,
                                                const double *__restrict__ ux, const double *__restrict__ uy,
                                                const double *__restrict__ vof, const double *__restrict__ normal,
                                                const double *__restrict__ den0, const double *__restrict__ curv,
                                                double *__restrict__ fluxx, double *__restrict__ fluxy,
                                                double *__restrict__ ifrcx, double *__restrict__ ifrcy) {
  const Phys ph = zphys(g, ph0);
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr;
  const double v0 = vof[ix(g, r, I)];
  const double vxm = vof[ix(g, r, I - 1)];
  const double vym = vof[ix(g, rm, I)];
  if (FLUX) {
    if (I >= 2) {
      const double vel = ux[ix(g, r, I - 1)];
      const bool n = neg(vel);
      const int iu = n ? I : I - 1;
      const double phi = n ? v0 : vxm;
      if (single_phase(phi)) {
        fluxx[ix(g, r, I - 1)] = vel * phi;
      } else if (!BULK_ONLY) {
        const double *nv = normal + (size_t)r * g.p3 + (size_t)(iu - 1) * 3;
        const double K = HAVE_K ? nv[2] : exp(-2. * nv[2]);
        fluxx[ix(g, r, I - 1)] = vel * thinc_face(n ? nv[0] : -nv[0], nv[1], K);
      }
    }
    {
      const double vel = uy[ix(g, r, I)];
      const bool n = neg(vel);
      const int ru = n ? r : rm;
      const double phi = n ? v0 : vym;
      if (single_phase(phi)) {
        fluxy[ix(g, r, I)] = vel * phi;
      } else if (!BULK_ONLY) {
        const double *nv = normal + (size_t)ru * g.p3 + (size_t)(I - 1) * 3;
        const double K = HAVE_K ? nv[2] : exp(-2. * nv[2]);
        fluxy[ix(g, r, I)] = vel * thinc_face(n ? nv[1] : -nv[1], nv[0], K);
      }
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
    // f = 0.5 (rho_l + rho_r) 2 / (1 + denr) / We 0.5 (k_l + k_r) (phi_r - phi_l) / h
    if (I >= 2) {
      double f = 0.;
      if (!same(vxm, v0)) {
        const double rho = den0[ix(g, r, I - 1)] + den0[ix(g, r, I)];
        const double kap = ITF_KAPPA ? face_kappa_sum(vxm, v0, curv[ix(g, r, I - 1)], curv[ix(g, r, I)])
                                     : curv[ix(g, r, I - 1)] + curv[ix(g, r, I)];
        f = (rho * kap) * ((ph.qf * m.ihxxf[I]) * (v0 - vxm));
      }
      ifrcx[ix(g, r, I - 2)] = f;
    }
    double f = 0.;
    if (!same(vym, v0)) {
      const double rho = den0[ix(g, rm, I)] + den0[ix(g, r, I)];
      const double kap = ITF_KAPPA ? face_kappa_sum(vym, v0, curv[ix(g, rm, I)], curv[ix(g, r, I)])
                                   : curv[ix(g, rm, I)] + curv[ix(g, r, I)];
      f = (rho * kap) * (ph.qfy * (v0 - vym));
    }
    ifrcy[ix(g, r, I - 1)] = f;
  }
}

template <bool FLUX, bool FORCE, bool HAVE_K, bool BULK_ONLY = false, bool ITF_KAPPA = false>
__global__ void __launch_bounds__(BX *BY)
    k_flux_force(Grid g, Metrics m, Phys ph0, const double *__restrict__ ux, const double *__restrict__ uy,
                 const double *__restrict__ vof, const double *__restrict__ normal, const double *__restrict__ den0,
                 const double *__restrict__ curv, double *__restrict__ fluxx, double *__restrict__ fluxy,
                 double *__restrict__ ifrcx, double *__restrict__ ifrcy) {
  pdl_entry();
  flux_force_body<FLUX, FORCE, HAVE_K, BULK_ONLY, ITF_KAPPA>(g, m, ph0, ux, uy, vof, normal, den0, curv, fluxx, fluxy,
                                                             ifrcx, ifrcy);
}

// the fluxes of the faces whose upwind cell is single-phase (flux = vel phi)
// and the wall faces; the faces of upwind interface cells are k_face_flux's
__global__ void __launch_bounds__(BX *BY)
    k_bulk_flux(Grid g, Metrics m, Phys ph0, const double *__restrict__ ux, const double *__restrict__ uy,
                const double *__restrict__ vof, double *__restrict__ fluxx, double *__restrict__ fluxy) {
  pdl_entry();
  flux_force_body<true, false, true, true, false>(g, m, ph0, ux, uy, vof, nullptr, nullptr, nullptr, fluxx, fluxy,
                                                  nullptr, nullptr);
}

// the CSF force alone (it needs no velocity), into the force buffers given
template <bool ITF_KAPPA>
__global__ void __launch_bounds__(BX *BY)
    k_csf_force(Grid g, Metrics m, Phys ph0, const double *__restrict__ vof, const double *__restrict__ den0,
                const double *__restrict__ curv, double *__restrict__ ifrcx, double *__restrict__ ifrcy) {
  pdl_entry();
  flux_force_body<false, true, false, false, ITF_KAPPA>(g, m, ph0, nullptr, nullptr, vof, nullptr, den0, curv,
                                                        nullptr, nullptr, ifrcx, ifrcy);
}

// ---------------------------------------------------------------------------
// Interface compaction of the fused step.  THINC work (normal, intercept,
// two exponentials per face) exists only in interface cells, a few percent
// of the domain scattered along the bubbles; done in place it makes whole
// warps wait on a few lanes.  Two arrangements, the same arithmetic:
// listed faces (the step's first form):
//   k_curv_list<true> curvature of every cell (curvature_tensor.c:100-135),
//                     a list of the interface cells and a list of the faces
//                     they are upwind of (block-aggregated appends)
//   k_interface_cells one thread per listed face: the cell's normal and
//                     K = 1/phi - 1 (curvature_tensor.c:51-97), then the THINC
//                     flux of that face (update/fluxx.c, fluxy.c); a cell
//                     with two upwind faces is set up twice, but no warp
//                     runs a face branch only some of its lanes take
//   k_flux_force<.., BULK_ONLY>  every other face (upwind cell single-phase:
//                     flux = vel phi) and the CSF force
// Each face is written by exactly one of them: the upwind choice and the
// vofmin test are the same integer tests in both.
// geometry ahead (the default): everything but the upwind choice depends on
// vof alone, so it runs beside the previous substage's predictor and
// Poisson solve, and no flux kernel stands between the correction and the
// VOF update:
//   k_curv_list<false> curvature, the interface-cell list and per interface
//                     cell its THINC factors K exp(+-n_a) for its four faces
//                     and exp(-2 g n_b) across x and y faces (the block's
//                     interface cells handed to its first threads)
//   k_csf_force       the CSF force
//   k_face_flux       one thread per face of a listed cell: the upwind test,
//                     then the THINC flux from the cell's factors
//   k_bulk_flux       every other face, as k_flux_force<.., BULK_ONLY>
// ---------------------------------------------------------------------------
// kappa = -div n of cell (I, J) of a case from its four corner normals
// (curvature_tensor.c:100-135)
__device__ __forceinline__ void cell_curv(const Grid &g, const Metrics &m, const double2 *__restrict__ dv,
                                          double *__restrict__ curv, int zr, int I, int J) {
  const size_t q = g.p2 / 2;
  const int r = J - 1 + zr, rp = wrap(J + 1, g.ny) + zr;
  const double2 d00 = dv[(size_t)r * q + (I - 1)], d10 = dv[(size_t)r * q + I];
  const double2 d01 = dv[(size_t)rp * q + (I - 1)], d11 = dv[(size_t)rp * q + I];
  const double ddx = (d10.x + d11.x) - (d00.x + d01.x);
  const double ddy = (d01.y + d11.y) - (d00.y + d10.y);
  curv[ix(g, r, I)] = -fma(m.hihxxc[I], ddx, g.hihy * ddy);
}

// unit normal (n0, n1) and K = 1/phi - 1 of interface cell (I, J) of a case
// (curvature_tensor.c:51-97)
__device__ __forceinline__ void cell_normal_k(const Grid &g, const Metrics &m, const double2 *__restrict__ dv,
                                              const double *__restrict__ vof, int zr, int I, int J, double &n0,
                                              double &n1, double &K) {
  const size_t q = g.p2 / 2;
  const int r = J - 1 + zr, rp = wrap(J + 1, g.ny) + zr;
  const double2 d00 = dv[(size_t)r * q + (I - 1)], d10 = dv[(size_t)r * q + I];
  const double2 d01 = dv[(size_t)rp * q + (I - 1)], d11 = dv[(size_t)rp * q + I];
  const double mx = (((d00.x + d10.x) + d01.x) + d11.x) * m.ihxxc[I];
  const double my = (((d00.y + d10.y) + d01.y) + d11.y) * g.ihy;
  const double inv = inv_norm(fma(mx, mx, my * my));
  n0 = mx * inv;
  n1 = my * inv;
  K = rcp_nr(vof[ix(g, r, I)]) - 1.;
}

// THINC factors of interface cell (I, J), stored at its cell index `at`
// (planar, cap entries a table, kThincTabs of them): a of its left, right,
// bottom and top faces (thinc_face's K exp(-2 n_a s)), then b of its x and
// of its y faces
__device__ __forceinline__ void cell_thinc_factors(const Grid &g, const Metrics &m, const double2 *__restrict__ dv,
                                                   const double *__restrict__ vof, int zr, int I, int J,
                                                   double *__restrict__ tf, size_t cap, int at) {
  double n0, n1, K;
  cell_normal_k(g, m, dv, vof, zr, I, J, n0, n1, K);
  tf[at] = __dmul_rn(K, exp(n0));
  tf[cap + at] = __dmul_rn(K, exp(-n0));
  tf[2 * cap + at] = __dmul_rn(K, exp(n1));
  tf[3 * cap + at] = __dmul_rn(K, exp(-n1));
  tf[4 * cap + at] = exp(-2. * kGaussPt * n1);
  tf[5 * cap + at] = exp(-2. * kGaussPt * n0);
}

// compact: the cells with a corner normal hand their curvature to the
// block's first threads (interface-branch compaction); otherwise each thread
// computes its own.  The same arithmetic either way.
// FACES: also the list of the faces the interface cells are upwind of (from
// the velocity); else, without the velocity, the THINC factors of every
// interface cell (tables by cell index), by the block's first threads
template <bool FACES>
__global__ void __launch_bounds__(BX *BY) k_curv_list(Grid g, Metrics m, const double *__restrict__ vof,
                                                      const double *__restrict__ dvof, const double *__restrict__ ux,
                                                      const double *__restrict__ uy, double *__restrict__ curv,
                                                      int *__restrict__ list, int *__restrict__ count,
                                                      int *__restrict__ flist, int *__restrict__ fcount,
                                                      double *__restrict__ tf, int compact) {
  pdl_entry();
  const size_t cap = (size_t)g.nx * g.ny;
  list += (size_t)blockIdx.z * cap;
  count += (size_t)blockIdx.z * (1);
  if (FACES) {
    flist += (size_t)blockIdx.z * (4 * cap);
    fcount += (size_t)blockIdx.z * (1);
  } else {
    tf += (size_t)blockIdx.z * (kThincTabs * cap);
  }
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const bool in = I <= g.nx && J <= g.ny;
  const int zr = blockIdx.z * g.ny;
  const double2 *dv = reinterpret_cast<const double2 *>(dvof);
  const size_t q = g.p2 / 2;
  bool itf = false, kap = false;  // kap: some corner normal of the cell is not +-0
  unsigned up = 0u;  // faces this cell is upwind of: bit 0 left, 1 right, 2 bottom, 3 top
  if (in) {
    const int r = J - 1 + zr, rp = wrap(J + 1, g.ny) + zr;
    const double2 d00 = dv[(size_t)r * q + (I - 1)], d10 = dv[(size_t)r * q + I];
    const double2 d01 = dv[(size_t)rp * q + (I - 1)], d11 = dv[(size_t)rp * q + I];
    const long long any = dbits(d00.x) | dbits(d00.y) | dbits(d10.x) | dbits(d10.y) | dbits(d01.x) | dbits(d01.y) |
                          dbits(d11.x) | dbits(d11.y);
    kap = (any << 1) != 0;
    if (!kap) curv[ix(g, r, I)] = -0.;
    else if (!compact) cell_curv(g, m, dv, curv, zr, I, J);
    itf = !single_phase(vof[ix(g, r, I)]);
    if (FACES && itf) {
      // upwind tests of update/fluxx.c, fluxy.c; the wall faces belong to k_flux_force
      up |= (I >= 2 && neg(ux[ix(g, r, I - 1)])) ? 1u : 0u;
      up |= (I < g.nx && !neg(ux[ix(g, r, I)])) ? 2u : 0u;
      up |= neg(uy[ix(g, r, I)]) ? 4u : 0u;
      up |= !neg(uy[ix(g, rp, I)]) ? 8u : 0u;
    }
  }
  // block-aggregated appends: per warp (32 consecutive threads of the block,
  // whatever its shape) the ballots of its cells and faces, per block one
  // atomic per list; the order of the entries is free (each is processed on
  // its own)
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = (blockDim.x * blockDim.y + 31) >> 5;
  const int cell = (J - 1) * g.nx + (I - 1);
  const unsigned below = (1u << lane) - 1u;
  const unsigned kmask = __ballot_sync(0xffffffffu, kap);
  const unsigned mask = __ballot_sync(0xffffffffu, itf);
  unsigned fm[4] = {0u, 0u, 0u, 0u};
  int nfw = 0;
  if (FACES) {
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      fm[f] = __ballot_sync(0xffffffffu, (up >> f) & 1u);
      nfw += __popc(fm[f]);
    }
  }
  // per warp: its interface cell / face / curvature cell count, then its
  // offset in the block (lists) or among the block's curvature cells
  __shared__ int wofs[3][BX * BY / 32];
  __shared__ int bbase[3], btot[3];
  __shared__ int klist[BX * BY];
  __shared__ int ilocal[FACES ? 1 : BX * BY];
  if (lane == 0) {
    wofs[0][warp] = __popc(mask);
    wofs[1][warp] = nfw;
    wofs[2][warp] = __popc(kmask);
  }
  __syncthreads();
  if (tid < 3) {
    int run = 0;
    for (int w = 0; w < nwarp; ++w) {
      const int c = wofs[tid][w];
      wofs[tid][w] = run;
      run += c;
    }
    btot[tid] = run;
    bbase[tid] = tid == 2 ? run : (run ? atomicAdd(tid == 0 ? count : fcount, run) : 0);
  }
  __syncthreads();
  const int ipos = wofs[0][warp] + __popc(mask & below);  // this cell's place among the block's interface cells
  if (itf) list[bbase[0] + ipos] = cell;
  if (FACES) {
    int fo = bbase[1] + wofs[1][warp];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      if ((up >> f) & 1u) flist[fo + __popc(fm[f] & below)] = 4 * cell + f;
      fo += __popc(fm[f]);
    }
  } else if (itf) {
    ilocal[ipos] = tid;
  }
  // compacted curvature: the cells with a corner normal lie in the THINC
  // tails, often a few to a warp (the prefix of their counts came with the
  // lists' above)
  if (compact && kap) klist[wofs[2][warp] + __popc(kmask & below)] = tid;
  if (!FACES || compact) __syncthreads();  // uniform over the block
  if (compact && tid < bbase[2]) {
    const int sy = klist[tid] / blockDim.x, sx = klist[tid] - sy * blockDim.x;
    cell_curv(g, m, dv, curv, zr, blockIdx.x * blockDim.x + sx + 1, blockIdx.y * blockDim.y + sy + 1);
  }
  // the THINC factors of the block's interface cells
  if (!FACES && tid < btot[0]) {
    const int c = ilocal[tid];
    const int sy = c / blockDim.x, sx = c - sy * blockDim.x;
    const int Ic = blockIdx.x * blockDim.x + sx + 1, Jc = blockIdx.y * blockDim.y + sy + 1;
    cell_thinc_factors(g, m, dv, vof, zr, Ic, Jc, tf, cap, (Jc - 1) * g.nx + (Ic - 1));
  }
}

__global__ void __launch_bounds__(256)
    k_interface_cells(Grid g, Metrics m, const double *__restrict__ ux, const double *__restrict__ uy,
                      const double *__restrict__ vof, const double *__restrict__ dvof, const int *__restrict__ flist,
                      const int *__restrict__ fcount, double *__restrict__ fluxx, double *__restrict__ fluxy) {
  pdl_entry();
  flist += (size_t)blockIdx.z * (4 * (size_t)g.nx * g.ny);
  fcount += (size_t)blockIdx.z * (1);
  const int n = *fcount;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const double2 *dv = reinterpret_cast<const double2 *>(dvof);
  // one thread per upwind face of an interface cell: every thread runs the
  // same instructions (no face branches)
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int code = flist[t];
    const int id = code >> 2, f = code & 3;
    const int r0 = id / g.nx, I = id - r0 * g.nx + 1;
    const int J = r0 + 1, r = r0 + zr, rp = wrap(J + 1, g.ny) + zr;
    double n0, n1, K;
    cell_normal_k(g, m, dv, vof, zr, I, J, n0, n1, K);
    // face f: 0 left (x face I), 1 right (x face I + 1), 2 bottom (y face J - 1/2), 3 top (J + 1/2)
    const bool xf = f < 2;
    const double na = xf ? n0 : n1, nb = xf ? n1 : n0;
    const double ena = (f & 1) ? -na : na;  // -2 n_a s with s = -1/2 (left, bottom) or +1/2
    const size_t at = xf ? ix(g, r, I - 1 + f) : ix(g, f == 2 ? r : rp, I);
    const double vel = xf ? ux[at] : uy[at];
    const double fl = vel * thinc_face(ena, nb, K);
    if (xf)
      fluxx[at] = fl;
    else
      fluxy[at] = fl;
  }
}

// ---------------------------------------------------------------------------
// vof source (flux divergence), RK update and vof boundaries
//   src/interface/update/main.c:54-136, src/interface/boundary.c:15-42
//   src = (F_x(i) - F_x(i+1)) / HXXC + (F_y(j) - F_y(j+1)) / hy
// FUSED additionally writes rho^{k+1} (src/fluid/density.c) and the mass
// fluxes u + (rho_r - 1) flux into separate buffers
// (src/interface/mass_flux.c:10-58).  OUT: vof^{k+1} goes to vof_out
// (the geometry-ahead step, whose side stream still reads vof^k), else in
// place.
// thread (I, J): I = 1..nx
// ---------------------------------------------------------------------------
template <bool FUSED, bool OUT>
__global__ void __launch_bounds__(BX *BY)
    k_vof_advance(Grid g, Metrics m, Phys ph0, const double *__restrict__ sc, int k, double *vof, double *vof_out,
                  const double *__restrict__ fluxx, const double *__restrict__ fluxy, double *__restrict__ src_a,
                  const double *__restrict__ src_b, const double *__restrict__ ux, const double *__restrict__ uy,
                  double *__restrict__ mfx, double *__restrict__ mfy, double *__restrict__ den1) {
  pdl_entry();
  const Phys ph = zphys(g, ph0);
  sc += (size_t)blockIdx.z * (kScalars);
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rp = wrap(J + 1, g.ny) + zr;
  const double fxm = fluxx[ix(g, r, I - 1)], fxp = fluxx[ix(g, r, I)];
  const double fym = fluxy[ix(g, r, I)], fyp = fluxy[ix(g, rp, I)];
  const double s = fma(m.ihxxc[I], fxm - fxp, g.ihy * (fym - fyp));
  src_a[ix(g, r, I - 1)] = s;
  double v = vof[ix(g, r, I)];
  v = fma(sc[sc_adt(k)], s, v);
  if (k != 0) v = fma(sc[sc_bdt(k)], src_b[ix(g, r, I - 1)], v);
  double *vo = OUT ? vof_out : vof;
  vo[ix(g, r, I)] = v;
  if (I == 1) vo[ix(g, r, 0)] = 0.;
  if (I == g.nx) vo[ix(g, r, g.nx + 1)] = 0.;
  if (FUSED) {
    const double c = ph.dm1;
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

// one thread per face of a listed interface cell (four per cell, face f = 0
// left, 1 right, 2 bottom, 3 top): the upwind test of update/fluxx.c and
// fluxy.c, then, where the cell is upwind of the face, its THINC flux from
// the cell's factors (k_curv_list<false>, tables by cell index) into fluxx /
// fluxy.  The wall faces carry no flux.  Each block takes a contiguous share
// of the entries, so that every SM gets some.
__global__ void __launch_bounds__(256)
    k_face_flux(Grid g, const double *__restrict__ ux, const double *__restrict__ uy, const int *__restrict__ list,
                const int *__restrict__ count, const double *__restrict__ tf, double *__restrict__ fluxx,
                double *__restrict__ fluxy) {
  pdl_entry();
  const size_t cap = (size_t)g.nx * g.ny;
  list += (size_t)blockIdx.z * cap;
  count += (size_t)blockIdx.z * (1);
  tf += (size_t)blockIdx.z * (kThincTabs * cap);
  const int n4 = 4 * *count;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int per = ((n4 + (int)gridDim.x - 1) / (int)gridDim.x + 31) & ~31;
  const int t0 = blockIdx.x * per, t1 = min(n4, t0 + per);
  for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const int f = t & 3;
    const int id = list[t >> 2];
    const int r0 = id / g.nx, I = id - r0 * g.nx + 1;
    const int J = r0 + 1, r = r0 + zr, rp = wrap(J + 1, g.ny) + zr;
    const bool xf = f < 2;
    const size_t at = xf ? ix(g, r, I - 1 + f) : ix(g, f == 2 ? r : rp, I);
    const double vel = xf ? ux[at] : uy[at];
    const bool up = f == 0 ? (I >= 2 && neg(vel)) : (f == 1 ? (I < g.nx && !neg(vel)) : (f == 2 ? neg(vel) : !neg(vel)));
    if (!up) continue;
    const double fl = vel * thinc_ab(tf[f * cap + id], tf[(4 + (f >> 1)) * cap + id]);
    if (xf)
      fluxx[at] = fl;
    else
      fluxy[at] = fl;
  }
}

// vof flux -> mass flux in place (src/interface/mass_flux.c:10-58); I = 0..nx+1
__global__ void k_mass_flux(Grid g, Phys ph, const double *__restrict__ ux, const double *__restrict__ uy,
                            double *__restrict__ fluxx, double *__restrict__ fluxy) {
  pdl_entry();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int r = J - 1;
  const double c = ph.denr - 1.;
  if (I >= 1) fluxx[ix(g, r, I - 1)] = fma(c, fluxx[ix(g, r, I - 1)], ux[ix(g, r, I - 1)]);
  fluxy[ix(g, r, I)] = fma(c, fluxy[ix(g, r, I)], uy[ix(g, r, I)]);
}

// ---------------------------------------------------------------------------
// viscous stress tensor: txx, tyy at centres, txy at corners
//   src/fluid/predict/txx.c:11-40, txy.c:13-50, tyy.c:10-38
//   txx = 2 mu du/dx = (mu_l + mu_r) (u_r - u_l) / HXXC, likewise tyy;
//   txy = 0.5 (mu_s + mu_n) du/dy + 0.5 (mu_w + mu_e) dv/dx
// thread (I, J): I = 1..nx+1
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BX *BY)
    k_stress(Grid g, Metrics m, const double *__restrict__ ux, const double *__restrict__ uy,
             const double *__restrict__ visux, const double *__restrict__ visuy, double *__restrict__ txx,
             double *__restrict__ txy, double *__restrict__ tyy) {
  pdl_entry();
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr, rp = wrap(J + 1, g.ny) + zr;
  const double u0 = ux[ix(g, r, I - 1)];
  const double vx0 = visux[ix(g, r, I - 1)];
  const double w0 = uy[ix(g, r, I)];
  const double vy0 = visuy[ix(g, r, I)];
  if (I <= g.nx) {
    txx[ix(g, r, I - 1)] = (vx0 + visux[ix(g, r, I)]) * ((ux[ix(g, r, I)] - u0) * m.ihxxc[I]);
    tyy[ix(g, r, I - 1)] = (vy0 + visuy[ix(g, rp, I)]) * ((uy[ix(g, rp, I)] - w0) * g.ihy);
  }
  const double sx = visux[ix(g, rm, I - 1)] + vx0;
  const double sy = visuy[ix(g, r, I - 1)] + vy0;
  const double lxy = (u0 - ux[ix(g, rm, I - 1)]) * g.hihy;
  const double lyx = (w0 - uy[ix(g, r, I - 1)]) * m.hihxxf[I];
  txy[ix(g, r, I - 1)] = fma(sx, lxy, sy * lyx);
}

// ---------------------------------------------------------------------------
// momentum right-hand sides and the RK predictor
//   ux: src/fluid/predict/ux.c:29-273, uy: src/fluid/predict/uy.c:29-251,
//   src/fluid/predict/main.c:9-80, walls: src/fluid/boundary/ux.c, uy.c
// With JD = H hy the ux terms reduce to
//   adv_x = 0.25 / HXXF(i) [(F_i + F_i+1)(u_i + u_i+1) - (F_i-1 + F_i)(u_i-1 + u_i)]
//   adv_y = 0.25 HXXC / (HXXF(i) hy) [(G_j+1 sums)(u_j + u_j+1) - (G_j sums)(u_j-1 + u_j)]
//   dif_x = nu / HXXF(i) (txx_i - txx_i-1),  dif_y = nu / hy (txy_j+1 - txy_j)
// and the uy terms likewise with HXXC in place of HXXF.
// This is the fine-grained entry point's form (fluid_predict_field returns
// txx, txy, tyy and the sources); the fused step uses k_momflux and
// k_predict_mf below, the same terms with every flux formed once.
// thread (I, J): I = 1..nx handles the ux face I (I >= 2) and the uy face
// (I, J - 1/2)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BX *BY)
    k_predict(Grid g, Metrics m, Phys ph0, const double *__restrict__ sc, int k, const double *__restrict__ ux,
              const double *__restrict__ uy, double *__restrict__ ux_out, double *__restrict__ uy_out,
              const double *__restrict__ mfx, const double *__restrict__ mfy, const double *__restrict__ txx,
              const double *__restrict__ txy, const double *__restrict__ tyy, const double *__restrict__ p,
              const double *__restrict__ ifrcx, const double *__restrict__ ifrcy, const double *__restrict__ den0,
              const double *__restrict__ den1, double *__restrict__ sxa, const double *__restrict__ sxb,
              double *__restrict__ sxg, double *__restrict__ sya, const double *__restrict__ syb,
              double *__restrict__ syg) {
  pdl_entry();
  const Phys ph = zphys(g, ph0);
  const double *__restrict__ nuf = m.nuf + (size_t)blockIdx.z * g.cm;
  const double *__restrict__ nuc = m.nuc + (size_t)blockIdx.z * g.cm;
  sc += (size_t)blockIdx.z * (kScalars);
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr, rp = wrap(J + 1, g.ny) + zr;
  // the update is carried as 2u with 2 alpha dt, ... and 1 / (2 rho_face):
  // powers of two, so every rounding is the one of the plain form
  const double adt2 = sc[sc_adt2(k)], bdt2 = sc[sc_bdt2(k)], gdt2 = sc[sc_gdt2(k)];
  const double nuy = ph.nuy;
  // ---- ux at face I
  if (I >= 2) {
    const double fx0 = mfx[ix(g, r, I - 1)];
    const double u0 = ux[ix(g, r, I - 1)];
    const double sxm = mfx[ix(g, r, I - 2)] + fx0, sxp = fx0 + mfx[ix(g, r, I)];
    const double um = ux[ix(g, r, I - 2)] + u0, up = u0 + ux[ix(g, r, I)];
    const double sym = mfy[ix(g, r, I - 1)] + mfy[ix(g, r, I)];
    const double syp = mfy[ix(g, rp, I - 1)] + mfy[ix(g, rp, I)];
    const double vm = ux[ix(g, rm, I - 1)] + u0, vp = u0 + ux[ix(g, rp, I - 1)];
    double a = ifrcx[ix(g, r, I - 2)];
    const double rho0 = den0[ix(g, r, I - 1)] + den0[ix(g, r, I)];  // 2 rho^k
    a = fma(ph.hgrav, rho0, a);
    a = fma(nuf[I], txx[ix(g, r, I - 1)] - txx[ix(g, r, I - 2)], a);
    a = fma(nuy, txy[ix(g, rp, I - 1)] - txy[ix(g, r, I - 1)], a);
    a = fma(-m.q4f[I], fma(sxp, up, -sxm * um), a);
    a = fma(-m.q4fy[I], fma(syp, vp, -sym * vm), a);
    const double gs = (p[ix(g, r, I - 1)] - p[ix(g, r, I)]) * m.ihxxf[I];
    const double ir2 = rcp_nr(den1[ix(g, r, I - 1)] + den1[ix(g, r, I)]);  // 1 / (2 rho^{k+1})
    double u = fma(adt2, a, rho0 * u0);
    if (k != 0) u = fma(bdt2, sxb[ix(g, r, I - 2)], u);
    u = fma(gdt2, gs, u);
    ux_out[ix(g, r, I - 1)] = u * ir2;
    sxa[ix(g, r, I - 2)] = a;
    if (sxg) sxg[ix(g, r, I - 2)] = gs;
  }
  // ---- uy at face (I, J - 1/2)
  {
    const double w0 = uy[ix(g, r, I)];
    const double sxm = mfx[ix(g, rm, I - 1)] + mfx[ix(g, r, I - 1)];
    const double sxp = mfx[ix(g, rm, I)] + mfx[ix(g, r, I)];
    const double um = uy[ix(g, r, I - 1)] + w0, up = w0 + uy[ix(g, r, I + 1)];
    const double f0 = mfy[ix(g, r, I)];
    const double sym = mfy[ix(g, rm, I)] + f0, syp = f0 + mfy[ix(g, rp, I)];
    const double vm = uy[ix(g, rm, I)] + w0, vp = w0 + uy[ix(g, rp, I)];
    double a = ifrcy[ix(g, r, I - 1)];
    a = fma(nuc[I], txy[ix(g, r, I)] - txy[ix(g, r, I - 1)], a);
    a = fma(nuy, tyy[ix(g, r, I - 1)] - tyy[ix(g, rm, I - 1)], a);
    a = fma(-m.q4c[I], fma(sxp, up, -sxm * um), a);
    a = fma(-g.q4y, fma(syp, vp, -sym * vm), a);
    const double gs = (p[ix(g, rm, I)] - p[ix(g, r, I)]) * g.ihy;
    const double rho0 = den0[ix(g, rm, I)] + den0[ix(g, r, I)];  // 2 rho^k
    const double ir2 = rcp_nr(den1[ix(g, rm, I)] + den1[ix(g, r, I)]);
    double u = fma(adt2, a, rho0 * w0);
    if (k != 0) u = fma(bdt2, syb[ix(g, r, I - 1)], u);
    u = fma(gdt2, gs, u);
    uy_out[ix(g, r, I)] = u * ir2;
    sya[ix(g, r, I - 1)] = a;
    if (syg) syg[ix(g, r, I - 1)] = gs;
  }
  // walls: impermeable, no-slip
  if (I == 1) {
    ux_out[ix(g, r, 0)] = 0.;
    uy_out[ix(g, r, 0)] = 0.;
  }
  if (I == g.nx) {
    ux_out[ix(g, r, g.nx)] = 0.;
    uy_out[ix(g, r, g.nx + 1)] = 0.;
  }
}

// ---------------------------------------------------------------------------
// momentum fluxes of the fused step, one per centre and corner
//   src/fluid/predict/ux.c:29-144, uy.c:29-130 (advective and diffusive
//   terms), txx.c:11-40, txy.c:13-50, tyy.c:10-38 (the stress components)
// The reference's advective term of ux at face i is a difference of products
// at the two neighbouring cell centres (along x) and corners (along y), and
// its diffusive term a difference of txx and txy at the same points; k_predict
// forms each product twice, once for each face it borders.  Here each point
// gets its flux once, scaled by 4 so that the 1/4 of the face averages
// moves into the face coefficient:
//   centre (I, J):     Pxx = 4 nu txx - (mfx_I + mfx_I+1) (ux_I + ux_I+1)
//                      Pyy = 4 nu tyy - (mfy_J-1/2 + mfy_J+1/2) (uy_J-1/2 + uy_J+1/2)
//   corner (I, J-1/2): Pxy = 4 nu txy - r_I (mfy_I-1 + mfy_I) (ux_J-1 + ux_J)
//                      Pyx = 4 nu txy - (mfx_J-1 + mfx_J) (uy_I-1 + uy_I)
// (mfx, mfy the mass fluxes, r_I = HXXC / HXXF(I) the metric ratio of the
// reference's y advection of ux).  k_predict_mf then adds, with nu / H =
// 4 nu (0.25 / H), the reference's diffusion minus advection
//   ux face I:    0.25 / HXXF(I) (Pxx_I - Pxx_I-1) + 0.25 / hy (Pxy_J+1/2 - Pxy_J-1/2)
//   uy face J-1/2: 0.25 / HXXC(I) (Pyx_I+1 - Pyx_I) + 0.25 / hy (Pyy_J - Pyy_J-1)
// FP64 operations per cell: 29 here (27 with the viscosities pre-scaled)
// and 33 in k_predict_mf (with the Poisson face values it also writes)
// against 16 + 61 for k_stress + k_predict.
// STRESS 1: also txy at the wall columns I = 1, nx + 1 (what the wall-stress
// log reads, src/logging/stress.c); 2: the whole of txx, txy, tyy, in the
// reference's form.  SCALED: visux, visuy come times nuy2 and nuy4
// (k_props<..., true>), so 4 nu txy = sx du + sy dw hy / (2 HXXF) and
// 4 nu tyy = sy dw: two FP64 multiplies per cell fewer (STRESS 0 or 1)
// thread (I, J): I = 1..nx+1 handles the corner (I, J - 1/2) and, for I <= nx,
// the centre (I, J)
// ---------------------------------------------------------------------------
template <int STRESS, bool SCALED>
__global__ void __launch_bounds__(BX *BY)
    k_momflux(Grid g, Metrics m, Phys ph0, const double *__restrict__ ux, const double *__restrict__ uy,
              const double *__restrict__ visux, const double *__restrict__ visuy, const double *__restrict__ mfx,
              const double *__restrict__ mfy, double *__restrict__ pxx, double *__restrict__ pyy,
              double *__restrict__ pxy, double *__restrict__ pyx, double *__restrict__ txx, double *__restrict__ txy,
              double *__restrict__ tyy) {
  pdl_entry();
  const Phys ph = zphys(g, ph0);
  static_assert(!(SCALED && STRESS == 2), "the reference-form stresses take unscaled viscosities");
  const double *__restrict__ c4nuc = SCALED ? m.c4nucs : m.c4nuc + (size_t)blockIdx.z * g.cm;
  const double *__restrict__ c2nuf = SCALED ? m.c2nufs : m.c2nuf + (size_t)blockIdx.z * g.cm;
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr, rp = wrap(J + 1, g.ny) + zr;
  const double u0 = ux[ix(g, r, I - 1)];    // ux at face I, row J
  const double vx0 = visux[ix(g, r, I - 1)];
  const double w0 = uy[ix(g, r, I)];        // uy of cell I at J - 1/2
  const double vy0 = visuy[ix(g, r, I)];
  {
    // corner (I, J - 1/2): txy = 0.5 (mu_s + mu_n) du/dy + 0.5 (mu_w + mu_e) dv/dx
    const double us = ux[ix(g, rm, I - 1)], ww = uy[ix(g, r, I - 1)];
    const double sx = visux[ix(g, rm, I - 1)] + vx0;
    const double sy = visuy[ix(g, r, I - 1)] + vy0;
    const double du = u0 - us, dw = w0 - ww;
    const double t4 = SCALED ? fma(sx, du, sy * (dw * c2nuf[I])) : fma(sx, du * ph.nuy2, sy * (dw * c2nuf[I]));  // 4 nu txy
    const double fy = mfy[ix(g, r, I - 1)] + mfy[ix(g, r, I)];
    const double fx = mfx[ix(g, rm, I - 1)] + mfx[ix(g, r, I - 1)];
    pxy[ix(g, r, I - 1)] = fma(-(m.rq[I] * fy), us + u0, t4);
    pyx[ix(g, r, I - 1)] = fma(-fx, ww + w0, t4);
    if (STRESS == 2 || (STRESS == 1 && (I == 1 || I == g.nx + 1)))
      txy[ix(g, r, I - 1)] = SCALED ? fma(sx, du * (g.hihy * ph.inuy2), sy * (dw * (m.hihxxf[I] * ph.inuy4)))
                                    : fma(sx, du * g.hihy, sy * (dw * m.hihxxf[I]));
  }
  if (I <= g.nx) {
    // centre (I, J): txx = (mu_l + mu_r) du/dx, tyy = (mu_s + mu_n) dv/dy
    const double u1 = ux[ix(g, r, I)], w1 = uy[ix(g, rp, I)];
    const double sx = vx0 + visux[ix(g, r, I)], sy = vy0 + visuy[ix(g, rp, I)];
    const double du = u1 - u0, dw = w1 - w0;
    pxx[ix(g, r, I - 1)] = fma(-(mfx[ix(g, r, I - 1)] + mfx[ix(g, r, I)]), u0 + u1, sx * (du * c4nuc[I]));
    pyy[ix(g, r, I - 1)] = fma(-(mfy[ix(g, r, I)] + mfy[ix(g, rp, I)]), w0 + w1, SCALED ? sy * dw : sy * (dw * ph.nuy4));
    if (STRESS == 2) {
      txx[ix(g, r, I - 1)] = sx * (du * m.ihxxc[I]);
      tyy[ix(g, r, I - 1)] = sy * (dw * g.ihy);
    }
  }
}

// ---------------------------------------------------------------------------
// momentum right-hand sides and the RK predictor of the fused step, from the
// fluxes of k_momflux (the terms of k_predict, same discretisation)
//   src/fluid/predict/ux.c:146-273, uy.c:132-251, main.c:9-80
// Also stores, at both faces, e grad psi_old with e = rho_ref / rho^{k+1} - 1
// and psi_old the potential of the previous substage: the variable-density
// term of the Poisson right-hand side (src/fluid/compute_potential.c:
// 285-363) and of the velocity correction (src/fluid/correct_velocity/ux.c:
// 18-66, uy.c:17-64) is the same face quantity, so both read it from here.
// CACHED: 2 rho^k at the faces is the 2 rho^{k+1} the previous substage's
// predictor formed (srx, sry, which this one overwrites with its own), and
// psi_old's differences across the faces are the ones the previous
// substage's correction formed (dpx, dpy); else both come from den0 and
// psio (first substage of a step whose state may be new).  The same values
// either way.
// thread (I, J): I = 1..nx handles the ux face I (I >= 2) and the uy face
// (I, J - 1/2)
// ---------------------------------------------------------------------------
template <bool CACHED>
__global__ void __launch_bounds__(BX *BY)
    k_predict_mf(Grid g, Metrics m, Phys ph0, const double *__restrict__ sc, int k, const double *__restrict__ ux,
                 const double *__restrict__ uy, double *__restrict__ ux_out, double *__restrict__ uy_out,
                 const double *__restrict__ pxx, const double *__restrict__ pyy, const double *__restrict__ pxy,
                 const double *__restrict__ pyx, const double *__restrict__ p, const double *__restrict__ ifrcx,
                 const double *__restrict__ ifrcy, const double *__restrict__ den0, const double *__restrict__ den1,
                 const double *__restrict__ psio, double *__restrict__ sxa, const double *__restrict__ sxb,
                 double *__restrict__ sya, const double *__restrict__ syb, double *__restrict__ egx,
                 double *__restrict__ egy, const double *__restrict__ coltab, double *__restrict__ qx,
                 double *__restrict__ qy, double *__restrict__ srx, double *__restrict__ sry,
                 const double *__restrict__ dpx, const double *__restrict__ dpy) {
  pdl_entry();
  sc += (size_t)blockIdx.z * (kScalars);
  const double *__restrict__ gx = coltab + ((size_t)blockIdx.z * 3 * kColTabs + ct_gdt2x(k)) * g.ct;
  // the Poisson right-hand side's face values q = pd u* + pa e grad psi_old
  // (k_poisson_fwd<W, true> takes their differences across each cell)
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr, rp = wrap(J + 1, g.ny) + zr;
  // the update is carried as 2u with 2 alpha dt, ... and 1 / (2 rho_face):
  // powers of two, so every rounding is the one of the plain form; the
  // pressure term's 2 gamma dt / H comes per column (gx) or per case
  const double adt2 = sc[sc_adt2(k)], bdt2 = sc[sc_bdt2(k)];
  const Phys ph = zphys(g, ph0);
  // e grad psi_old is stored times the Poisson factor pax (x faces) or pay
  // (y faces): e pa = (2 rho_ref pa) / (2 rho) - pa
  const double rpx = sc[sc_rpx(k)], pax = sc[sc_pax(k)];
  const double ps0 = CACHED && I != 1 && I != g.nx ? 0. : psio[ix(g, r, I)];
  // ---- ux at face I
  if (I >= 2) {
    const double u0 = ux[ix(g, r, I - 1)];
    double a = ifrcx[ix(g, r, I - 2)];
    const double rho0 = CACHED ? srx[ix(g, r, I - 1)] : den0[ix(g, r, I - 1)] + den0[ix(g, r, I)];  // 2 rho^k
    a = fma(ph.hgrav, rho0, a);
    a = fma(m.q4f[I], pxx[ix(g, r, I - 1)] - pxx[ix(g, r, I - 2)], a);
    a = fma(g.q4y, pxy[ix(g, rp, I - 1)] - pxy[ix(g, r, I - 1)], a);
    const double rho1 = den1[ix(g, r, I - 1)] + den1[ix(g, r, I)];  // 2 rho^{k+1}
    srx[ix(g, r, I - 1)] = rho1;
    const double ir2 = rcp_nr(rho1);
    double u = fma(adt2, a, rho0 * u0);
    if (k != 0) u = fma(bdt2, sxb[ix(g, r, I - 2)], u);
    u = fma(gx[I], p[ix(g, r, I - 1)] - p[ix(g, r, I)], u);
    const double us = u * ir2;
    ux_out[ix(g, r, I - 1)] = us;
    sxa[ix(g, r, I - 2)] = a;
    const double e = fma(rpx, ir2, -pax) * (CACHED ? dpx[ix(g, r, I - 1)] : ps0 - psio[ix(g, r, I - 1)]);
    egx[ix(g, r, I - 1)] = e;
    qx[ix(g, r, I - 1)] = fma(sc[sc_pdx(k)], us, e);
  }
  // ---- uy at face (I, J - 1/2)
  {
    const double w0 = uy[ix(g, r, I)];
    double a = ifrcy[ix(g, r, I - 1)];
    a = fma(m.q4c[I], pyx[ix(g, r, I)] - pyx[ix(g, r, I - 1)], a);
    a = fma(g.q4y, pyy[ix(g, r, I - 1)] - pyy[ix(g, rm, I - 1)], a);
    const double rho0 = CACHED ? sry[ix(g, r, I)] : den0[ix(g, rm, I)] + den0[ix(g, r, I)];  // 2 rho^k
    const double rho1 = den1[ix(g, rm, I)] + den1[ix(g, r, I)];
    sry[ix(g, r, I)] = rho1;
    const double ir2 = rcp_nr(rho1);
    double u = fma(adt2, a, rho0 * w0);
    if (k != 0) u = fma(bdt2, syb[ix(g, r, I - 1)], u);
    u = fma(sc[sc_gdt2y(k)], p[ix(g, rm, I)] - p[ix(g, r, I)], u);
    const double ws = u * ir2;
    uy_out[ix(g, r, I)] = ws;
    sya[ix(g, r, I - 1)] = a;
    const double e =
        fma(sc[sc_rpy(k)], ir2, -sc[sc_pay(k)]) * (CACHED ? dpy[ix(g, r, I)] : ps0 - psio[ix(g, rm, I)]);
    egy[ix(g, r, I)] = e;
    qy[ix(g, r, I)] = fma(sc[sc_pdy(k)], ws, e);
  }
  // walls: impermeable, no-slip; the wall faces' e grad psi_old (zero for a
  // Neumann psi_old, computed as the reference does)
  if (I == 1) {
    ux_out[ix(g, r, 0)] = 0.;
    uy_out[ix(g, r, 0)] = 0.;
    const double e = fma(rpx, rcp_nr(den1[ix(g, r, 0)] + den1[ix(g, r, 1)]), -pax) * (ps0 - psio[ix(g, r, 0)]);
    egx[ix(g, r, 0)] = e;
    qx[ix(g, r, 0)] = fma(sc[sc_pdx(k)], 0., e);
  }
  if (I == g.nx) {
    ux_out[ix(g, r, g.nx)] = 0.;
    uy_out[ix(g, r, g.nx + 1)] = 0.;
    const double e =
        fma(rpx, rcp_nr(den1[ix(g, r, g.nx)] + den1[ix(g, r, g.nx + 1)]), -pax) * (psio[ix(g, r, g.nx + 1)] - ps0);
    egx[ix(g, r, g.nx)] = e;
    qx[ix(g, r, g.nx)] = fma(sc[sc_pdx(k)], 0., e);
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
//      285-363 for a tile of W columns,
//        rhs = rho_ref/dt_new div u* - dt_old/dt_new div((rho_ref/rho - 1) grad psi_old)
//      (the face values of (rho_ref/rho - 1) grad psi_old come from k_predict_mf,
//      already times their Poisson coefficient; in the fused step the
//      predictor also adds the u* term at each face, so the transform only
//      differences the sums)
//      with div and the face differences in the JD = H hy form, packed two
//      reals per complex, a mixed radix-4/2 Stockham FFT of length ny/2 in
//      shared memory and the real-to-complex split; spectrum [I][m]
//   2. k_poisson_tdm: tridiagonal solves along x (warp-parallel scan)
//   3. k_poisson_inv: inverse of step 1, psi and its Neumann ghosts
// The 1 / ny of the inverse DFT and the 1/2 of the real split are folded
// into the right-hand-side coefficients.
// ---------------------------------------------------------------------------

// Stockham FFT (radix 4, one radix-8 stage first when log2 M is odd) of W
// rows of length M in shared memory.  Returns the buffer holding the result.
// tw: the twiddle buffer, exp(-2 pi i m / 2M) for m = 0..M, then W_M^e for
// e < M, then their conjugates (the inverse's): one load per twiddle.
template <int W>
__device__ double2 *fft_rows(double2 *x, double2 *y, int M, const double2 *__restrict__ tw, bool inverse) {
  const double2 *__restrict__ wm = tw + (M + 1) + (inverse ? M : 0);
  int Ns = 1;
  if ((__ffs(M) - 1) & 1) {  // log2 M odd (M >= 8): an untwiddled radix-8 stage
    // X_2m = DFT4(v_q + v_q+4)_m, X_2m+1 = DFT4((v_q - v_q+4) W8^q)_m; the
    // 1/sqrt(2) of W8 and W8^3 rides in the odd half's last FMAs: 52 FP64
    // operations for 8 points, where a radix-2 stage and a twiddled radix-4
    // stage take 64 for the same three levels
    const double c8 = 0.70710678118654752440;
    const int q8 = M >> 3;
    for (int t = threadIdx.x; t < W * q8; t += blockDim.x) {
      const int c = t / q8, j = t - c * q8;
      const double2 *xr = x + c * M;
      double2 *yr = y + c * M + 8 * j;
      double2 a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double2 u = xr[j + q * q8], w = xr[j + (q + 4) * q8];
        a[q] = cadd(u, w);
        b[q] = csub(u, w);
      }
      // even outputs: DFT4 of a; -i (forward) or +i (inverse) rotations are sign flips
      const double2 e0 = cadd(a[0], a[2]), e1 = csub(a[0], a[2]), e2 = cadd(a[1], a[3]), e3 = csub(a[1], a[3]);
      const double2 re3 = inverse ? make_double2(-e3.y, e3.x) : make_double2(e3.y, -e3.x);
      yr[0] = cadd(e0, e2);
      yr[2] = cadd(e1, re3);
      yr[4] = csub(e0, e2);
      yr[6] = csub(e1, re3);
      // odd outputs: t1 = b1 W8 = c8 P1, t2 = b2 W8^2 (a rotation), t3 = b3 W8^3 = c8 P3
      const double2 P1 = inverse ? make_double2(b[1].x - b[1].y, b[1].x + b[1].y)
                                 : make_double2(b[1].x + b[1].y, b[1].y - b[1].x);
      const double2 P3 = inverse ? make_double2(-(b[3].x + b[3].y), b[3].x - b[3].y)
                                 : make_double2(b[3].y - b[3].x, -(b[3].x + b[3].y));
      const double2 t2 = inverse ? make_double2(-b[2].y, b[2].x) : make_double2(b[2].y, -b[2].x);
      const double2 A0 = cadd(b[0], t2), A1 = csub(b[0], t2);
      const double2 E = cadd(P1, P3), D = csub(P1, P3);  // t1 + t3 = c8 E, t1 - t3 = c8 D
      const double2 rD = inverse ? make_double2(-D.y, D.x) : make_double2(D.y, -D.x);
      yr[1] = make_double2(fma(c8, E.x, A0.x), fma(c8, E.y, A0.y));
      yr[3] = make_double2(fma(c8, rD.x, A1.x), fma(c8, rD.y, A1.y));
      yr[5] = make_double2(fma(-c8, E.x, A0.x), fma(-c8, E.y, A0.y));
      yr[7] = make_double2(fma(-c8, rD.x, A1.x), fma(-c8, rD.y, A1.y));
    }
    __syncthreads();
    double2 *tmp = x;
    x = y;
    y = tmp;
    Ns = 8;
  }
  const int q4 = M >> 2;
  for (; Ns < M; Ns <<= 2) {
    const int step = M / (4 * Ns);
    for (int t = threadIdx.x; t < W * q4; t += blockDim.x) {
      const int c = t / q4, j = t - c * q4;
      const double2 *xr = x + c * M;
      double2 *yr = y + c * M;
      const int kk = j & (Ns - 1);
      const double2 v0 = xr[j], v1 = xr[j + q4], v2 = xr[j + 2 * q4], v3 = xr[j + 3 * q4];
      double2 a0, a1, a2, a3;
      if (Ns > 1) {
        // a0 = v0 + w2 v2 and a2 = w1 v1 + w3 v3 with the products folded into
        // FMAs, a1 = 2 v0 - a0 and a3 = 2 (w1 v1) - a2: 24 FP64 operations per
        // butterfly instead of 28 (cmul, then add and subtract)
        const int e = kk * step;
        const double2 w1 = wm[e], w2 = wm[2 * e], w3 = wm[3 * e];
        a0 = make_double2(fma(w2.x, v2.x, fma(-w2.y, v2.y, v0.x)), fma(w2.x, v2.y, fma(w2.y, v2.x, v0.y)));
        a1 = make_double2(fma(2., v0.x, -a0.x), fma(2., v0.y, -a0.y));
        const double2 t1 = cmul(v1, w1);
        a2 = make_double2(fma(w3.x, v3.x, fma(-w3.y, v3.y, t1.x)), fma(w3.x, v3.y, fma(w3.y, v3.x, t1.y)));
        a3 = make_double2(fma(2., t1.x, -a2.x), fma(2., t1.y, -a2.y));
      } else {
        a0 = cadd(v0, v2);
        a1 = csub(v0, v2);
        a2 = cadd(v1, v3);
        a3 = csub(v1, v3);
      }
      // -i a3 (forward) or +i a3 (inverse)
      const double2 r3 = inverse ? make_double2(-a3.y, a3.x) : make_double2(a3.y, -a3.x);
      const int d = ((j - kk) << 2) + kk;
      yr[d] = cadd(a0, a2);
      yr[d + Ns] = cadd(a1, r3);
      yr[d + 2 * Ns] = csub(a0, a2);
      yr[d + 3 * Ns] = csub(a1, r3);
    }
    __syncthreads();
    double2 *tmp = x;
    x = y;
    y = tmp;
  }
  return x;
}

// Q: the right-hand side from the predictor's face values q = pd u* + pa e
// grad psi_old (ux, uy are qx, qy; egx, egy unused): 3 FP64 operations per
// cell instead of 7
template <int W, bool Q>
__global__ void __launch_bounds__(256)
    k_poisson_fwd(Grid g, const double *__restrict__ sc, int k, const double *__restrict__ ux,
                  const double *__restrict__ uy, const double *__restrict__ egx, const double *__restrict__ egy,
                  const double2 *__restrict__ tw, double2 *__restrict__ spec) {
  pdl_entry();
  sc += (size_t)blockIdx.z * (kScalars);
  spec += (size_t)blockIdx.z * (g.css);
  extern __shared__ double2 smem[];
  const int ny = g.ny, M = ny >> 1;
  double2 *A = smem, *B = smem + W * M;
  double *Ad = reinterpret_cast<double *>(A);
  const int I0 = blockIdx.x * W + 1;
  const double pdx = sc[sc_pdx(k)], pdy = sc[sc_pdy(k)];
  for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
    const int c = t % W, r = t / W;
    const int I = I0 + c;
    double val = 0.;
    if (I <= g.nx) {
      // global rows of this case (the case's rows follow each other)
      const int zr = blockIdx.z * ny;
      const int rg = r + zr, rp = (r == ny - 1 ? 0 : r + 1) + zr;
      // differences of pax e grad psi_old and pay e grad psi_old across the
      // cell (its faces' values written by k_predict_mf or k_face_factor)
      if (Q) {
        val = (ux[ix(g, rg, I)] - ux[ix(g, rg, I - 1)]) + (uy[ix(g, rp, I)] - uy[ix(g, rg, I)]);
      } else {
        const double X = egx[ix(g, rg, I)] - egx[ix(g, rg, I - 1)];
        const double Y = egy[ix(g, rp, I)] - egy[ix(g, rg, I)];
        const double dux = ux[ix(g, rg, I)] - ux[ix(g, rg, I - 1)];
        const double duy = uy[ix(g, rp, I)] - uy[ix(g, rg, I)];
        val = fma(pdx, dux, fma(pdy, duy, X + Y));
      }
    }
    Ad[c * ny + r] = val;
  }
  __syncthreads();
  double2 *Z = fft_rows<W>(A, B, M, tw, false);
  // the packed transform z_m, m < M; k_poisson_tdm does the real-to-complex
  // split (there the FP64 pipe has room)
  const int M1 = M + 1;
  for (int t = threadIdx.x; t < W * M; t += blockDim.x) {
    const int c = t / M, mm = t - c * M;
    const int I = I0 + c;
    if (I > g.nx) continue;
    spec[(size_t)(I - 1) * M1 + mm] = Z[c * M + mm];
  }
}

template <int W>
__global__ void __launch_bounds__(256)
    k_poisson_inv(Grid g, const double2 *__restrict__ tw, const double2 *__restrict__ spec, double *__restrict__ psi) {
  pdl_entry();
  spec += (size_t)blockIdx.z * (g.css);
  extern __shared__ double2 smem[];
  const int ny = g.ny, M = ny >> 1, M1 = M + 1;
  double2 *A = smem, *B = smem + W * M;
  const int I0 = blockIdx.x * W + 1;
  for (int t = threadIdx.x; t < W * M; t += blockDim.x) {
    const int c = t / M, mm = t - c * M;
    const int I = I0 + c;
    // the packed input of the inverse transform, complex-to-real split done
    // by k_poisson_tdm
    A[c * M + mm] = I <= g.nx ? spec[(size_t)(I - 1) * M1 + mm] : make_double2(0., 0.);
  }
  __syncthreads();
  const double2 *zr = fft_rows<W>(A, B, M, tw, true);
  const double *xd = reinterpret_cast<const double *>(zr);
  for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
    const int c = t % W, r = t / W;
    const int I = I0 + c;
    if (I > g.nx) continue;
    const double v = xd[c * ny + r];
    const int rg = r + (int)blockIdx.z * ny;
    psi[ix(g, rg, I)] = v;
    if (I == 1) psi[ix(g, rg, 0)] = v;
    if (I == g.nx) psi[ix(g, rg, g.nx + 1)] = v;
  }
}

// Tridiagonal solves along x, one per real system (y wavenumber m, real or
// imaginary part), one warp per system.  The pivots of the constant operator
// are precomputed, so the Thomas forward sweep is the first-order linear
// recurrence y_i = w_i r_i - v_i y_{i-1} and the back substitution is
// x_i = y_i - v_i x_{i+1}.  Lane l owns the L consecutive rows l*L..l*L+L-1:
// it runs both recurrences on its rows from a zero carry, the lanes combine
// their chunk maps (T, B): y -> T + B y with a shuffle scan, and each row is
// fixed up with the precomputed cumulative products P_i (forward) and Q_i
// (backward) of the recurrence coefficients inside its chunk.  Per row: 5
// FP64 operations instead of the 3 of a sequential sweep, but 32-way
// parallel per system.  fac[(m*L + k)*32 + l] = (w, v, P, Q) for row l*L+k.
// The singular m = 0 mode (Neumann in x, constant null space) has its last
// pivot pinned (w = v = 0) and is shifted to zero mean.
// Staging: per system a planar array with an odd lane stride S, in shared
// memory; when four systems of nx rows exceed it (nx above about 6900), in
// this block's slab of the global buffer stage (L2-resident, same arithmetic).
template <bool kGlobalStage>
__global__ void __launch_bounds__(512)
    k_poisson_tdm(Grid g, int PB, int G, int L, int S, const double4_32a *__restrict__ fac,
                  const double2 *__restrict__ tw, double2 *__restrict__ spec, double *__restrict__ stage) {
  pdl_entry();
  extern __shared__ double2 smem_d2[];
  __shared__ double xch[16][4][2];  // per system of the block, per warp of the system: a chunk-map total
  const int nx = g.nx, M = g.ny / 2, M1 = M + 1;
  const int p0 = blockIdx.x * PB;
  const int np = min(PB, M / 2 + 1 - p0);  // pairs (p, M - p), p = 0 .. M/2
  const int lanes = 32 * G;                // chunks per system
  const int sys_len = lanes * S;
  double *sm = kGlobalStage ? stage + ((size_t)blockIdx.z * gridDim.x + blockIdx.x) * 4 * PB * sys_len
                            : reinterpret_cast<double *>(smem_d2);
  double2 *sp = spec + (size_t)blockIdx.z * g.css;
  // ---- load the packed transform of both wavenumbers of each pair, split
  // it (real-to-complex, times 2: X_m = (z_m + conj z_{M-m}) + w^m (-i)(z_m -
  // conj z_{M-m})) into four planar systems: X_p re, im, X_{M-p} re, im
  for (int t = threadIdx.x; t < lanes * L * np; t += blockDim.x) {
    const int i = t / np, q = t - i * np;
    const int p = p0 + q;
    const int at = (i / L) * S + (i % L);
    double2 xa = make_double2(0., 0.), xb = make_double2(0., 0.);
    if (i < nx) {
      const double2 zm = sp[(size_t)i * M1 + p];
      const double2 zr = sp[(size_t)i * M1 + (p == 0 ? 0 : M - p)];
      const double2 E = make_double2(zm.x + zr.x, zm.y - zr.y);
      const double2 O = make_double2(zm.y + zr.y, zr.x - zm.x);  // -i (zm - conj zr)
      // X_p = E + w^p O; X_{M-p} = conj E + w^{M-p} conj O (the pair's E and O
      // with the signs of their imaginary parts flipped), products in FMAs
      const double2 wa = tw[p], wb = tw[M - p];
      xa = make_double2(fma(wa.x, O.x, fma(-wa.y, O.y, E.x)), fma(wa.x, O.y, fma(wa.y, O.x, E.y)));
      xb = make_double2(fma(wb.x, O.x, fma(wb.y, O.y, E.x)), fma(wb.y, O.x, fma(-wb.x, O.y, -E.y)));
    }
    sm[(4 * q) * sys_len + at] = xa.x;
    sm[(4 * q + 1) * sys_len + at] = xa.y;
    sm[(4 * q + 2) * sys_len + at] = xb.x;
    sm[(4 * q + 3) * sys_len + at] = xb.y;
  }
  __syncthreads();
  // warp -> system (4 per pair) and its part sub of G; chunk j of the
  // system = this lane's L rows
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sys = warp / G, sub = warp - sys * G, j = sub * 32 + lane;
  const bool act = sys < 4 * np;  // warp-uniform
  const int pq = p0 + (sys >> 2);
  const int m = (sys & 2) ? M - pq : pq;  // the wavenumber of this system
  double *x = sm + sys * sys_len + j * S;
  const double4_32a *f = fac + (size_t)m * L * lanes + j;
  double T = 0., B = 0.;
  if (act) {
    // forward, local from a zero carry
    double t = 0.;
#pragma unroll 8
    for (int k = 0; k < L; ++k) {
      const double4_32a c = f[(size_t)k * lanes];
      t = fma(-c.y, t, c.x * x[k]);
      x[k] = t;
    }
    T = t;
    B = f[(size_t)(L - 1) * lanes].z;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double Tp = __shfl_up_sync(0xffffffffu, T, d), Bp = __shfl_up_sync(0xffffffffu, B, d);
      if (lane >= d) {
        T = fma(B, Tp, T);
        B *= Bp;
      }
    }
  }
  // the map of the system's chunks before this warp's (G > 1: warp totals)
  double Cin = 0.;
  if (G > 1) {
    if (act && lane == 31) {
      xch[sys][sub][0] = T;
      xch[sys][sub][1] = B;
    }
    __syncthreads();
    if (act)
      for (int q = 0; q < sub; ++q) Cin = fma(xch[sys][q][1], Cin, xch[sys][q][0]);
    __syncthreads();
  }
  double Sx = 0., Cc = 0.;
  if (act) {
    const double Tu = __shfl_up_sync(0xffffffffu, T, 1), Bu = __shfl_up_sync(0xffffffffu, B, 1);
    const double carry = lane == 0 ? Cin : fma(Bu, Cin, Tu);
    // fix up the forward solution, then the backward sweep from a zero carry
    double u = 0.;
#pragma unroll 8
    for (int k = L - 1; k >= 0; --k) {
      const double4_32a c = f[(size_t)k * lanes];
      const double y = fma(c.z, carry, x[k]);
      u = fma(-c.y, u, y);
      x[k] = u;
    }
    Sx = u;
    Cc = f[0].w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double Sp = __shfl_down_sync(0xffffffffu, Sx, d), Cp = __shfl_down_sync(0xffffffffu, Cc, d);
      if (lane + d < 32) {
        Sx = fma(Cc, Sp, Sx);
        Cc *= Cp;
      }
    }
  }
  // the map of the chunks after this warp's
  double Din = 0.;
  if (G > 1) {
    if (act && lane == 0) {
      xch[sys][sub][0] = Sx;
      xch[sys][sub][1] = Cc;
    }
    __syncthreads();
    if (act)
      for (int q = G - 1; q > sub; --q) Din = fma(xch[sys][q][1], Din, xch[sys][q][0]);
    __syncthreads();
  }
  // the singular mode m = 0 (systems 0, 1 of pair 0): zero mean over x, imaginary part 0
  const bool gauge = act && m == 0 && (sys & 2) == 0;
  double acc = 0.;
  if (act) {
    const double Sd = __shfl_down_sync(0xffffffffu, Sx, 1), Cd = __shfl_down_sync(0xffffffffu, Cc, 1);
    const double next = lane == 31 ? Din : fma(Cd, Din, Sd);
#pragma unroll 8
    for (int k = 0; k < L; ++k) x[k] = fma(f[(size_t)k * lanes].w, next, x[k]);
    if (gauge) {
      for (int k = 0; k < L; ++k) acc += (j * L + k < nx) ? x[k] : 0.;
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
    }
  }
  if (G > 1) {
    if (gauge && lane == 0) xch[sys][sub][0] = acc;
    __syncthreads();
    if (gauge) {
      acc = 0.;
      for (int q = 0; q < G; ++q) acc += xch[sys][q][0];
    }
  }
  if (gauge) {
    const double mean = (sys & 1) ? 0. : acc / nx;
    for (int k = 0; k < L; ++k) x[k] = (sys & 1) ? 0. : x[k] - mean;
  }
  __syncthreads();
  // ---- complex-to-real split of the solved pair into the packed input of the
  // inverse transform: z_m = E + i O, E = X_m + conj X_{M-m},
  // O = (X_m - conj X_{M-m}) conj w^m, for m = p and m = M - p (< M)
  for (int t = threadIdx.x; t < nx * np; t += blockDim.x) {
    const int i = t / np, q = t - i * np;
    const int p = p0 + q;
    const int at = (i / L) * S + (i % L);
    const double2 Xa = make_double2(sm[(4 * q) * sys_len + at], sm[(4 * q + 1) * sys_len + at]);
    const double2 Xb = make_double2(sm[(4 * q + 2) * sys_len + at], sm[(4 * q + 3) * sys_len + at]);
    // z_p = E + i D conj w^p and z_{M-p} = conj E - i conj D conj w^{M-p}, with
    // E = X_p + conj X_{M-p}, D = X_p - conj X_{M-p}; products in FMAs
    const double2 E = make_double2(Xa.x + Xb.x, Xa.y - Xb.y);
    const double2 D = make_double2(Xa.x - Xb.x, Xa.y + Xb.y);
    const double2 wa = tw[p];
    sp[(size_t)i * M1 + p] =
        make_double2(fma(D.x, wa.y, fma(-D.y, wa.x, E.x)), fma(D.y, wa.y, fma(D.x, wa.x, E.y)));
    if (p != 0 && 2 * p != M) {
      const double2 wb = tw[M - p];
      sp[(size_t)i * M1 + (M - p)] =
          make_double2(fma(-D.y, wb.x, fma(-D.x, wb.y, E.x)), fma(D.y, wb.y, fma(-D.x, wb.x, -E.y)));
    }
  }
}

// The same solves with four warps per system, spread over a cluster of four
// CTAs: CTA r of a cluster owns rows 32 L r .. 32 L (r + 1) - 1 of the four
// systems of one wavenumber pair (warp s: system s), so a launch has four
// CTAs per pair where k_poisson_tdm has one block per pair or two, and the
// 4 (ny/4 + 1) CTAs of a case even out over the SMs (in a launch of blocks
// of one or two pairs, ny/4 + 1 pairs leave SMs idle while the last blocks
// run, one in six for ny = 1024).  The chunk-map totals of
// the other CTAs come through distributed shared memory and are combined in
// the order k_poisson_tdm<false> combines its warps' at G = 4, so both give
// the same bits.  L = tdm_chunk(nx, 4), S = L | 1; fac is the G = 4 table.
constexpr int kTdmCluster = 4;
__global__ void __cluster_dims__(kTdmCluster, 1, 1) __launch_bounds__(128)
    k_poisson_tdm_cl(Grid g, int L, int S, const double4_32a *__restrict__ fac, const double2 *__restrict__ tw,
                     double2 *__restrict__ spec) {
  pdl_entry();
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double smem_cl[];
  // per system: forward (T, B) and backward (S, C) totals of this CTA's warp, the gauge sum
  __shared__ double xf[4][2], xb[4][2], xg[4];
  const int nx = g.nx, M = g.ny / 2, M1 = M + 1;
  const int rank = (int)cl.block_rank();
  const int p = (int)blockIdx.x / kTdmCluster;  // the pair (p, M - p), p = 0 .. M/2
  const int rows = 32 * L, r0 = rank * rows;   // this CTA's rows r0 .. r0 + rows - 1
  const int sys_len = 32 * S;
  double2 *sp = spec + (size_t)blockIdx.z * g.css;
  // ---- load and split (as in k_poisson_tdm), this CTA's rows
  for (int t = threadIdx.x; t < rows; t += blockDim.x) {
    const int i = r0 + t;
    const int at = (t / L) * S + (t % L);
    double2 xa = make_double2(0., 0.), xbv = make_double2(0., 0.);
    if (i < nx) {
      const double2 zm = sp[(size_t)i * M1 + p];
      const double2 zr = sp[(size_t)i * M1 + (p == 0 ? 0 : M - p)];
      const double2 E = make_double2(zm.x + zr.x, zm.y - zr.y);
      const double2 O = make_double2(zm.y + zr.y, zr.x - zm.x);
      const double2 wa = tw[p], wb = tw[M - p];
      xa = make_double2(fma(wa.x, O.x, fma(-wa.y, O.y, E.x)), fma(wa.x, O.y, fma(wa.y, O.x, E.y)));
      xbv = make_double2(fma(wb.x, O.x, fma(wb.y, O.y, E.x)), fma(wb.y, O.x, fma(-wb.x, O.y, -E.y)));
    }
    smem_cl[0 * sys_len + at] = xa.x;
    smem_cl[1 * sys_len + at] = xa.y;
    smem_cl[2 * sys_len + at] = xbv.x;
    smem_cl[3 * sys_len + at] = xbv.y;
  }
  __syncthreads();
  const int sys = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lanes = 32 * kTdmCluster, j = rank * 32 + lane;  // chunk of the system
  const int m = (sys & 2) ? M - p : p;
  double *x = smem_cl + sys * sys_len + lane * S;
  const double4_32a *f = fac + (size_t)m * L * lanes + j;
  double T, B;
  {
    double t = 0.;
#pragma unroll 8
    for (int k = 0; k < L; ++k) {
      const double4_32a c = f[(size_t)k * lanes];
      t = fma(-c.y, t, c.x * x[k]);
      x[k] = t;
    }
    T = t;
    B = f[(size_t)(L - 1) * lanes].z;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double Tp = __shfl_up_sync(0xffffffffu, T, d), Bp = __shfl_up_sync(0xffffffffu, B, d);
      if (lane >= d) {
        T = fma(B, Tp, T);
        B *= Bp;
      }
    }
  }
  if (lane == 31) {
    xf[sys][0] = T;
    xf[sys][1] = B;
  }
  cl.sync();
  double Cin = 0.;
  for (int q = 0; q < rank; ++q) {
    const double *o = cl.map_shared_rank(&xf[sys][0], q);
    Cin = fma(o[1], Cin, o[0]);
  }
  double Sx, Cc;
  {
    const double Tu = __shfl_up_sync(0xffffffffu, T, 1), Bu = __shfl_up_sync(0xffffffffu, B, 1);
    const double carry = lane == 0 ? Cin : fma(Bu, Cin, Tu);
    double u = 0.;
#pragma unroll 8
    for (int k = L - 1; k >= 0; --k) {
      const double4_32a c = f[(size_t)k * lanes];
      const double y = fma(c.z, carry, x[k]);
      u = fma(-c.y, u, y);
      x[k] = u;
    }
    Sx = u;
    Cc = f[0].w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double Sp = __shfl_down_sync(0xffffffffu, Sx, d), Cp = __shfl_down_sync(0xffffffffu, Cc, d);
      if (lane + d < 32) {
        Sx = fma(Cc, Sp, Sx);
        Cc *= Cp;
      }
    }
  }
  if (lane == 0) {
    xb[sys][0] = Sx;
    xb[sys][1] = Cc;
  }
  cl.sync();
  double Din = 0.;
  for (int q = kTdmCluster - 1; q > rank; --q) {
    const double *o = cl.map_shared_rank(&xb[sys][0], q);
    Din = fma(o[1], Din, o[0]);
  }
  {
    const double Sd = __shfl_down_sync(0xffffffffu, Sx, 1), Cd = __shfl_down_sync(0xffffffffu, Cc, 1);
    const double next = lane == 31 ? Din : fma(Cd, Din, Sd);
#pragma unroll 8
    for (int k = 0; k < L; ++k) x[k] = fma(f[(size_t)k * lanes].w, next, x[k]);
  }
  // the singular mode m = 0 (systems 0, 1 of pair 0): zero mean over x,
  // imaginary part 0 (p is the same on the whole cluster)
  if (p == 0) {
    const bool gauge = (sys & 2) == 0;
    double acc = 0.;
    if (gauge) {
      for (int k = 0; k < L; ++k) acc += (j * L + k < nx) ? x[k] : 0.;
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
      if (lane == 0) xg[sys] = acc;
    }
    cl.sync();
    if (gauge) {
      acc = 0.;
      for (int q = 0; q < kTdmCluster; ++q) acc += *cl.map_shared_rank(&xg[sys], q);
      const double mean = (sys & 1) ? 0. : acc / nx;
      for (int k = 0; k < L; ++k) x[k] = (sys & 1) ? 0. : x[k] - mean;
    }
  }
  // no CTA of the cluster reads another's shared memory after this point
  cl.sync();
  // ---- complex-to-real split (as in k_poisson_tdm), this CTA's rows
  for (int t = threadIdx.x; t < rows; t += blockDim.x) {
    const int i = r0 + t;
    if (i >= nx) break;
    const int at = (t / L) * S + (t % L);
    const double2 Xa = make_double2(smem_cl[0 * sys_len + at], smem_cl[1 * sys_len + at]);
    const double2 Xb = make_double2(smem_cl[2 * sys_len + at], smem_cl[3 * sys_len + at]);
    const double2 E = make_double2(Xa.x + Xb.x, Xa.y - Xb.y);
    const double2 D = make_double2(Xa.x - Xb.x, Xa.y + Xb.y);
    const double2 wa = tw[p];
    sp[(size_t)i * M1 + p] =
        make_double2(fma(D.x, wa.y, fma(-D.y, wa.x, E.x)), fma(D.y, wa.y, fma(D.x, wa.x, E.y)));
    if (p != 0 && 2 * p != M) {
      const double2 wb = tw[M - p];
      sp[(size_t)i * M1 + (M - p)] =
          make_double2(fma(-D.y, wb.x, fma(-D.x, wb.y, E.x)), fma(D.y, wb.y, fma(-D.x, wb.x, -E.y)));
    }
  }
}

// ---------------------------------------------------------------------------
// velocity correction (+ pressure update)
//   src/fluid/correct_velocity/ux.c:18-66, uy.c:17-64
//   src/fluid/update_pressure.c:7-53
//   u -= dt_new / rho_ref dpsi_new / h;  u += -dt_old (1/rho - 1/rho_ref) dpsi_old / h
//   with 1/rho - 1/rho_ref = e / rho_ref; pax e dpsi_old and pay e dpsi_old at
//   the faces are egx, egy (k_predict_mf or k_face_factor); the x coefficients
//   come per column (cnew / HXXF(I), cold / HXXF(I) / pax), the y ones per case
// thread (I, J): I = 1..nx
// ---------------------------------------------------------------------------
// DP: also stores psi_new's differences across the faces for the next
// substage's predictor (dpx, dpy; the fused step)
template <bool PRES, bool DP>
__global__ void __launch_bounds__(BX *BY)
    k_correct(Grid g, const double *__restrict__ sc, const double *__restrict__ coltab, int k,
              double *__restrict__ ux, double *__restrict__ uy, const double *__restrict__ psin,
              const double *__restrict__ egx, const double *__restrict__ egy, double *__restrict__ p,
              double *__restrict__ dpx, double *__restrict__ dpy) {
  pdl_entry();
  sc += (size_t)blockIdx.z * (kScalars);
  const double *__restrict__ ct = coltab + (size_t)blockIdx.z * 3 * kColTabs * g.ct;
  const double *__restrict__ cn = ct + ct_cnewx(k) * g.ct, *__restrict__ co = ct + ct_coldx(k) * g.ct;
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx || J > g.ny) return;
  const int zr = blockIdx.z * g.ny;  // first row of this case
  const int r = J - 1 + zr, rm = wrap(J - 1, g.ny) + zr;
  const double cnewy = sc[sc_cnewy(k)], coldyp = sc[sc_coldyp(k)];
  const double pn0 = psin[ix(g, r, I)];
  if (I >= 2) {
    double u = ux[ix(g, r, I - 1)];
    const double d = pn0 - psin[ix(g, r, I - 1)];
    if (DP) dpx[ix(g, r, I - 1)] = d;
    u = fma(-cn[I], d, u);
    u = fma(co[I], egx[ix(g, r, I - 1)], u);
    ux[ix(g, r, I - 1)] = u;
  }
  {
    double u = uy[ix(g, r, I)];
    const double d = pn0 - psin[ix(g, rm, I)];
    if (DP) dpy[ix(g, r, I)] = d;
    u = fma(-cnewy, d, u);
    u = fma(coldyp, egy[ix(g, r, I)], u);
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
  pdl_entry();
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
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
// fixed h because both roundings are monotone; so k_decide_dt reduces max |u|
// per x column (ux) and over the domain (uy) on the integer patterns of the
// non-negative doubles, and k_decide_dt_fin forms the nx - 1 quotients of the
// columns over its blocks and their minimum (the minimum of positive doubles
// is that of their bit patterns), then its last block the dt and every
// per-substage scalar of the step.  A non-finite velocity sets bit 0 of the
// status word.  Scratch per case (nx + 8 words, zero between launches):
// [2..nx] column max |ux| bits, [nx+2] max |uy| bits, [nx+4] the complement
// of the least quotient's bits (so that zero means none yet), [nx+5] the
// finishing blocks' counter.
// ---------------------------------------------------------------------------
constexpr unsigned long long kAbsMask = 0x7fffffffffffffffULL;
constexpr unsigned long long kInfBits = 0x7ff0000000000000ULL;

__global__ void __launch_bounds__(BX *BY)
    k_decide_dt(Grid g, const double *__restrict__ ux, const double *__restrict__ uy,
                unsigned long long *__restrict__ acc) {
  pdl_entry();
  acc += (size_t)blockIdx.z * ((size_t)g.nx + 8);
  __shared__ unsigned long long colmax[BY][BX];
  __shared__ unsigned long long ymax[BY * BX];
  const int I = blockIdx.x * BX + threadIdx.x + 1;  // 1..nx+1
  unsigned long long mx = 0ULL, my = 0ULL;
  if (I <= g.nx) {
#pragma unroll 4
    for (int J = blockIdx.y * BY + threadIdx.y + 1; J <= g.ny; J += gridDim.y * BY) {
      const int r = J - 1 + (int)blockIdx.z * g.ny;
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
  }
  for (int w = BX * BY / 2; w > 0; w >>= 1) {
    if (tid < w) ymax[tid] = ymax[tid + w] > ymax[tid] ? ymax[tid + w] : ymax[tid];
    __syncthreads();
  }
  if (tid == 0 && ymax[0]) atomicMax(acc + g.nx + 2, ymax[0]);
}

// the finishing kernel: one column per thread (I = 2..nx over the blocks),
// then the last block of each case: dt, the scalars and the reset of the
// scratch
constexpr int kDtFinThreads = 256;
__global__ void __launch_bounds__(kDtFinThreads)
    k_decide_dt_fin(Grid g, Metrics m, Phys ph0, unsigned long long *__restrict__ acc, double *__restrict__ sc,
                    int *__restrict__ status, double dt_fixed, double coef_adv) {
  pdl_entry();
  const Phys ph = zphys(g, ph0);
  if (g.phys) dt_fixed = ph.dtfix;
  acc += (size_t)blockIdx.z * ((size_t)g.nx + 8);
  sc += (size_t)blockIdx.z * (kScalars);
  status += (size_t)blockIdx.z * (1);
  __shared__ double wmin[kDtFinThreads / 32];
  __shared__ int wbad[kDtFinThreads / 32];
  __shared__ bool last;
  const double small = 1.e-8;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // dt_adv = coef * min(1, min_i hx_i / (max|ux|_i + small), hy / (max|uy| + small))
  double d = 1.;
  int bad = 0;
  const int i = blockIdx.x * kDtFinThreads + tid + 2;
  if (i <= g.nx) {
    // the column maxima are final (the stream order) and were formed at L2
    const unsigned long long b = __ldcg(acc + i);
    bad = b >= kInfBits ? 1 : 0;
    d = m.hxxf[i] / (__longlong_as_double((long long)b) + small);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    d = fmin(d, __shfl_xor_sync(0xffffffffu, d, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if (lane == 0) {
    wmin[warp] = d;
    wbad[warp] = bad;
  }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < kDtFinThreads / 32; ++w) {
      d = fmin(d, wmin[w]);
      bad |= wbad[w];
    }
    // a positive d (or 1): the least bit pattern is the least value
    atomicMax(acc + g.nx + 4, ~(unsigned long long)dbits(d));
    if (bad) atomicOr(status, 1);
    __threadfence();
    const unsigned int done = atomicAdd(reinterpret_cast<unsigned int *>(acc + g.nx + 5), 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (tid == 0) {
    const double dmin = __longlong_as_double((long long)~__ldcg(acc + g.nx + 4));
    const unsigned long long by = __ldcg(acc + g.nx + 2);
    double dt = fmin(dmin, g.hy / (__longlong_as_double((long long)by) + small));
    dt *= coef_adv;
    dt = fmin(dt, dt_fixed);
    if (by >= kInfBits) atomicOr(status, 1);
    // per-substage scalars; RK3 coefficients of src/runge_kutta.c:8-15
    const double al[3] = {32. / 60., 25. / 60., 45. / 60.};
    const double be[3] = {0. / 60., -17. / 60., -25. / 60.};
    sc[0] = dt;
    for (int k = 0; k < 3; ++k) {
      const int ko = (k + 2) % 3;
      const double dtold = (al[ko] + be[ko]) * dt, dtnew = (al[k] + be[k]) * dt;
      sc[sc_adt(k)] = al[k] * dt;
      sc[sc_bdt(k)] = be[k] * dt;
      sc[sc_gdt(k)] = (al[k] + be[k]) * dt;
      sc[sc_adt2(k)] = 2. * (al[k] * dt);
      sc[sc_bdt2(k)] = 2. * (be[k] * dt);
      sc[sc_gdt2(k)] = 2. * ((al[k] + be[k]) * dt);
      sc[sc_dtold(k)] = dtold;
      sc[sc_dtnew(k)] = dtnew;
      const double cdiv = ph.refden / dtnew * (0.5 / g.ny);
      const double cadd = -(dtold / dtnew) * (0.5 / g.ny);
      sc[sc_pdx(k)] = cdiv * g.idx;
      sc[sc_pdy(k)] = cdiv * g.ihy;
      sc[sc_pax(k)] = cadd * (g.idx * g.idx);
      sc[sc_pay(k)] = cadd * (g.ihy * g.ihy);
      sc[sc_cnew(k)] = dtnew * ph.irefden;
      sc[sc_cold(k)] = -dtold * ph.irefden;
      sc[sc_cnewy(k)] = sc[sc_cnew(k)] * g.ihy;
      sc[sc_coldy(k)] = sc[sc_cold(k)] * g.ihy;
      sc[sc_gdt2y(k)] = sc[sc_gdt2(k)] * g.ihy;
      sc[sc_coldyp(k)] = sc[sc_coldy(k)] / sc[sc_pay(k)];
      sc[sc_rpx(k)] = ph.rref2 * sc[sc_pax(k)];
      sc[sc_rpy(k)] = ph.rref2 * sc[sc_pay(k)];
    }
  }
  __syncthreads();
  // reset the scratch for the next launch
  for (int t = tid; t <= g.nx + 5; t += kDtFinThreads) acc[t] = 0ULL;
}

// the per-column coefficients of the three substages from the scalars (one
// column per thread, over many blocks: on one block they were the finishing
// kernel's tail)
__global__ void __launch_bounds__(kDtFinThreads)
    k_decide_dt_tab(Grid g, Metrics m, const double *__restrict__ sc, double *__restrict__ coltab) {
  pdl_entry();
  sc += (size_t)blockIdx.z * (kScalars);
  coltab += (size_t)blockIdx.z * 3 * kColTabs * g.ct;
  const int I = blockIdx.x * kDtFinThreads + threadIdx.x;
  if (I > g.nx + 1) return;
  const double ih = m.ihxxf[I];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // cold / pax once per column and substage (the same quotient everywhere)
    const double cop = sc[sc_cold(k)] / sc[sc_pax(k)];
    coltab[(size_t)ct_gdt2x(k) * g.ct + I] = sc[sc_gdt2(k)] * ih;
    coltab[(size_t)ct_cnewx(k) * g.ct + I] = sc[sc_cnew(k)] * ih;
    coltab[(size_t)ct_coldx(k) * g.ct + I] = cop * ih;
  }
}

// pax e grad psi_old and pay e grad psi_old, e = rho_ref / rho - 1, at ux
// faces (I = 1..nx+1) and uy faces (I = 1..nx) from a density field and
// psi_old, as k_predict_mf stores them (fine-grained entry points; the
// scalars of slot 0)
__global__ void k_face_factor(Grid g, const double *__restrict__ sc, const double *__restrict__ den,
                              const double *__restrict__ psio, double *__restrict__ egx, double *__restrict__ egy) {
  pdl_entry();
  const int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int r = J - 1, rm = wrap(J - 1, g.ny);
  const double ps = psio[ix(g, r, I)];
  const double ex = fma(sc[sc_rpx(0)], rcp_nr(den[ix(g, r, I - 1)] + den[ix(g, r, I)]), -sc[sc_pax(0)]);
  egx[ix(g, r, I - 1)] = ex * (ps - psio[ix(g, r, I - 1)]);
  if (I <= g.nx) {
    const double ey = fma(sc[sc_rpy(0)], rcp_nr(den[ix(g, rm, I)] + den[ix(g, r, I)]), -sc[sc_pay(0)]);
    egy[ix(g, r, I)] = ey * (ps - psio[ix(g, rm, I)]);
  }
}

// ---------------------------------------------------------------------------
// diagnostics of the reference's log files (src/logging/), reduced on the device:
//   [0] max |div u|                     src/logging/divergence.c:41-64
//   [1] min vof, [2] max vof, [3] sum vof J, [4] sum J, [5] interface area
//                                       src/logging/interface.c:34-65
//   [6..7] momentum x, y                src/logging/momentum.c:40-56
//   [8..9] kinetic energy x, y          src/logging/energy.c:42-58
//   [10..11] max |ux|, max |uy|         src/logging/extrema.c:25-38
//   [12..13] wall shear stress x = 0, lx  src/logging/stress.c:29-35
// Per-block partials in a fixed order, then one block: deterministic.
// ---------------------------------------------------------------------------
constexpr int kDiag = 16;

__device__ __forceinline__ void block_reduce(double (*sm)[BX * BY], int tid, const double *v) {
  for (int q = 0; q < kDiag; ++q) sm[q][tid] = v[q];
  __syncthreads();
  for (int w = BX * BY / 2; w > 0; w >>= 1) {
    if (tid < w) {
      for (int q = 0; q < kDiag; ++q) {
        const double a = sm[q][tid], b = sm[q][tid + w];
        // 0 and 2 and 10..11 are maxima, 1 is a minimum, the rest sums
        sm[q][tid] = (q == 0 || q == 2 || q == 10 || q == 11) ? fmax(a, b) : (q == 1 ? fmin(a, b) : a + b);
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(BX *BY)
    k_diag_partial(Grid g, Metrics m, const double *__restrict__ ux, const double *__restrict__ uy,
                   const double *__restrict__ vof, const double *__restrict__ den, const double *__restrict__ txy,
                   double nu, double *__restrict__ part) {
  pdl_entry();
  __shared__ double sm[kDiag][BX * BY];
  const int I = blockIdx.x * BX + threadIdx.x + 1;
  const int J = blockIdx.y * BY + threadIdx.y + 1;
  const int tid = threadIdx.y * BX + threadIdx.x;
  double v[kDiag];
  for (int q = 0; q < kDiag; ++q) v[q] = 0.;
  v[1] = 1.;  // the reference starts min at 1 and max at 0
  if (I <= g.nx && J <= g.ny) {
    const int r = J - 1, rm = wrap(J - 1, g.ny), rp = wrap(J + 1, g.ny);
    const double jdxc = g.dx * g.hy;
    const double div = (ux[ix(g, r, I)] - ux[ix(g, r, I - 1)]) * g.idx + (uy[ix(g, rp, I)] - uy[ix(g, r, I)]) * g.ihy;
    v[0] = fabs(div);
    const double phi = vof[ix(g, r, I)];
    v[1] = phi;
    v[2] = phi;
    v[3] = phi * jdxc;
    v[4] = jdxc;
    v[5] = fabs(phi - vof[ix(g, r, I - 1)]) * g.hy + fabs(phi - vof[ix(g, rm, I)]) * g.dx;
    if (I == g.nx) v[5] += fabs(vof[ix(g, r, g.nx + 1)] - phi) * g.hy;
    if (I >= 2) {
      const double u = ux[ix(g, r, I - 1)];
      const double jdxf = m.hxxf[I] * g.hy;
      const double rho = 0.5 * den[ix(g, r, I - 1)] + 0.5 * den[ix(g, r, I)];
      v[6] = rho * u * jdxf;
      v[8] = 0.5 * rho * u * u * jdxf;
      v[10] = fabs(u);
    }
    const double w = uy[ix(g, r, I)];
    const double rhoy = 0.5 * den[ix(g, rm, I)] + 0.5 * den[ix(g, r, I)];
    v[7] = rhoy * w * jdxc;
    v[9] = 0.5 * rhoy * w * w * jdxc;
    v[11] = fabs(w);
    // JDXF / HXXF = hy at the wall faces
    if (I == 1) v[12] = nu * g.hy * txy[ix(g, r, 0)];
    if (I == g.nx) v[13] = nu * g.hy * txy[ix(g, r, g.nx)];
  }
  block_reduce(sm, tid, v);
  if (tid < kDiag) part[(size_t)(blockIdx.y * gridDim.x + blockIdx.x) * kDiag + tid] = sm[tid][0];
}

__global__ void __launch_bounds__(BX *BY) k_diag_final(const double *__restrict__ part, int nblocks,
                                                       double *__restrict__ out) {
  pdl_entry();
  __shared__ double sm[kDiag][BX * BY];
  const int tid = threadIdx.x;
  double v[kDiag];
  for (int q = 0; q < kDiag; ++q) v[q] = 0.;
  v[1] = 1.;
  for (int b = tid; b < nblocks; b += BX * BY) {
    for (int q = 0; q < kDiag; ++q) {
      const double x = part[(size_t)b * kDiag + q];
      v[q] = (q == 0 || q == 2 || q == 10 || q == 11) ? fmax(v[q], x) : (q == 1 ? fmin(v[q], x) : v[q] + x);
    }
  }
  block_reduce(sm, tid, v);
  if (tid < kDiag) out[tid] = sm[tid][0];
}

// running sums of the statistics (src/statistics.c:99-151): ux1 += ux over
// I = 1..nx+1, uy1 += uy and vof1 += vof over I = 0..nx+1
__global__ void k_stats_collect(Grid g, const double *__restrict__ ux, const double *__restrict__ uy,
                                const double *__restrict__ vof, double *__restrict__ ux1, double *__restrict__ uy1,
                                double *__restrict__ vof1) {
  pdl_entry();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (I > g.nx + 1 || J > g.ny) return;
  const int r = J - 1;
  if (I >= 1) ux1[ix(g, r, I - 1)] += ux[ix(g, r, I - 1)];
  uy1[ix(g, r, I)] += uy[ix(g, r, I)];
  vof1[ix(g, r, I)] += vof[ix(g, r, I)];
}

// ---- boundary kernels of the fine-grained entry points (one thread per row)
__global__ void k_bc_ux(Grid g, double *ux) {
  pdl_entry();
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  ux[ix(g, J - 1, 0)] = 0.;
  ux[ix(g, J - 1, g.nx)] = 0.;
}
__global__ void k_bc_uy(Grid g, double *uy) {
  pdl_entry();
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  uy[ix(g, J - 1, 0)] = 0.;
  uy[ix(g, J - 1, g.nx + 1)] = 0.;
}
__global__ void k_bc_neumann(Grid g, double *f) {
  pdl_entry();
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  f[ix(g, J - 1, 0)] = f[ix(g, J - 1, 1)];
  f[ix(g, J - 1, g.nx + 1)] = f[ix(g, J - 1, g.nx)];
}
__global__ void k_bc_vof(Grid g, double *vof) {
  pdl_entry();
  const int J = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (J > g.ny) return;
  vof[ix(g, J - 1, 0)] = 0.;
  vof[ix(g, J - 1, g.nx + 1)] = 0.;
}

// test hook: the Newton-Raphson reciprocal and inverse square root on n inputs
__global__ void k_nr_check(const double *__restrict__ x, double *__restrict__ rcp, double *__restrict__ rsq, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  rcp[i] = rcp_nr(x[i]);
  rsq[i] = rsqrt_nr(x[i]);
}

// columns per transform block before tuning: with 2, 256 threads and 32 KB
// at ny = 1024, five blocks share an SM (40 warps); with 4, three (24 warps).
// The 2048 x 1024 swarm stepped 3% faster and 1024 x 512 11% faster.
constexpr int kFftCols = 2;
// dynamic shared memory of k_poisson_tdm<false> (its static xch lies beside)
constexpr size_t kTdmSmemMax = 227 * 1024 - 4096;

// FP64 fused multiply-add throughput: 8 independent chains per thread, every
// thread writes only its own output element
__global__ void k_fp64_peak(double *out, int iters, double seed) {
  const double m = 0.999999, c = 1e-7;
  double a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = seed + 1e-3 * j + 1e-9 * threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = fma(a[j], m, c);
  }
  double s = 0.;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

cudaError_t measure_fp64_peak(double *gflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 8192;
  double *out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * blocks * threads);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int w = 0; w < 3; ++w) k_fp64_peak<<<blocks, threads>>>(out, iters, 0.1);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_fp64_peak<<<blocks, threads>>>(out, iters, 0.1);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *gflops = 2.0 * 8.0 * blocks * threads * (double)iters / (best * 1e-3) / 1e9;
  return e;
}

cudaError_t nr_check(const double *x, double *rcp, double *rsq, int n) {
  k_nr_check<<<(n + 255) / 256, 256>>>(x, rcp, rsq, n);
  return cudaDeviceSynchronize();
}

// ===========================================================================
// launch helpers
// ===========================================================================

// columns per block of the transforms: kFftCols, halved while a block's two
// ny/2 complex rows per column exceed shared memory (ny = 8192 takes 1)
int poisson_fft_cols(int ny) {
  int w = kFftCols;
  while (w > 1 && !fft_w_fits(ny, w)) w >>= 1;
  return w;
}
size_t poisson_fft_smem(int ny, int w) { return sizeof(double2) * 2 * w * (size_t)(ny / 2); }
bool fft_w_fits(int ny, int w) { return poisson_fft_smem(ny, w) <= 227 * 1024; }

int compaction(const Tiles &t) { return g_compact >= 0 ? g_compact : t.compact; }

Tiles default_tiles(int ny) {
  Tiles t{};
  for (int k = 0; k < TK_COUNT; ++k) {
    t.bx[k] = BX;
    t.by[k] = BY;
  }
  t.fft_w = poisson_fft_cols(ny);
  t.tdm_mb = 0;
  t.tdm_g = 1;
  t.compact = 1;
  t.tdm_cl = 1;
  return t;
}
int tdm_chunk(int nx, int G) { return (nx + 32 * G - 1) / (32 * G); }
int tdm_stride(int nx, int G) { return tdm_chunk(nx, G) | 1; }
int poisson_tdm_modes(int nx) {
  const size_t per_mode = 4 * 32 * (size_t)tdm_stride(nx, 1) * sizeof(double);
  return per_mode * 4 <= 200 * 1024 ? 4 : (per_mode * 2 <= 200 * 1024 ? 2 : 1);
}
// mb: wavenumber pairs (p, M - p) per block, four systems each
size_t poisson_tdm_smem(int nx, int mb, int G) {
  return 4 * 32 * (size_t)G * tdm_stride(nx, G) * sizeof(double) * mb;
}
size_t poisson_tdm_smem(int nx) { return poisson_tdm_smem(nx, poisson_tdm_modes(nx), 1); }
bool tdm_global_stage(int nx, int G) { return poisson_tdm_smem(nx, 1, G) > kTdmSmemMax; }
size_t tdm_stage_doubles(int nx, int ny, int nc, int G) {
  return tdm_global_stage(nx, G) ? (size_t)(ny / 4 + 1) * nc * 4 * 32 * G * tdm_stride(nx, G) : 0;
}
int tdm_group_index(int G) { return G == 4 ? 2 : (G == 2 ? 1 : 0); }
// warps per tridiagonal system for a grid of nc cases: the fewest (1, 2, 4)
// that put about 2048 warps in flight (13 per SM), as long as every lane
// keeps at least 4 rows (with 2, the cross-warp combine costs more than the
// shorter recurrences save; 4 rows a lane beat 8 and 16 on every grid from
// 256 x 128 to 1024 x 512; on the 2048 x 1024 swarm 4 warps a system in
// clusters balance the SMs better but add 6% to the solve's FP64 work, and
// the step gains nothing: the side stream fills the SMs a block-per-pair
// launch leaves idle).  At 4 warps a system the solves of a pair run as a
// cluster of four CTAs (k_poisson_tdm_cl).  A rule of the grid, not a tuned choice: it sets how
// the chunk maps are combined, and so the rounding of the solve.
int tdm_modes_per_block(const Tiles &t, int nx) {
  const int G = t.tdm_g > 0 ? t.tdm_g : 1;
  const int mb = t.tdm_mb > 0 ? t.tdm_mb : poisson_tdm_modes(nx);
  return mb * G > 4 ? 4 / G : mb;  // at most 512 threads a block
}
int tdm_warps_for(int nx, int ny, int nc) {
  const long systems = 4L * (ny / 4 + 1) * nc;
  int G = 1;
  while (G < 4 && systems * G < 2048 && tdm_chunk(nx, 2 * G) >= 4) G *= 2;
  return G;
}

cudaError_t configure_kernels() {
  cudaError_t e;
  const int big = 227 * 1024;
  e = cudaFuncSetAttribute(k_poisson_fwd<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_fwd<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_fwd<4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_fwd<4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_fwd<8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_fwd<8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_inv<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_inv<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_inv<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_fwd<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_fwd<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_inv<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_tdm<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTdmSmemMax);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_poisson_tdm_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTdmSmemMax);
  return e;
}

void launch_props(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b, bool den, bool vis,
                  bool grad, double *den_out, bool scaled) {
  const dim3 gr = tile_grid(b.tiles, TK_PROPS, g.nx + 2, g.ny, g.nc), bl = tile_block(b.tiles, TK_PROPS);
  if (scaled && vis && grad && !den)
    launch_pdl(k_props<false, true, true, true>, gr, bl, 0, s, g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof,
               compaction(b.tiles));
  else if (den && vis && grad)
    launch_pdl(k_props<true, true, true>, gr, bl, 0, s, g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof,
               compaction(b.tiles));
  else if (vis && grad)
    launch_pdl(k_props<false, true, true>, gr, bl, 0, s, g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof,
               compaction(b.tiles));
  else if (den)
    launch_pdl(k_props<true, false, false>, gr, bl, 0, s, g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof,
               compaction(b.tiles));
  else if (vis)
    launch_pdl(k_props<false, true, false>, gr, bl, 0, s, g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof,
               compaction(b.tiles));
  else if (grad)
    launch_pdl(k_props<false, false, true>, gr, bl, 0, s, g, m, ph, b.vof, den_out, b.visux, b.visuy, b.dvof,
               compaction(b.tiles));
}

void launch_normal_curv(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, bool normal, bool curv,
                        bool store_k) {
  const dim3 gr = grid2d(g.nx, g.ny), bl(BX, BY);
  if (normal && curv && store_k)
    launch_pdl(k_normal_curv<true, true, true>, gr, bl, 0, s, g, m, b.vof, b.dvof, b.normal, b.curv);
  else if (normal && curv)
    launch_pdl(k_normal_curv<true, true, false>, gr, bl, 0, s, g, m, b.vof, b.dvof, b.normal, b.curv);
  else if (normal)
    launch_pdl(k_normal_curv<true, false, false>, gr, bl, 0, s, g, m, b.vof, b.dvof, b.normal, b.curv);
  else if (curv)
    launch_pdl(k_normal_curv<false, true, false>, gr, bl, 0, s, g, m, b.vof, b.dvof, b.normal, b.curv);
}

void launch_flux_force(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                       const double *ux, const double *uy, const double *den0, bool flux, bool force, bool have_k) {
  const dim3 gr = grid2d(g.nx, g.ny), bl(BX, BY);
  if (flux && force && have_k)
    launch_pdl(k_flux_force<true, true, true>, gr, bl, 0, s, g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx,
                                                     b.fluxy, b.ifrcx, b.ifrcy);
  else if (flux && force)
    launch_pdl(k_flux_force<true, true, false>, gr, bl, 0, s, g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx,
                                                      b.fluxy, b.ifrcx, b.ifrcy);
  else if (flux)
    launch_pdl(k_flux_force<true, false, false>, gr, bl, 0, s, g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx,
                                                       b.fluxy, b.ifrcx, b.ifrcy);
  else if (force)
    launch_pdl(k_flux_force<false, true, false>, gr, bl, 0, s, g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx,
                                                       b.fluxy, b.ifrcx, b.ifrcy);
}

void launch_interface_stage(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                            const double *ux, const double *uy, const double *den0, int stage) {
  const dim3 gr = tile_grid(b.tiles, TK_FLUX_FORCE, g.nx, g.ny, g.nc), bl = tile_block(b.tiles, TK_FLUX_FORCE);
  if (stage == 0) {
    cudaMemsetAsync(b.icount, 0, sizeof(int) * 2 * g.nc, s);  // cell and face counts
    launch_pdl(k_curv_list<true>, tile_grid(b.tiles, TK_CURV_LIST, g.nx, g.ny, g.nc), tile_block(b.tiles, TK_CURV_LIST),
               0, s, g, m, b.vof, b.dvof, ux, uy, b.curv, b.ilist, b.icount, b.flist, b.fcount, (double *)nullptr,
               compaction(b.tiles));
  } else if (stage == 1) {
    launch_pdl(k_interface_cells, dim3(max(2, (4 * 152 + g.nc - 1) / g.nc), 1, g.nc), 256, 0, s,
        g, m, ux, uy, b.vof, b.dvof, b.flist, b.fcount, b.fluxx, b.fluxy);
  } else if (stage == 2) {
    launch_pdl(k_flux_force<true, true, true, true>, gr, bl, 0, s, g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv, b.fluxx,
                                                           b.fluxy, b.ifrcx, b.ifrcy);
  } else {
    launch_pdl(k_flux_force<true, true, true, true, true>, gr, bl, 0, s, g, m, ph, ux, uy, b.vof, b.normal, den0, b.curv,
                                                                 b.fluxx, b.fluxy, b.ifrcx, b.ifrcy);
  }
}

void launch_geometry(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b) {
  cudaMemsetAsync(b.icount, 0, sizeof(int) * 2 * g.nc, s);  // cell and face counts
  launch_pdl(k_curv_list<false>, tile_grid(b.tiles, TK_CURV_LIST, g.nx, g.ny, g.nc), tile_block(b.tiles, TK_CURV_LIST),
             0, s, g, m, b.vof, b.dvof, (const double *)nullptr, (const double *)nullptr, b.curv, b.ilist, b.icount,
             b.flist, b.fcount, b.tf, compaction(b.tiles));
}

void launch_bulk_flux(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                      const double *ux, const double *uy) {
  launch_pdl(k_bulk_flux, tile_grid(b.tiles, TK_FLUX_FORCE, g.nx, g.ny, g.nc), tile_block(b.tiles, TK_FLUX_FORCE), 0, s,
             g, m, ph, ux, uy, b.vof, b.fluxx, b.fluxy);
}

void launch_csf_force(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                      const double *den0, double *ifx, double *ify, bool itf_kappa) {
  const dim3 gr = tile_grid(b.tiles, TK_FORCE, g.nx, g.ny, g.nc), bl = tile_block(b.tiles, TK_FORCE);
  if (itf_kappa)
    launch_pdl(k_csf_force<true>, gr, bl, 0, s, g, m, ph, b.vof, den0, b.curv, ifx, ify);
  else
    launch_pdl(k_csf_force<false>, gr, bl, 0, s, g, m, ph, b.vof, den0, b.curv, ifx, ify);
}

void launch_vof_advance(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                        const double *sc, int k, double *src_a, const double *src_b, bool fused, const double *ux,
                        const double *uy, double *den1, double *vof_out) {
  const dim3 gr = tile_grid(b.tiles, TK_VOF_ADVANCE, g.nx, g.ny, g.nc), bl = tile_block(b.tiles, TK_VOF_ADVANCE);
  if (fused && vof_out)
    launch_pdl(k_vof_advance<true, true>, gr, bl, 0, s, g, m, ph, sc, k, b.vof, vof_out, b.fluxx, b.fluxy, src_a, src_b,
               ux, uy, b.mfluxx, b.mfluxy, den1);
  else if (fused)
    launch_pdl(k_vof_advance<true, false>, gr, bl, 0, s, g, m, ph, sc, k, b.vof, (double *)nullptr, b.fluxx, b.fluxy,
               src_a, src_b, ux, uy, b.mfluxx, b.mfluxy, den1);
  else
    launch_pdl(k_vof_advance<false, false>, gr, bl, 0, s, g, m, ph, sc, k, b.vof, (double *)nullptr, b.fluxx, b.fluxy,
               src_a, src_b, ux, uy, (double *)nullptr, (double *)nullptr, (double *)nullptr);
}

void launch_face_flux(cudaStream_t s, const Grid &g, const Bufs &b, const double *ux, const double *uy) {
  launch_pdl(k_face_flux, dim3(max(2, (4 * 152 + g.nc - 1) / g.nc), 1, g.nc), 256, 0, s, g, ux, uy, b.ilist, b.icount,
             b.tf, b.fluxx, b.fluxy);
}

void launch_mass_flux_inplace(cudaStream_t s, const Grid &g, const Phys &ph, const Bufs &b, const double *ux,
                              const double *uy) {
  launch_pdl(k_mass_flux, grid2d(g.nx + 2, g.ny), dim3(BX, BY), 0, s, g, ph, ux, uy, b.fluxx, b.fluxy);
}

void launch_stress(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, const double *ux,
                   const double *uy) {
  launch_pdl(k_stress, tile_grid(b.tiles, TK_MOMFLUX, g.nx + 1, g.ny, g.nc), tile_block(b.tiles, TK_MOMFLUX), 0, s, g,
             m, ux, uy, b.visux, b.visuy, b.txx, b.txy, b.tyy);
}

void launch_momflux(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                    const double *ux, const double *uy, int stress, bool scaled) {
  const dim3 gr = tile_grid(b.tiles, TK_MOMFLUX, g.nx + 1, g.ny, g.nc), bl = tile_block(b.tiles, TK_MOMFLUX);
  auto k = stress == 2 ? k_momflux<2, false>
                       : (scaled ? (stress == 1 ? k_momflux<1, true> : k_momflux<0, true>)
                                 : (stress == 1 ? k_momflux<1, false> : k_momflux<0, false>));
  launch_pdl(k, gr, bl, 0, s, g, m, ph, ux, uy, b.visux, b.visuy, b.mfluxx, b.mfluxy, b.pxx, b.pyy, b.pxy, b.pyx,
             b.txx, b.txy, b.tyy);
}

void launch_predict_mf(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                       const double *sc, int k, const double *ux, const double *uy, double *ux_out, double *uy_out,
                       const double *den0, const double *den1, const double *psi_old, double *srcux_a,
                       const double *srcux_b, double *srcuy_a, const double *srcuy_b, const double *ifx,
                       const double *ify, bool cached) {
  auto kern = cached ? k_predict_mf<true> : k_predict_mf<false>;
  launch_pdl(kern, tile_grid(b.tiles, TK_PREDICT, g.nx, g.ny, g.nc), tile_block(b.tiles, TK_PREDICT), 0, s, g, m, ph,
             sc, k, ux, uy, ux_out, uy_out, b.pxx, b.pyy, b.pxy, b.pyx, b.p, ifx, ify, den0, den1, psi_old, srcux_a,
             srcux_b, srcuy_a, srcuy_b, b.egx, b.egy, b.coltab, b.qx, b.qy, b.rhofx, b.rhofy, b.dpsix, b.dpsiy);
}

void launch_predict(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b, const double *sc,
                    int k, const double *ux, const double *uy, double *ux_out, double *uy_out, const double *mfx,
                    const double *mfy, const double *den0, const double *den1, double *srcux_a,
                    const double *srcux_b, double *srcux_g, double *srcuy_a, const double *srcuy_b,
                    double *srcuy_g) {
  launch_pdl(k_predict, tile_grid(b.tiles, TK_PREDICT, g.nx, g.ny, g.nc), tile_block(b.tiles, TK_PREDICT), 0, s, g, m, ph, sc, k, ux, uy, ux_out, uy_out, mfx, mfy, b.txx,
                                                        b.txy, b.tyy, b.p, b.ifrcx, b.ifrcy, den0, den1, srcux_a,
                                                        srcux_b, srcux_g, srcuy_a, srcuy_b, srcuy_g);
}

template <int W, bool Q>
void poisson_fwd_w(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k, const double *ux,
                   const double *uy) {
  const int nb = (g.nx + W - 1) / W;
  launch_pdl(k_poisson_fwd<W, Q>, dim3(nb, 1, g.nc), 256, poisson_fft_smem(g.ny, W), s, g, sc, k, ux, uy, b.egx,
             b.egy, b.twiddle, b.spec);
}

template <bool Q>
void poisson_fwd_any(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k, const double *ux,
                     const double *uy) {
  if (b.tiles.fft_w == 1)
    poisson_fwd_w<1, Q>(s, g, b, sc, k, ux, uy);
  else if (b.tiles.fft_w == 2)
    poisson_fwd_w<2, Q>(s, g, b, sc, k, ux, uy);
  else if (b.tiles.fft_w == 8)
    poisson_fwd_w<8, Q>(s, g, b, sc, k, ux, uy);
  else
    poisson_fwd_w<4, Q>(s, g, b, sc, k, ux, uy);
}

void launch_poisson_fwd(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k, const double *ux,
                        const double *uy) {
  poisson_fwd_any<false>(s, g, b, sc, k, ux, uy);
}

void launch_poisson_fwd_q(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k) {
  poisson_fwd_any<true>(s, g, b, sc, k, b.qx, b.qy);
}

int g_tdm_cluster = 1;

bool tdm_uses_cluster(const Tiles &t, int nx) {
  return g_tdm_cluster && t.tdm_cl && t.tdm_g == 4 &&
         4 * 32 * (size_t)tdm_stride(nx, 4) * sizeof(double) <= kTdmSmemMax;
}

void launch_poisson_tdm(cudaStream_t s, const Grid &g, const Bufs &b) {
  const int G = b.tiles.tdm_g > 0 ? b.tiles.tdm_g : 1;
  const int pairs = g.ny / 4 + 1;
  const double4_32a *fac = reinterpret_cast<const double4_32a *>(b.tdm_fac[tdm_group_index(G)]);
  if (tdm_uses_cluster(b.tiles, g.nx)) {  // four CTAs per pair, four warps each
    const int L = tdm_chunk(g.nx, 4), S = tdm_stride(g.nx, 4);
    launch_pdl(k_poisson_tdm_cl, dim3(kTdmCluster * pairs, 1, g.nc), 128, 4 * 32 * (size_t)S * sizeof(double), s, g,
               L, S, fac, b.twiddle, b.spec);
    return;
  }
  if (tdm_global_stage(g.nx, G)) {  // one pair per block, staged in b.tdm_stage
    launch_pdl(k_poisson_tdm<true>, dim3(pairs, 1, g.nc), 128 * G, 0, s, g, 1, G, tdm_chunk(g.nx, G), tdm_stride(g.nx, G),
                                                                 fac, b.twiddle, b.spec, b.tdm_stage);
    return;
  }
  const int mb = tdm_modes_per_block(b.tiles, g.nx);  // wavenumber pairs per block
  launch_pdl(k_poisson_tdm<false>, dim3((pairs + mb - 1) / mb, 1, g.nc), 128 * mb * G, poisson_tdm_smem(g.nx, mb, G), s,
      g, mb, G, tdm_chunk(g.nx, G), tdm_stride(g.nx, G), fac, b.twiddle, b.spec, nullptr);
}

template <int W>
void poisson_inv_w(cudaStream_t s, const Grid &g, const Bufs &b, double *psi_new) {
  const int nb = (g.nx + W - 1) / W;
  launch_pdl(k_poisson_inv<W>, dim3(nb, 1, g.nc), 256, poisson_fft_smem(g.ny, W), s, g, b.twiddle, b.spec, psi_new);
}

void launch_poisson_inv(cudaStream_t s, const Grid &g, const Bufs &b, double *psi_new) {
  if (b.tiles.fft_w == 1)
    poisson_inv_w<1>(s, g, b, psi_new);
  else if (b.tiles.fft_w == 2)
    poisson_inv_w<2>(s, g, b, psi_new);
  else if (b.tiles.fft_w == 8)
    poisson_inv_w<8>(s, g, b, psi_new);
  else
    poisson_inv_w<4>(s, g, b, psi_new);
}

void launch_poisson(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k, const double *ux,
                    const double *uy, double *psi_new) {
  launch_poisson_fwd(s, g, b, sc, k, ux, uy);
  launch_poisson_tdm(s, g, b);
  launch_poisson_inv(s, g, b, psi_new);
}

void launch_correct(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, const double *sc, int k,
                    double *ux, double *uy, const double *psi_new, bool pressure, bool dpsi) {
  const dim3 gr = tile_grid(b.tiles, TK_CORRECT, g.nx, g.ny, g.nc), bl = tile_block(b.tiles, TK_CORRECT);
  auto kern = pressure ? (dpsi ? k_correct<true, true> : k_correct<true, false>)
                       : (dpsi ? k_correct<false, true> : k_correct<false, false>);
  launch_pdl(kern, gr, bl, 0, s, g, sc, b.coltab, k, ux, uy, psi_new, b.egx, b.egy, b.p, b.dpsix, b.dpsiy);
}

void launch_pressure(cudaStream_t s, const Grid &g, const Bufs &b, const double *psi_new) {
  launch_pdl(k_pressure, grid2d(g.nx, g.ny), dim3(BX, BY), 0, s, g, psi_new, b.p);
}

void launch_decide_dt(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                      const double *ux, const double *uy, double dt_fixed, double coef_adv) {
  launch_decide_dt_raw(s, g, m, ph, ux, uy, b.dt_acc, b.scalars, b.status, dt_fixed, coef_adv, b.coltab);
}

void launch_decide_dt_raw(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const double *ux,
                          const double *uy, unsigned long long *acc, double *sc, int *status, double dt_fixed,
                          double coef_adv, double *coltab) {
  int gy = (g.ny + BY - 1) / BY;
  const int gx = (g.nx + BX) / BX;
  while (gy > 1 && gx * gy * g.nc > 16 * 152) gy = (gy + 1) / 2;
  launch_pdl(k_decide_dt, dim3(gx, gy, g.nc), dim3(BX, BY), 0, s, g, ux, uy, acc);
  launch_pdl(k_decide_dt_fin, dim3((g.nx - 1 + kDtFinThreads - 1) / kDtFinThreads, 1, g.nc), dim3(kDtFinThreads), 0, s,
             g, m, ph, acc, sc, status, dt_fixed, coef_adv);
  if (coltab)
    launch_pdl(k_decide_dt_tab, dim3((g.nx + 2 + kDtFinThreads - 1) / kDtFinThreads, 1, g.nc), dim3(kDtFinThreads), 0,
               s, g, m, (const double *)sc, coltab);
}

void launch_face_factor(cudaStream_t s, const Grid &g, const Phys &ph, const Bufs &b, const double *den,
                        const double *psi_old) {
  launch_pdl(k_face_factor, grid2d(g.nx + 1, g.ny), dim3(BX, BY), 0, s, g, b.scalars, den, psi_old, b.egx, b.egy);
}

int diag_partial_blocks(const Grid &g) {
  const dim3 gr = grid2d(g.nx, g.ny);
  return (int)(gr.x * gr.y);
}

void launch_diagnostics(cudaStream_t s, const Grid &g, const Metrics &m, const double *ux, const double *uy,
                        const double *vof, const double *den, const double *txy, double nu, double *part,
                        double *out) {
  const dim3 gr = grid2d(g.nx, g.ny);
  launch_pdl(k_diag_partial, gr, dim3(BX, BY), 0, s, g, m, ux, uy, vof, den, txy, nu, part);
  launch_pdl(k_diag_final, 1, BX * BY, 0, s, part, (int)(gr.x * gr.y), out);
}

void launch_stats_collect(cudaStream_t s, const Grid &g, const double *ux, const double *uy, const double *vof,
                          double *ux1, double *uy1, double *vof1) {
  launch_pdl(k_stats_collect, grid2d(g.nx + 2, g.ny), dim3(BX, BY), 0, s, g, ux, uy, vof, ux1, uy1, vof1);
}

void launch_bc_ux(cudaStream_t s, const Grid &g, double *ux) { launch_pdl(k_bc_ux, (g.ny + 127) / 128, 128, 0, s, g, ux); }
void launch_bc_uy(cudaStream_t s, const Grid &g, double *uy) { launch_pdl(k_bc_uy, (g.ny + 127) / 128, 128, 0, s, g, uy); }
void launch_bc_neumann(cudaStream_t s, const Grid &g, double *f) {
  launch_pdl(k_bc_neumann, (g.ny + 127) / 128, 128, 0, s, g, f);
}
void launch_bc_vof(cudaStream_t s, const Grid &g, double *vof) {
  launch_pdl(k_bc_vof, (g.ny + 127) / 128, 128, 0, s, g, vof);
}

// ---------------------------------------------------------------------------
// the caller's host arrays <-> device fields, copied by the GPU itself over
// the CPU-GPU link (host memory the device can address: pageable memory on a
// system with host page-table access, or registered memory).  In: host rows
// J = 1..ny (x ghosts included) into the pitched device rows.  Out: every host
// row J = 1 - ay0 .. ny + ay1, the y ghost rows from their periodic images
// (what the reference's halo exchange leaves there, src/halo.c:18-76).  Case
// z of a batch is blockIdx.y: its arrays are tab[z * kLinkSlots + slot], its
// device rows start at dev + z * cs1.  Each thread keeps four loads in flight:
// the link's latency is microseconds.
template <bool kIn>
__global__ void __launch_bounds__(256) k_host_rows(Grid g, double *const *tab, HostRows a, HostRows b, int nf) {
  pdl_entry();
  const int z = blockIdx.y;
  const int stride = gridDim.x * blockDim.x;
  for (int q = 0; q < nf; ++q) {
    const HostRows f = q == 0 ? a : b;
    double *h = tab[(size_t)z * kLinkSlots + f.slot];
    double *dev = f.dev + (size_t)z * g.cs1;
    const int n = (kIn ? g.ny : g.ny + f.ay0 + f.ay1) * f.row;
    for (int t0 = blockIdx.x * blockDim.x + threadIdx.x; t0 < n; t0 += 4 * stride) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int t = t0 + u * stride;
        if (t >= n) break;
        const int r = t / f.row, i = t - r * f.row;
        // in: host row J = r + 1 (index r + ay0); out: host row index r holds J = r + 1 - ay0
        v[u] = kIn ? h[(size_t)(r + f.ay0) * f.row + i] : dev[(size_t)wrap(r - f.ay0 + 1, g.ny) * g.p1 + i];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int t = t0 + u * stride;
        if (t >= n) break;
        if (kIn) {
          const int r = t / f.row, i = t - r * f.row;
          dev[(size_t)r * g.p1 + i] = v[u];
        } else {
          h[t] = v[u];
        }
      }
    }
  }
}

void launch_host_rows(cudaStream_t s, const Grid &g, double *const *tab, bool in, HostRows a, HostRows b, int nf,
                      int width) {
  const dim3 grid(std::max(1, width / g.nc), g.nc);
  if (in)
    launch_pdl(k_host_rows<true>, grid, 256, 0, s, g, tab, a, b, nf);
  else
    launch_pdl(k_host_rows<false>, grid, 256, 0, s, g, tab, a, b, nf);
}

}  // namespace sbfs
