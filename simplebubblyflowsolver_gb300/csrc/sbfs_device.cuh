// Device-side data layout and helpers of the GB300 time step.
//
// Layout in HBM.  Every field is stored as ny rows (one per periodic y cell,
// J = 1..ny), x-fastest, with the same x extent and the same x index map as
// the reference's host arrays (include/array_macros/): element I of a field
// whose lower x ghost width is ax0 sits in column (I - 1 + ax0) (times the
// number of components for the AoS fields dvof and normal).  Rows are padded
// to a pitch that is a multiple of 32 doubles.  y ghost rows are not stored:
// y is periodic and every kernel wraps J (J = 0 -> ny, J = ny + 1 -> 1, ...),
// which replaces the reference's halo exchange (src/halo.c:18-76) without any
// copy.  x ghost cells are stored and written by the producing kernel.
//
// Metrics.  The reference writes its stencils for general x metrics but
// accepts uniform x grids only (src/domain.c:213-219); its Jacobians are
// JDXF = HXXF * hy and JDXC = HXXC * hy (src/domain.c:114-144).  The kernels
// use those identities to fold the metric factors of every stencil into one
// coefficient per column (the half cells at the walls keep their own HXXF),
// which changes the rounding of the reference's expressions, not their value.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sbfs {

// per-column coefficients, index = I (0..nx+2), built on the host
struct Metrics {
  const double *ihxxf;  // 1 / HXXF(I)          (faces)
  const double *ihxxc;  // 1 / HXXC(I)          (centres)
  const double *q4f;    // 0.25 / HXXF(I)       (ux advection in x)
  const double *q4fy;   // 0.25 HXXC / (HXXF(I) hy) (ux advection in y)
  const double *nuf;    // (1 / Re) / HXXF(I)   (ux diffusion in x)
  const double *hxxf;   // HXXF(I)              (decide_dt)
  const double *nuc;    // (1 / Re) / HXXC(I)   (uy diffusion in x)
  const double *q4c;    // 0.25 / HXXC(I)       (uy advection in x)
  const double *hihxxf; // 0.5 / HXXF(I)        (txy)
  const double *hihxxc; // 0.5 / HXXC(I)        (curvature)
  // momentum fluxes of the fused step (k_momflux)
  const double *rq;     // HXXC / HXXF(I)       (metric ratio of the ux advection along y)
  const double *c4nuc;  // 4 (1 / Re) / HXXC(I) (4 nu txx)
  const double *c2nuf;  // 2 (1 / Re) / HXXF(I) (4 nu txy)
  // the same with the viscosities pre-scaled (k_props<..., true>): c4nuc / nuy2
  // and c2nuf / nuy4, which no longer depend on the case
  const double *c4nucs;  // 2 hy / HXXC(I)
  const double *c2nufs;  // hy / (2 HXXF(I))
};

struct Grid {
  int nx, ny;
  int p1;  // pitch of scalar fields (doubles)
  int p2;  // pitch of dvof (2 doubles per element)
  int p3;  // pitch of normal (3 doubles per element)
  double hy, ihy;
  double dx, idx;  // uniform cell width HXXC and its inverse
  double q4y, hihy;  // 0.25 / hy, 0.5 / hy
  // batch of nc cases on this grid (the case is blockIdx.z; 1 for a single
  // case): element strides between cases of the scalar-pitched fields, of
  // dvof, of normal, of the Poisson spectrum (double2) and of the per-case
  // metric columns (nuf); per-case physics, or nullptr to use the kernel's
  // Phys argument
  int nc;
  int cm;
  size_t cs1, cs2, cs3, css;
  int ct;  // doubles per column table (nx + 2 rounded up; kColTabs x 3 tables per case)
  const struct Phys *phys;
};

// physical parameters of one case
struct Phys {
  double denr, visr, refden;
  double den_lo, den_hi, vis_lo, vis_hi;
  double grav;        // -1 / Fr / Fr
  double force_coef;  // 2 / (1 + denr) / We
  double irefden;     // 1 / refden
  double nu;          // 1 / Re
  double dtfix;       // diffusive / capillary bound of dt (batches: per case)
  double dm1;         // denr - 1
  double vm1, hvm1;   // visr - 1, (visr - 1) / 2
  double hgrav;       // grav / 2
  double rref2;       // 2 refden
  double nuy;         // nu / hy
  double qf, qfy;     // force_coef / 4, force_coef / 4 / hy
  double nuy2, nuy4;  // 2 nu / hy, 4 nu / hy (k_momflux)
  // the fused step's viscosities pre-scaled for k_momflux, visux by nuy2 and
  // visuy by nuy4: visr - 1, (visr - 1) / 2, 1 and the clip bounds scaled alike
  double vsx_c, vsx_c2, vsx_1, vsx_lo, vsx_hi;
  double vsy_c2, vsy_1, vsy_lo, vsy_hi;
  double inuy2, inuy4;  // 1 / nuy2, 1 / nuy4 (the wall stress from scaled sums)
};

// x / 2 for a positive normal x (x >= 2^-1021), exactly: the exponent field
// drops by one.  Integer work, so the FP64 pipe is not used.
__device__ __forceinline__ double half_pos_normal(double x) {
  return __longlong_as_double(__double_as_longlong(x) - (1LL << 52));
}

// pointer of case blockIdx.z in a batch (null stays null)
template <class T>
__device__ __forceinline__ T *zp(T *p, size_t stride) {
  return p ? p + (size_t)blockIdx.z * stride : p;
}
// physics of case blockIdx.z
__device__ __forceinline__ Phys zphys(const Grid &g, const Phys &ph) { return g.phys ? g.phys[blockIdx.z] : ph; }

// per-step scalars written by the time-step kernel and read by all others:
// [0] dt; for substage k: alpha_k dt, beta_k dt, gamma_k dt, dt_old_k,
// dt_new_k; the Poisson right-hand-side coefficients (already divided by
// 2 ny for the unnormalised real DFT pair) and the correction coefficients
constexpr int kScalars = 64;
__host__ __device__ constexpr int sc_adt(int k) { return 1 + 5 * k; }
__host__ __device__ constexpr int sc_bdt(int k) { return 2 + 5 * k; }
__host__ __device__ constexpr int sc_gdt(int k) { return 3 + 5 * k; }
__host__ __device__ constexpr int sc_dtold(int k) { return 4 + 5 * k; }
__host__ __device__ constexpr int sc_dtnew(int k) { return 5 + 5 * k; }
// rhs = pdx dux + pdy duy + pax X + pay Y (see k_poisson_fwd)
__host__ __device__ constexpr int sc_pdx(int k) { return 16 + 4 * k; }
__host__ __device__ constexpr int sc_pdy(int k) { return 17 + 4 * k; }
__host__ __device__ constexpr int sc_pax(int k) { return 18 + 4 * k; }
__host__ __device__ constexpr int sc_pay(int k) { return 19 + 4 * k; }
// correction: u -= cnew * ih * dpsi_new; u += cold * ih * e * dpsi_old
__host__ __device__ constexpr int sc_cnew(int k) { return 28 + 2 * k; }
__host__ __device__ constexpr int sc_cold(int k) { return 29 + 2 * k; }
// 2 alpha dt, 2 beta dt, 2 gamma dt (the predictor works on 2u)
__host__ __device__ constexpr int sc_adt2(int k) { return 34 + 3 * k; }
__host__ __device__ constexpr int sc_bdt2(int k) { return 35 + 3 * k; }
__host__ __device__ constexpr int sc_gdt2(int k) { return 36 + 3 * k; }
// the correction coefficients times 1 / hy
__host__ __device__ constexpr int sc_cnewy(int k) { return 43 + 2 * k; }
__host__ __device__ constexpr int sc_coldy(int k) { return 44 + 2 * k; }
// fused step: 2 gamma dt / hy (the uy pressure term), coldy / pay (the uy
// correction by the stored pay e grad psi_old), 2 rho_ref pax and 2 rho_ref
// pay (k_predict_mf stores e grad psi_old times pax at ux faces and times pay
// at uy faces: e pa = 2 rho_ref pa / (2 rho) - pa)
__host__ __device__ constexpr int sc_gdt2y(int k) { return 49 + k; }
__host__ __device__ constexpr int sc_coldyp(int k) { return 52 + k; }
__host__ __device__ constexpr int sc_rpx(int k) { return 55 + k; }
__host__ __device__ constexpr int sc_rpy(int k) { return 58 + k; }
// per-column coefficients of substage k (Bufs::coltab, kColTabs tables of
// Grid::ct doubles per substage, I = 0..nx+1), written with the scalars:
// 2 gamma dt / HXXF(I) (ux pressure term), cnew / HXXF(I) and (cold / pax) /
// HXXF(I) (ux correction by the stored pax e grad psi_old)
constexpr int kColTabs = 3;
__host__ __device__ constexpr int ct_gdt2x(int k) { return 3 * k; }
__host__ __device__ constexpr int ct_cnewx(int k) { return 3 * k + 1; }
__host__ __device__ constexpr int ct_coldx(int k) { return 3 * k + 2; }

// THINC constants (reference src/interface/common.c:4-14)
constexpr double kGaussPt = 0.2886751345948129;
constexpr double kVofMin = 1.e-8;

// programmatic dependent launch: every kernel of the step starts here and
// waits until the kernel before it on the stream has completed and its
// writes are visible.  The next kernel's launch is prepared while this one
// runs and its blocks start as this one's last blocks exit (the implicit
// trigger).  An explicit early trigger (griddepcontrol.launch_dependents at
// entry) was slower: 1% on the 2048 x 1024 swarm, 12% on the 256 x 128
// bubble, its waiting blocks sharing the SMs with an FP64-bound kernel.  A
// kernel launched without the attribute passes the wait at once.
__device__ __forceinline__ void pdl_entry() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// periodic row of J (J may be -1 .. ny + 2)
__device__ __forceinline__ int wrap(int J, int ny) {
  int r = J - 1;
  r += (r < 0) ? ny : 0;
  r -= (r >= ny) ? ny : 0;
  return r;
}

// bit-level helpers: sign and threshold tests on the integer pattern of a
// double keep these comparisons off the FP64 pipe
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// x < t for a positive threshold t: holds iff the signed bit pattern is
// smaller (negative doubles have negative patterns, positive ones are ordered)
__device__ __forceinline__ bool lt_pos(double x, double t) { return dbits(x) < dbits(t); }
__device__ __forceinline__ bool gt_pos(double x, double t) { return dbits(x) > dbits(t); }

// vof outside the interface band (phi < vofmin or 1 - vofmin < phi),
// reference src/interface/curvature_tensor.c:67 and update/fluxx.c:58
__device__ __forceinline__ bool single_phase(double phi) {
  return lt_pos(phi, kVofMin) || gt_pos(phi, 1. - kVofMin);
}

// clip(v, lo, hi) for 0 < lo <= hi as integer compares (exact fmax/fmin)
__device__ __forceinline__ double clip_pos(double v, double lo, double hi) {
  v = lt_pos(v, lo) ? lo : v;
  v = gt_pos(v, hi) ? hi : v;
  return v;
}

// vel < 0. as in the reference upwind choice (false for -0.)
__device__ __forceinline__ bool neg(double v) {
  const long long b = dbits(v);
  return b < 0 && (b << 1) != 0;
}

// 1 / x for finite normal x > 0 (or < 0): the hardware seed
// rcp.approx.ftz.f64 refined by one third-order step r <- r (1 + e + e^2),
// e = 1 - x r (1/x = r / (1 - e); the truncated series leaves e^3, about
// 2^-69 from the seed's 2^-23); result within an ulp or so of the correctly
// rounded reciprocal, two FP64 FMAs instead of a division.
__device__ __forceinline__ double rcp_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.);
  return fma(r, fma(e, e, e), r);
}

// 1 / sqrt(s) for finite normal s > 0: rsqrt.approx.ftz.f64 seed and one
// third-order step y <- y (1 + e/2 + 3e^2/8), e = 1 - s y^2 (the series of
// (1 - e)^(-1/2) truncated after e^2): five FP64 operations
__device__ __forceinline__ double rsqrt_nr(double s) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(s));
  const double e = fma(-(s * y), y, 1.);
  return fma(y * e, fma(e, 0.375, 0.5), y);
}

// 1 / max(sqrt(s), eps) with eps = DBL_EPSILON (the reference normalises a
// gradient by 1 / fmax(|g|, DBL_EPSILON), curvature_tensor.c:43, 87)
__device__ __forceinline__ double inv_norm(double s) {
  constexpr double eps = 2.220446049250313080847e-16;
  return lt_pos(s, eps * eps) ? 1. / eps : rsqrt_nr(s);
}

}  // namespace sbfs
