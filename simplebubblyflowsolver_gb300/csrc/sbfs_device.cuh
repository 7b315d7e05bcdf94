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
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sbfs {

// per-column coefficients, evaluated on the host with the reference's own
// expressions (hence the reference's rounding); index = I (0..nx+2)
struct Metrics {
  const double *ihxxf;     // 1 / HXXF(I)
  const double *ihxxc;     // 1 / HXXC(I)
  const double *ijdxf;     // 1 / JDXF(I)
  const double *ijdxc;     // 1 / JDXC(I)
  const double *qf;        // JDXF(I) / HXXF(I)
  const double *qc;        // JDXC(I) / HXXC(I)
  const double *qf_hy;     // JDXF(I) / hy
  const double *qc_hy;     // JDXC(I) / hy
  const double *hqf;       // 0.5 * JDXF(I) / HXXF(I)
  const double *hqc_hy;    // 0.5 * JDXC(I) / hy
  const double *nu_ijdxf;  // (1 / Re) / JDXF(I)
  const double *nu_ijdxc;  // (1 / Re) / JDXC(I)
  const double *hxxf;      // HXXF(I)
};

struct Grid {
  int nx, ny;
  int p1;  // pitch of scalar fields (doubles)
  int p2;  // pitch of dvof (2 doubles per element)
  int p3;  // pitch of normal (3 doubles per element)
  double hy, ihy;
};

// physical parameters of one case
struct Phys {
  double denr, visr, refden;
  double den_lo, den_hi, vis_lo, vis_hi;
  double grav;        // -1 / Fr / Fr
  double force_coef;  // 2 / (1 + denr), times 1 / We applied separately
  double tension;     // 1 / We
  double irefden;     // 1 / refden
};

// per-step scalars written by the time-step kernel and read by all others:
// [0] dt; for substage k: [1+5k] alpha_k dt, [2+5k] beta_k dt, [3+5k] gamma_k dt,
// [4+5k] dt_old_k, [5+5k] dt_new_k; [16..21] Poisson/correction factors:
// [16+2k] refden / dt_new_k / ny, [17+2k] -dt_old_k / dt_new_k / ny
// [22+2k] dt_new_k / refden, [23+2k] -dt_old_k
constexpr int kScalars = 32;
__host__ __device__ constexpr int sc_adt(int k) { return 1 + 5 * k; }
__host__ __device__ constexpr int sc_bdt(int k) { return 2 + 5 * k; }
__host__ __device__ constexpr int sc_gdt(int k) { return 3 + 5 * k; }
__host__ __device__ constexpr int sc_dtold(int k) { return 4 + 5 * k; }
__host__ __device__ constexpr int sc_dtnew(int k) { return 5 + 5 * k; }
__host__ __device__ constexpr int sc_pdiv(int k) { return 16 + 2 * k; }
__host__ __device__ constexpr int sc_padd(int k) { return 17 + 2 * k; }
__host__ __device__ constexpr int sc_cnew(int k) { return 22 + 2 * k; }
__host__ __device__ constexpr int sc_cold(int k) { return 23 + 2 * k; }

// THINC constants (reference src/interface/common.c:4-14)
constexpr double kGaussPt = 0.2886751345948129;
constexpr double kVofMin = 1.e-8;

// periodic row of J (J may be -1 .. ny + 2)
__device__ __forceinline__ int wrap(int J, int ny) {
  int r = J - 1;
  r += (r < 0) ? ny : 0;
  r -= (r >= ny) ? ny : 0;
  return r;
}

// scalar field accessor: x offset ox = ax0 - 1 so that column = I + ox
template <int OX>
struct Fld {
  double *d;
  int pitch;
  __device__ __forceinline__ double &at(int I, int row) const { return d[(size_t)row * pitch + (I + OX)]; }
};

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

// vel < 0. as in the reference upwind choice: true for negative numbers,
// false for +0 and -0
__device__ __forceinline__ bool neg(double v) { return v < 0.; }

}  // namespace sbfs
