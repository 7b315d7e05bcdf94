// decide_dt for callers that cannot allocate GPU memory.
//
// Some host programs own every byte of the GPU themselves: a coupled solver
// that hands out device memory only from its own pre-sized arena, or a
// program that must not call cudaMalloc / cudaFree once it is running
// because those calls synchronise the device and take unbounded time.  Such
// a caller already holds the velocity fields on the GPU and only needs the
// time step.  This entry point runs the library's decide_dt kernels on the
// caller's device arrays with their scratch (the per-column maxima of |ux|,
// the |uy| maximum, the least quotient and a block counter) taken from a
// fixed array in the library's own device image, so nothing is allocated.
//
// The scratch array is sized for nx <= SBFS_NOALLOC_MAX_NX; it exists once
// per GPU that loads the library and stays there until the process exits.
// Every call uses the same array: calls that overlap on the GPU (issued on
// streams without an order between them) race on it and give wrong results.
//
// Set-up: the first call on each GPU is where the CUDA runtime loads this
// file's device code onto that GPU (with the default lazy module loading);
// loading places the code and the scratch array in device memory and may
// synchronise.  A caller that must not see that mid-run makes one warm-up
// call per GPU while it initialises, before any stream capture.  Every call
// looks the array's device address up again (a host-side lookup that
// allocates nothing once the code is loaded), so an address never outlives
// the context it belongs to (after cudaDeviceReset the code is loaded anew,
// possibly elsewhere).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "sbfs_gb300.h"
#include "sbfs_kernels.cuh"

using namespace sbfs;

namespace {

// per-column maxima (nx + 2 words), the |uy| maximum, the least quotient
// and the block counter (words nx + 2 .. nx + 5)
constexpr int kScratchWords = SBFS_NOALLOC_MAX_NX + 8;
static __device__ __align__(256) unsigned long long g_dt_scratch[kScratchWords];

// message of this thread's last failure (threads driving different GPUs do
// not overwrite each other's)
thread_local char g_last_error[256];

int report(const char *msg, cudaError_t e) {
  snprintf(g_last_error, sizeof(g_last_error), "%s%s%s", msg, e == cudaSuccess ? "" : ": ",
           e == cudaSuccess ? "" : cudaGetErrorString(e));
  return 1;
}

}  // namespace

extern "C" const char *sbfs_noalloc_last_error(void) { return g_last_error; }

extern "C" int sbfs_decide_dt_noalloc(int nx, int ny, double lx, double ly, const double *ux, const double *uy,
                                      int pitch, const double *hxxf, double Re, double denr, double visr, double We,
                                      double coef_adv, double coef_dif, double coef_int, double *scalars, int *status,
                                      void *stream) {
  g_last_error[0] = '\0';
  if (nx < 2 || ny < 1) return report("sbfs_decide_dt_noalloc: grid must have nx >= 2 and ny >= 1", cudaSuccess);
  if (nx > SBFS_NOALLOC_MAX_NX)
    return report("sbfs_decide_dt_noalloc: nx exceeds SBFS_NOALLOC_MAX_NX (the size of its fixed scratch array)",
                  cudaSuccess);
  if (pitch < nx + 2) return report("sbfs_decide_dt_noalloc: pitch must be at least nx + 2 doubles", cudaSuccess);
  if (!ux || !uy || !hxxf || !scalars || !status)
    return report("sbfs_decide_dt_noalloc: null device pointer", cudaSuccess);
  // host code may not use g_dt_scratch as an address: the runtime gives the
  // device address of the current GPU's copy (on the first call on a GPU this
  // also loads the module, see above)
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_dt_scratch);
  if (e != cudaSuccess) return report("sbfs_decide_dt_noalloc: cudaGetSymbolAddress", e);
  unsigned long long *scratch = static_cast<unsigned long long *>(p);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the kernel needs zeroed accumulators; the array keeps the last call's words
  e = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * (nx + 6), s);
  if (e != cudaSuccess) return report("sbfs_decide_dt_noalloc: clearing the scratch", e);
  Grid g{};
  g.nc = 1;
  g.nx = nx;
  g.ny = ny;
  g.p1 = pitch;
  g.hy = ly / ny;
  g.ihy = 1. / g.hy;
  g.dx = lx / nx;
  g.idx = 1. / g.dx;
  Metrics m{};
  m.hxxf = hxxf - 1;  // the kernel indexes HXXF(I) by I = 1..nx+1
  Phys ph{};
  ph.refden = fmin(1., denr);
  ph.irefden = 1. / ph.refden;
  // diffusive and capillary limits (reference src/decide_dt.c:79-130)
  const double pi = 3.1415926535897932384626433832;
  // on the uniform x grid the interior face spacing is lx / nx (the host
  // entry point takes the minimum of HXXF, equal to it up to rounding)
  const double h[2] = {lx / nx, ly / ny};
  double dt_fixed = 1.e300;
  for (int d = 0; d < 2; ++d)
    dt_fixed = fmin(dt_fixed, fmin(1., denr / visr) / (1. / Re) * 0.5 / 2 * pow(h[d], 2.) * coef_dif);
  double cap = 1.;
  for (int d = 0; d < 2; ++d) cap = fmin(cap, sqrt(1. / (1. / We) / 4. / pi * pow(h[d], 3.)));
  dt_fixed = fmin(dt_fixed, cap * coef_int);
  Bufs b{};
  b.dt_acc = scratch;
  b.scalars = scalars;
  b.status = status;
  launch_decide_dt(s, g, m, ph, b, ux, uy, dt_fixed, coef_adv);
  e = cudaGetLastError();
  if (e != cudaSuccess) return report("sbfs_decide_dt_noalloc: kernel launch", e);
  return 0;
}
