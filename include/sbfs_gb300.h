/*
 * GB300 implementation of the SimpleBubblyFlowSolver 2-D time step.
 *
 * Drop-in boundary: the entry points below carry the reference solver's
 * names, prototypes, argument meaning and error convention (0 = success,
 * non-zero = failure; the reference's caller aborts on failure,
 * src/main.c:118-120).  A program built against the reference's headers links
 * this library in place of the reference's src/integrate.c, src/decide_dt.c,
 * src/fluid/ and src/interface/ objects.  All computation runs in
 * hand-written sm_103a CUDA kernels on one GPU; there is no CPU fallback.
 *
 * Host buffers: every array_t.data is the caller's host buffer, exactly as in
 * the reference.  The fine-grained operators copy what they read to the GPU
 * and what they write back, so their observable effect on the structs equals
 * the reference's (including its pointer swaps of the RK sources and of the
 * scalar potentials).  integrate() keeps the whole step on the device; by
 * default it uploads the state (ux, uy, p, psi[0], vof) on entry and writes
 * it back on exit (see sbfs_set_sync_mode for the device-resident mode).
 *
 * Limits: NDIMS == 2; uniform x grid (as the reference requires,
 * src/domain.c:213-219); ny a power of two, 8 <= ny <= 8192; 4 <= nx <= 8192.
 */
#ifndef SBFS_GB300_H
#define SBFS_GB300_H

#include <stddef.h>
#include "sbfs_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- time integration (reference include/integrate.h:5-10, src/integrate.c:11-70) */
int integrate(const domain_t *domain, fluid_t *fluid, interface_t *interface, double *dt);

/* ---- time step size (reference include/decide_dt.h:5-10, src/decide_dt.c:140-169);
 * safety factors from the environment keys coef_dt_adv, coef_dt_dif,
 * coef_dt_int on first use, as the reference, unless sbfs_set_dt_coefs was called */
int decide_dt(const domain_t *domain, const fluid_t *fluid, const interface_t *interface, double *dt);

/* ---- fluid operators (reference include/fluid_solver.h:10-89) */
int fluid_compute_density(const domain_t *domain, fluid_t *fluid, const interface_t *interface, const size_t index);
int fluid_compute_viscosity(const domain_t *domain, fluid_t *fluid, const interface_t *interface);
int fluid_predict_field(const domain_t *domain, const size_t rkstep, const double dt, fluid_t *fluid,
                        const interface_t *interface);
int fluid_compute_potential(const domain_t *domain, const double dt_old, const double dt_new, fluid_t *fluid);
int fluid_correct_velocity(const domain_t *domain, const double dt_old, const double dt_new, fluid_t *fluid);
int fluid_update_pressure(const domain_t *domain, fluid_t *fluid);
int fluid_update_boundaries_ux(const domain_t *domain, array_t *array);
int fluid_update_boundaries_uy(const domain_t *domain, array_t *array);
int fluid_update_boundaries_p(const domain_t *domain, array_t *array);
int fluid_update_boundaries_psi(const domain_t *domain, array_t *array);

/* ---- interface operators (reference include/interface_solver.h:8-48) */
int interface_compute_curvature_tensor(const domain_t *domain, interface_t *interface);
int interface_compute_force(const domain_t *domain, const fluid_t *fluid, interface_t *interface);
int interface_compute_mass_flux(const domain_t *domain, const fluid_t *fluid, interface_t *interface);
int interface_update_vof(const domain_t *domain, const size_t rkstep, const double dt, const fluid_t *fluid,
                         interface_t *interface);
int interface_update_boundaries_vof(const domain_t *domain, array_t *vof);

/* ---- initialisation and .npy I/O (reference include/domain.h:32-42,
 * include/fluid_solver.h:10-22, include/interface_solver.h:8-18,
 * src/fileio.c:268-508): same file names, shapes and dtypes ('<f8', '<u8').
 * fluid_init reads Re, Fr, denr, visr and interface_init reads We from the
 * environment, as the reference.  domain_t.info is left NULL (one process). */
int domain_init(const char dirname_ic[], domain_t *domain);
int domain_save(const char dirname[], const domain_t *domain);
int fluid_init(const char dirname_ic[], const domain_t *domain, fluid_t *fluid);
int fluid_save(const char dirname[], const domain_t *domain, const fluid_t *fluid);
int interface_init(const char dirname_ic[], const domain_t *domain, interface_t *interface);
int interface_save(const char dirname[], const domain_t *domain, const interface_t *interface);
/* frees what domain_init / fluid_init / interface_init allocated (no
 * reference counterpart: the reference never frees) */
int sbfs_free_state(domain_t *domain, fluid_t *fluid, interface_t *interface);

/* ---- GB300 additions (no reference counterpart) */

/* what integrate() copies between host and device:
 *   SBFS_SYNC_STATE (default): upload ux, uy, p, psi[0], vof on entry; write
 *     them (and psi[1]) back on exit;
 *   SBFS_SYNC_ALL: as STATE, and also write back every other array the
 *     reference leaves filled (den, viscosities, stresses, sources, fluxes,
 *     interface geometry), as the steps taken in this mode leave them (the
 *     other modes keep some of them in their own form: viscosities
 *     pre-scaled, the next step's interface geometry formed ahead);
 *   SBFS_SYNC_NONE: device-resident; the state is uploaded on the first call
 *     (or after sbfs_invalidate_device) and stays on the GPU between calls;
 *     call sbfs_sync_to_host before reading host arrays and
 *     sbfs_invalidate_device after changing them. */
#define SBFS_SYNC_STATE 0
#define SBFS_SYNC_ALL 1
#define SBFS_SYNC_NONE 2
int sbfs_set_sync_mode(int mode);
int sbfs_sync_to_host(const domain_t *domain, fluid_t *fluid, interface_t *interface);
int sbfs_invalidate_device(void);

/* capture each time step into a CUDA graph (default 1) */
int sbfs_set_use_graphs(int on);

/* launch the step's kernels with programmatic dependent launch (default 1):
 * a kernel's blocks may start while the kernel before it on its stream
 * finishes, and wait on the GPU for its results.  Same results either way. */
int sbfs_set_pdl(int on);

/* interface-branch compaction (the corner-gradient and curvature work handed
 * to the first threads of each block, so that it fills whole warps): -1 (the
 * default) as the autotuner chose, else 0 off or 1 on for every context.
 * Same results either way, bit for bit. */
int sbfs_set_compaction(int mode);

/* launch the step's kernels at their streams' priorities (default 1): the
 * main and copy streams high, the side stream (decide_dt, the interface
 * geometry, the bulk fluxes) low, so that the GPU schedules the main stream's
 * blocks first and the side stream's where SMs are free; 0 launches all at
 * the default priority.  Same results either way, bit for bit.  (No
 * counterpart in the reference.) */
int sbfs_set_stream_priorities(int on);

/* where a grid solves its tridiagonal systems with four warps each, run the
 * four systems of a wavenumber pair as a cluster of four CTAs, one quarter
 * of the rows each, exchanging the chunk maps through distributed shared
 * memory (default 1); 0 keeps one block per pair or two.  Same results
 * either way, bit for bit.  (No counterpart in the reference.) */
int sbfs_set_tdm_cluster(int on);

/* run each substage's interface geometry ahead of its velocity (default 1):
 * curvature, the interface-cell list with the cells' THINC factors, and the
 * CSF force depend on vof alone, so they are formed beside the previous
 * substage's predictor and Poisson solve, and only the upwind choice and the
 * face fluxes wait for the corrected velocity; 0 forms them all after the
 * correction.  Same results either way, bit for bit.  (No counterpart in
 * the reference, whose src/integrate.c:11-70 runs its operators in turn.) */
int sbfs_set_geometry_ahead(int on);

/* In SBFS_SYNC_STATE mode, let the step copy the state itself (default 1):
 * when the GPU can address the caller's arrays (pageable host memory on a
 * system with host page-table access, such as Grace-Blackwell, or arrays
 * registered with cudaHostRegister), kernels inside the step read ux, uy, p,
 * psi[0] and vof from them and write the results back, each field as early as
 * the step allows, overlapped with the step's own kernels.  Otherwise the
 * state moves by cudaMemcpy before and after the step.  Same results either
 * way, bit for bit.  sbfs_host_link_used says whether the last integrate()
 * was host-linked.  on = 2 links registered arrays only, as on a system
 * without host page-table access. */
int sbfs_set_host_link(int on);
int sbfs_host_link_used(void);

/* safety factors of decide_dt, overriding the environment keys */
int sbfs_set_dt_coefs(double adv, double dif, double itf);

/* advance nsteps steps device-resident and time them with CUDA events on the
 * library's stream; *ms = elapsed milliseconds, *dt_last = last dt */
int sbfs_run_steps_timed(const domain_t *domain, fluid_t *fluid, interface_t *interface, int nsteps, float *ms,
                         double *dt_last);

/* kernels launched by one integrate() step (for launch accounting) */
int sbfs_kernels_per_step(void);

/* FP64 fused multiply-add throughput of the current GPU in GFLOP/s (the FP64
 * roofline denominator), from an 8-chain FMA loop timed with CUDA events */
int sbfs_measure_fp64_peak(double *gflops);

/* the library's Newton-Raphson reciprocal and inverse square root applied
 * to n host values on the GPU (accuracy test of the device helpers) */
int sbfs_check_newton_raphson(const double *x, double *rcp, double *rsq, int n);

/* select the CUDA device for the following calls (drops the current context) */
int sbfs_set_device(int device);

/* page-lock the state arrays integrate() copies (ux, uy, p, psi[0..1], vof)
 * so the host<->device copies run at full link speed; unpin before freeing.
 * A host-linked step captures its copies for the arrays' registration at the
 * time; these two calls (and sbfs_invalidate_device, for arrays the caller
 * registers or unregisters itself) make the next step look again. */
int sbfs_pin_host_state(fluid_t *fluid, interface_t *interface);
int sbfs_unpin_host_state(fluid_t *fluid, interface_t *interface);

/* per-kernel timing of nsteps device-resident steps launched eagerly with a
 * CUDA event pair around every launch on the library's stream;
 * ms_per_class[k] / launches_per_class[k] for k < sbfs_kernel_classes() */
int sbfs_kernel_classes(void);
const char *sbfs_kernel_name(int cls);
int sbfs_profile_steps(const domain_t *domain, fluid_t *fluid, interface_t *interface, int nsteps,
                       float *ms_per_class, int *launches_per_class);

/* ---- monitoring on the GPU (reference src/logging/ and src/statistics.c);
 * they read the device state (uploading the host state first unless the
 * device-resident mode holds it) */
typedef struct {
  double divmax;           /* max |div u|                 logging/divergence.c:41-64 */
  double vof_min, vof_max; /* extrema of vof              logging/interface.c:34-45 */
  double vof_integral;     /* sum vof J                   logging/interface.c:36-41 */
  double volume;           /* sum J */
  double interface_area;   /* sum |d vof| over faces      logging/interface.c:47-62 */
  double momentum[2];      /* sum rho u J                 logging/momentum.c:40-56 */
  double energy[2];        /* sum rho u^2 J / 2           logging/energy.c:42-58 */
  double umax[2];          /* max |ux|, max |uy|          logging/extrema.c:25-38 */
  double wall_stress[2];   /* nu sum txy at x = 0, lx     logging/stress.c:29-35 */
} sbfs_diagnostics_t;
int sbfs_diagnostics(const domain_t *domain, fluid_t *fluid, interface_t *interface, sbfs_diagnostics_t *out);
/* appends the reference's monitor lines (progress, divergence, momentum,
 * extrema, energy, stress, vof .dat; src/logging/main.c:90-108 and the line
 * formats of src/logging/{divergence,momentum,...}.c) to the files in dirname, from the device
 * reductions above; the progress line also goes to stdout */
int sbfs_logging_output(const char dirname[], const domain_t *domain, fluid_t *fluid, interface_t *interface,
                        size_t step, double time, double dt, double wtime);
/* running sums ux1, uy1, vof1 and their count (statistics.c:99-166) */
int sbfs_statistics_collect(const domain_t *domain, fluid_t *fluid, interface_t *interface);
int sbfs_statistics_reset(void);
/* host copies: ux1 (ny, nx+1), uy1 and vof1 (ny, nx+2), the reference's layout */
int sbfs_statistics_fetch(double *ux1, double *uy1, double *vof1, size_t *num);
/* writes num, ux1, uy1, vof1 and the domain into dirname as the reference's
 * statistics output does (statistics.c:174-216) */
int sbfs_statistics_output(const char dirname[], const domain_t *domain);

/* ---- decide_dt without allocation (no counterpart in the reference).
 * For callers that may not allocate GPU memory -- programs that hand out
 * device memory only from their own pre-sized pool, or that must not call
 * cudaMalloc/cudaFree while running because those calls synchronise the GPU
 * and take unbounded time.  The velocities are already on the GPU; the
 * kernels' scratch (per-column maxima, the least quotient and a block
 * counter) lives in a fixed
 * array inside the library (SBFS_NOALLOC_MAX_NX + 8 words, 64 KB, one copy on
 * every GPU that loads the library, kept until the process exits), so the
 * call allocates nothing.
 *   ux, uy  device arrays of ny rows with `pitch` doubles per row; row j
 *           holds UX(1..nx+1, j+1) and UY(0..nx+1, j+1) from column 0
 *   hxxf    device array HXXF(1..nx+1)
 *   scalars device array of SBFS_STEP_SCALARS doubles; [0] receives dt
 *   status  device int; bit 0 is set when a velocity is not finite
 *   stream  the cudaStream_t to run on (NULL: the legacy default stream)
 * The result is ready when the stream reaches it.  Set-up: the first call on
 * each GPU is where the CUDA runtime loads the library's device code there
 * (lazy module loading), which places the code and the scratch array in
 * device memory and may synchronise; make one warm-up call per GPU while
 * initialising, before any stream capture.  Later calls allocate nothing.
 * Every call shares the one array: calls that overlap on the GPU race and
 * give wrong results.  nx > SBFS_NOALLOC_MAX_NX is rejected.  Message of the
 * calling thread's last failure: sbfs_noalloc_last_error(). */
#define SBFS_NOALLOC_MAX_NX 8192
#define SBFS_STEP_SCALARS 64
int sbfs_decide_dt_noalloc(int nx, int ny, double lx, double ly, const double *ux, const double *uy, int pitch,
                           const double *hxxf, double Re, double denr, double visr, double We, double coef_adv,
                           double coef_dif, double coef_int, double *scalars, int *status, void *stream);
const char *sbfs_noalloc_last_error(void);

/* ---- batches of independent cases (no reference counterpart) ----
 * integrate() for n cases at once, each described by the reference's own
 * structs (any mix of grids and physics; every case steps with its own dt,
 * returned in dts[i]).  Cases on the same grid form a group whose fields hold
 * the cases side by side; each kernel of the step runs all cases of a group
 * in one launch, and groups run on separate streams.  The sync mode applies
 * as for integrate(); in SBFS_SYNC_NONE the cases stay on the device between
 * calls as long as the same fluid/interface pointers are passed in the same
 * order.  The curvature model (sbfs_set_curvature_model) applies to every
 * case of a batch. */
int sbfs_integrate_batch(int n, const domain_t *const *domains, fluid_t *const *fluids,
                         interface_t *const *interfaces, double *dts);
/* advance the device-resident batch nsteps steps; *ms from CUDA events */
int sbfs_run_batch_steps_timed(int nsteps, float *ms);
/* copy the device-resident batch back into the callers' structs */
int sbfs_batch_sync_to_host(int n, const domain_t *const *domains, fluid_t *const *fluids,
                            interface_t *const *interfaces);
/* per-kernel-class device time (ms) and launches of nsteps eager steps of
 * the resident batch (classes as sbfs_kernel_name) */
int sbfs_profile_batch_steps(int nsteps, float *ms_per_class, int *launches_per_class);
/* autotuner of the launch shapes (default off): when on, the first step of
 * each device context (the single case, every batch group) times candidate
 * block shapes of the stencil kernels, Poisson transform widths and
 * tridiagonal batching on the context's own state (restored after every
 * trial) and keeps the fastest per kernel; results do not change */
int sbfs_set_autotune(int on);
/* shapes in use (group -1: the single-case context): bx[7], by[7] for
 * props, curvature list, flux/force, vof advance, stress, predict,
 * correct; the Poisson transform width, wavenumbers per tridiagonal block
 * (0: one pair per cluster of four CTAs) and warps per tridiagonal system;
 * compact (may be NULL): 1 when the corner-gradient and curvature work is
 * compacted within blocks */
int sbfs_tiles(int group, int *bx, int *by, int *fft_w, int *tdm_mb, int *tdm_warps, int *compact);
/* number of grid groups and cases per group of the current batch */
int sbfs_batch_groups(int *ngroups, int *cases_per_group);
int sbfs_batch_release(void);

/* ---- learned curvature closure (no reference counterpart) ----
 * A 16 -> 64 -> 64 -> 1 ReLU perceptron mapping the 3x3 vof stencil of an
 * interface cell and the cell normal to kappa * dx, evaluated with BF16
 * tensor-core products (FP32 accumulate).  Feature row (16 bf16): the nine
 * stencil values (y rows bottom to top, x fastest), the unit cell normal
 * (x, y), five zeros.  Parameters: one FP32 vector of sbfs_mlp_nparams()
 * values [W1 (64 x 16, row-major), b1 (64), W2 (64 x 64), b2 (64), w3 (64),
 * b3].  X, Y, idx and out below are device pointers. */
int sbfs_mlp_nparams(void);
int sbfs_mlp_set_params(const float *host_params, int n); /* also resets Adam */
int sbfs_mlp_get_params(float *host_params, int n);
/* gradient (host, n params) and loss of the mean-square error over rows
 * idx[0..n) of X (bf16 [rows][16]) against Y */
int sbfs_mlp_gradient(const void *X, const float *Y, const int *idx, int n, float *grad_out, double *loss);
/* Adam steps over consecutive batches of the row permutation idx[0..n) */
int sbfs_mlp_train_epoch(const void *X, const float *Y, const int *idx, int n, int batch, float lr,
                         double *mean_loss);
int sbfs_mlp_predict(const void *X, int n, float *out);
/* 0: kappa = -div n (the reference, default); 1: the learned closure in
 * interface cells whose stencil is in range (centre vof in [0.01, 0.99], a
 * prediction |kappa dx| in the closure's range), plain kappa elsewhere.
 * Square cells.  Applies to integrate() and the timed runs. */
int sbfs_set_curvature_model(int model);
/* the closure's range in |kappa dx| (default [1/128, 0.5]: the training
 * circles' radii, 2 .. 128 cells) */
int sbfs_mlp_set_range(double lo, double hi);
/* interface cells that took the learned curvature since the last call */
int sbfs_mlp_take_usage(long long *used);
const char *sbfs_mlp_last_error(void);

/* device status bits: 1 = non-finite velocity seen by decide_dt */
int sbfs_device_status(int *status);

/* message of the last failure ("" if none) */
const char *sbfs_last_error(void);

/* release all device memory, streams and graphs of the library */
int sbfs_release(void);

#ifdef __cplusplus
}
#endif

#endif
