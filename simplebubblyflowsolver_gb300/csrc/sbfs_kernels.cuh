// Kernel declarations and the device-buffer bundle shared by the host code.
#pragma once

#include "sbfs_device.cuh"

namespace sbfs {

// device pointers of one case; every scalar field uses pitch Grid::p1,
// dvof uses Grid::p2 and normal Grid::p3 (doubles)
// launch shapes of the fused step, picked by the autotuner (sbfs_api.cu) or
// the defaults below; results do not depend on them (every cell, column
// and mode is computed independently of its block)
// (TK_FORCE: k_csf_force, the force alone when the geometry runs ahead)
enum TileKernel {
  TK_PROPS, TK_CURV_LIST, TK_FLUX_FORCE, TK_VOF_ADVANCE, TK_MOMFLUX, TK_PREDICT, TK_CORRECT, TK_FORCE, TK_COUNT
};
struct Tiles {
  unsigned short bx[TK_COUNT], by[TK_COUNT];  // block shape (bx * by <= 256)
  int fft_w;   // columns per block of the Poisson transforms: 1, 2, 4 or 8
  int tdm_mb;  // wavenumbers per block of the tridiagonal solves (0: by size)
  int tdm_g;   // warps per tridiagonal system: 1, 2 or 4 (tdm_g * tdm_mb <= 4), set by
               // tdm_warps_for from the grid (it changes the rounding, so it is not tuned)
  int compact;  // 1: the FP64 work of the corner-gradient and curvature branches is
                // compacted to the first threads of each block; 0: done in place
  int tdm_cl;   // 1: at tdm_g = 4 the tridiagonal solves run as clusters of four CTAs per
                // wavenumber pair (k_poisson_tdm_cl, the same bits as one block per pair)
};
Tiles default_tiles(int ny);

// THINC factor tables per listed interface cell (Bufs::tf)
constexpr int kThincTabs = 6;

struct Bufs {
  // state
  double *ux, *uy, *p, *psi0, *psi1, *vof;
  // second velocity buffers (predictor output) for the fused step
  double *ux_star, *uy_star;
  // properties and interface geometry
  double *den0, *den1, *visux, *visuy, *txx, *txy, *tyy;
  double *dvof, *normal, *curv, *ifrcx, *ifrcy;
  // fluxes: vof fluxes (also the reference's fluxx/fluxy) and mass fluxes
  double *fluxx, *fluxy, *mfluxx, *mfluxy;
  // RK sources
  double *srcux[3], *srcuy[3], *srcvof[2];
  // momentum fluxes of the fused step (k_momflux): 4 nu txx - C and 4 nu tyy - E
  // at cell centres, the ux and uy fluxes 4 nu txy - r D at the corners
  double *pxx, *pyy, *pxy, *pyx;
  // e grad psi_old at the ux and uy faces, e = rho_ref / rho^{k+1} - 1: the
  // variable-density part of the Poisson right-hand side and of the correction
  double *egx, *egy;
  // the fused step's Poisson right-hand side at the faces, pd u* + e grad
  // psi_old (k_predict_mf writes them, the transform differences them)
  double *qx, *qy;
  // the fused step's 2 rho at the faces (the last predictor's den1 sums) and
  // psi's differences across the faces (the last correction's), which the
  // next substage's predictor reads instead of forming them again
  double *rhofx, *rhofy, *dpsix, *dpsiy;
  // Poisson: spectrum [nx][ny/2+1] complex, Thomas factors, twiddles
  double2 *spec;
  double2 *tdm_fac[3];  // (w, v, P, Q) per row for 1, 2, 4 warps per system, see k_poisson_tdm
  double *tdm_stage;    // systems of k_poisson_tdm when they exceed shared memory (else null)
  double2 *twiddle;  // exp(-2 pi i m / ny), m = 0..ny/2
  // decide_dt accumulators and per-step scalars
  unsigned long long *dt_acc;  // [0..nx+1] column max |ux| bits, [nx+2] max |uy| bits, [nx+3] block counter
  double *scalars;             // kScalars doubles
  double *coltab;              // per-column coefficients (3 kColTabs tables of Grid::ct doubles a case)
  int *status;                 // device error word
  // interface cells of the current substage (linear index (J-1)*nx + I-1) and their count;
  // the faces those cells are upwind of (4 * cell + face, face 0..3 = left, right, bottom, top)
  // and their count (fcount = icount + nc)
  int *ilist, *icount;
  int *flist, *fcount;
  // THINC factors of the interface cells (kThincTabs planar tables of nx * ny
  // entries a case, by cell index; k_curv_list<false>), read by k_face_flux
  double *tf;
  // the second vof buffer: the geometry-ahead step writes vof^{k+1} there
  // (the host code then swaps it with vof, which always holds the current vof)
  double *vof_alt;
  // second CSF force buffers: the force of the next substage is formed
  // beside the predictor that reads this one's
  double *ifrcx2, *ifrcy2;
  // third CSF force buffers: the first substage's force when the previous
  // step formed it (device-resident steps)
  double *ifrcx3, *ifrcy3;
  // launch shapes (host side)
  Tiles tiles;
};

// ---- launch helpers (defined in sbfs_kernels.cu), all on stream `s`
// scaled: the fused step's viscosities, pre-scaled for k_momflux (k_props<..., true>)
void launch_props(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                  bool den, bool vis, bool grad, double *den_out, bool scaled = false);
// store_k: normal[2] = 1/phi - 1 (fused step) instead of the intercept
void launch_normal_curv(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, bool normal, bool curv,
                        bool store_k);
// have_k: normal[2] holds 1/phi - 1 instead of the intercept
void launch_flux_force(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                       const double *ux, const double *uy, const double *den0, bool flux, bool force, bool have_k);
// fused interface stage: 0 = curvature + interface-cell list, 1 = dense THINC
// fluxes of the listed cells, 2 = bulk fluxes and the CSF force, 3 = as 2
// with the face curvature taken from the interface side (learned curvature)
void launch_interface_stage(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                            const double *ux, const double *uy, const double *den0, int stage);
// vof_out: vof^{k+1} there instead of in place (fused only)
void launch_vof_advance(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                        const double *sc, int k, double *src_a, const double *src_b, bool fused,
                        const double *ux, const double *uy, double *den1, double *vof_out = nullptr);
void launch_mass_flux_inplace(cudaStream_t s, const Grid &g, const Phys &ph, const Bufs &b,
                              const double *ux, const double *uy);
// the reference's txx, txy, tyy (fine-grained entry point)
void launch_stress(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, const double *ux, const double *uy);
// the reference's momentum right-hand sides and predictor from txx, txy, tyy
// and the mass fluxes (fine-grained entry point)
void launch_predict(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                    const double *sc, int k, const double *ux, const double *uy, double *ux_out, double *uy_out,
                    const double *mfx, const double *mfy, const double *den0, const double *den1,
                    double *srcux_a, const double *srcux_b, double *srcux_g,
                    double *srcuy_a, const double *srcuy_b, double *srcuy_g);
// fused step: the momentum fluxes of every centre and corner (b.pxx, b.pyy,
// b.pxy, b.pyx) from the velocity, the viscosities and the mass fluxes;
// stress = 1 also writes txy at the two wall columns (the wall-stress log
// reads it), 2 the whole of txx, txy, tyy
void launch_momflux(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                    const double *ux, const double *uy, int stress, bool scaled);
// fused step: the predictor from those fluxes and the CSF force ifx, ify;
// also writes e grad psi_old at the faces (b.egx, b.egy) for the correction
// and the Poisson right-hand side's face values (b.qx, b.qy)
void launch_predict_mf(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                       const double *sc, int k, const double *ux, const double *uy, double *ux_out, double *uy_out,
                       const double *den0, const double *den1, const double *psi_old, double *srcux_a,
                       const double *srcux_b, double *srcuy_a, const double *srcuy_b, const double *ifx,
                       const double *ify, bool cached);
// fused step with the interface geometry ahead of the velocity: curvature,
// interface-cell list and the cells' THINC factors from vof and the corner
// normals alone (counts reset first)
void launch_geometry(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b);
// the THINC fluxes of the faces the listed interface cells are upwind of
void launch_face_flux(cudaStream_t s, const Grid &g, const Bufs &b, const double *ux, const double *uy);
// the fluxes of every other face (upwind cell single-phase, walls)
void launch_bulk_flux(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                      const double *ux, const double *uy);
// the CSF force into ifx, ify (itf_kappa: the learned closure's face curvature)
void launch_csf_force(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                      const double *den0, double *ifx, double *ify, bool itf_kappa);
// the Poisson solve; the right-hand side reads b.egx, b.egy
void launch_poisson(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k, const double *ux,
                    const double *uy, double *psi_new);
void launch_poisson_fwd(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k, const double *ux,
                        const double *uy);
// fused step: the transform of the right-hand side from b.qx, b.qy
void launch_poisson_fwd_q(cudaStream_t s, const Grid &g, const Bufs &b, const double *sc, int k);
void launch_poisson_tdm(cudaStream_t s, const Grid &g, const Bufs &b);
void launch_poisson_inv(cudaStream_t s, const Grid &g, const Bufs &b, double *psi_new);
// velocity correction (+ pressure); reads b.egx, b.egy; dpsi: also stores
// psi_new's face differences (b.dpsix, b.dpsiy) for the next predictor
void launch_correct(cudaStream_t s, const Grid &g, const Metrics &m, const Bufs &b, const double *sc, int k,
                    double *ux, double *uy, const double *psi_new, bool pressure, bool dpsi);
void launch_pressure(cudaStream_t s, const Grid &g, const Bufs &b, const double *psi_new);
// decide_dt: the column and domain maxima, then the finishing kernel (dt, the
// scalars and, with a coltab, the column tables); acc holds nx + 8 zero
// words per case between launches
void launch_decide_dt(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const Bufs &b,
                      const double *ux, const double *uy, double dt_fixed, double coef_adv);
void launch_decide_dt_raw(cudaStream_t s, const Grid &g, const Metrics &m, const Phys &ph, const double *ux,
                          const double *uy, unsigned long long *acc, double *sc, int *status, double dt_fixed,
                          double coef_adv, double *coltab);
// e grad psi_old at the faces (b.egx, b.egy) from a density field and psi_old,
// as k_predict_mf stores it (fine-grained entry points)
void launch_face_factor(cudaStream_t s, const Grid &g, const Phys &ph, const Bufs &b, const double *den,
                        const double *psi_old);
// logging diagnostics (16 doubles, see k_diag_partial) and statistics sums
int diag_partial_blocks(const Grid &g);
void launch_diagnostics(cudaStream_t s, const Grid &g, const Metrics &m, const double *ux, const double *uy,
                        const double *vof, const double *den, const double *txy, double nu, double *part,
                        double *out);
void launch_stats_collect(cudaStream_t s, const Grid &g, const double *ux, const double *uy, const double *vof,
                          double *ux1, double *uy1, double *vof1);
// boundary kernels of the fine-grained entry points
void launch_bc_ux(cudaStream_t s, const Grid &g, double *ux);
void launch_bc_uy(cudaStream_t s, const Grid &g, double *uy);
void launch_bc_neumann(cudaStream_t s, const Grid &g, double *f);
void launch_bc_vof(cudaStream_t s, const Grid &g, double *vof);

// launches of the step kernels: programmatic stream serialisation, so that a
// kernel's blocks may start before the one before it on the stream ends (each
// kernel begins with pdl_entry, which waits for it); g_pdl = 0 launches
// them plainly
extern int g_pdl;
extern int g_compact;  // -1: per context (Tiles::compact), else 0 / 1 for all
// 1: each launch carries its stream's priority (the step's main and copy
// streams high, its side stream low), so that the block scheduler fills the
// SMs with the main stream's blocks first and the side stream's in the gaps;
// 0: every launch at the default priority.  Scheduling only: the same results
extern int g_stream_prio;
template <typename... P, typename... A>
void launch_pdl(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A &&...a) {
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = g_pdl ? 1 : 0;
  int prio = 0;
  if (g_stream_prio) cudaStreamGetPriority(s, &prio);
  at[1].id = cudaLaunchAttributePriority;
  at[1].val.priority = prio;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  cudaLaunchKernelEx(&cfg, k, static_cast<A &&>(a)...);
}

// smem budget checks (host side)
int poisson_fft_cols(int ny);
int poisson_tdm_modes(int nx);
int tdm_chunk(int nx, int G);
int tdm_group_index(int G);  // 1, 2, 4 -> 0, 1, 2
int tdm_warps_for(int nx, int ny, int nc);
int tdm_modes_per_block(const Tiles &t, int nx);
// the tridiagonal solves run as k_poisson_tdm_cl (switch g_tdm_cluster, tile choice tdm_cl, tdm_g = 4)
extern int g_tdm_cluster;
bool tdm_uses_cluster(const Tiles &t, int nx);
size_t poisson_tdm_smem(int nx, int mb, int G);
size_t poisson_fft_smem(int ny, int w);
bool fft_w_fits(int ny, int w);
size_t poisson_tdm_smem(int nx);
bool tdm_global_stage(int nx, int G);                   // k_poisson_tdm stages its systems in global memory
size_t tdm_stage_doubles(int nx, int ny, int nc, int G);  // size of Bufs::tdm_stage (0 if not staged)
cudaError_t configure_kernels();
// Newton-Raphson reciprocal / inverse square root of n device inputs (tests)
cudaError_t nr_check(const double *x, double *rcp, double *rsq, int n);
// FP64 FMA throughput of this GPU, GFLOP/s (2 flops per FMA)
cudaError_t measure_fp64_peak(double *gflops);
// learned curvature closure (sbfs_mlp.cu): parameters present, and the
// in-step kernel overwriting curv in the listed interface cells
bool mlp_ready();
void mlp_range(float *lo, float *hi);  // the closure's range in |kappa dx|
extern unsigned g_mlp_epoch;           // changes with the closure's parameters or range
void launch_mlp_curv(cudaStream_t s, const Grid &g, const Bufs &b);

// one scalar field between a host array of the reference's layout (tab[z *
// kLinkSlots + slot] for case z, rows of `row` doubles, ay0 / ay1 ghost rows)
// and its device field (pitch p1, case z at dev + z * cs1)
constexpr int kLinkSlots = 16;
struct HostRows {
  int slot, row, ay0, ay1;
  double *dev;
};
// nf (1 or 2) fields of every case, host -> device when in, else device ->
// host, on about `width` blocks (at least one per case)
void launch_host_rows(cudaStream_t s, const Grid &g, double *const *tab, bool in, HostRows a, HostRows b, int nf,
                      int width);

}  // namespace sbfs
