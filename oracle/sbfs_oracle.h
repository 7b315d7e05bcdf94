/*
 * CPU oracle: a project-written C restatement of the reference solver's
 * 2-D time step (SimpleBubblyFlowSolver src/integrate.c and everything it
 * calls), operating on the reference's own data structures (sbfs_types.h).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load it, and only as the checker or the timed
 * CPU baseline -- never as part of the product path.
 *
 * Every entry point mirrors the reference function of the same name without
 * the "orc_" prefix, with the same argument meaning, the same in-place
 * updates and the same pointer swaps, and returns 0 on success.
 */
#ifndef SBFS_ORACLE_H
#define SBFS_ORACLE_H

#include <stddef.h>
#include "sbfs_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* safety factors of decide_dt (reference env keys coef_dt_adv/dif/int) */
void orc_set_dt_coefs(double adv, double dif, double itf);
int orc_decide_dt(const domain_t *domain, const fluid_t *fluid, const interface_t *interface, double *dt);
int orc_integrate(const domain_t *domain, fluid_t *fluid, interface_t *interface, double *dt);

int orc_fluid_compute_density(const domain_t *domain, fluid_t *fluid, const interface_t *interface, size_t index);
int orc_fluid_compute_viscosity(const domain_t *domain, fluid_t *fluid, const interface_t *interface);
int orc_fluid_predict_field(const domain_t *domain, size_t rkstep, double dt, fluid_t *fluid, const interface_t *interface);
int orc_fluid_compute_potential(const domain_t *domain, double dt_old, double dt_new, fluid_t *fluid);
int orc_fluid_correct_velocity(const domain_t *domain, double dt_old, double dt_new, fluid_t *fluid);
int orc_fluid_update_pressure(const domain_t *domain, fluid_t *fluid);
int orc_fluid_update_boundaries_ux(const domain_t *domain, array_t *array);
int orc_fluid_update_boundaries_uy(const domain_t *domain, array_t *array);
int orc_fluid_update_boundaries_p(const domain_t *domain, array_t *array);
int orc_fluid_update_boundaries_psi(const domain_t *domain, array_t *array);

int orc_interface_compute_curvature_tensor(const domain_t *domain, interface_t *interface);
int orc_interface_compute_force(const domain_t *domain, const fluid_t *fluid, interface_t *interface);
int orc_interface_compute_mass_flux(const domain_t *domain, const fluid_t *fluid, interface_t *interface);
int orc_interface_update_vof(const domain_t *domain, size_t rkstep, double dt, const fluid_t *fluid, interface_t *interface);
int orc_interface_update_boundaries_vof(const domain_t *domain, array_t *vof);

/* diagnostics with the formulas of reference src/logging/divergence.c:41-64
 * and src/logging/interface.c:34-65: max |div u|; vof min, max, volume
 * integral sum(vof*J) and sum(J) */
int orc_max_divergence(const domain_t *domain, const fluid_t *fluid, double *divmax);
int orc_vof_stats(const domain_t *domain, const interface_t *interface, double out[4]);

/* every quantity of the reference's log files, see sbfs_diagnostics_t */
int orc_diagnostics(const domain_t *domain, const fluid_t *fluid, const interface_t *interface, double out[16]);

/* number of OpenMP threads the oracle uses (0 = library default) */
void orc_set_threads(int nthreads);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
