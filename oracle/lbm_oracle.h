/*
 * lbm_oracle.h -- CPU restatement of the reference LBM hot path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline arm as the oracle.  Never linked by the product.
 *
 * All arrays are FP64 in DMDA order (cell c = (z*ny+y)*nx+x, AoS c*Q+q).
 * Return 0 on success, negative on error.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stdint.h>

#include "../include/lbmgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

int orc_sizes(const lbm_config* cfg, int64_t* ncell, int* npop, int* nmac);
int orc_init(const lbm_config* cfg, const double* macros, double* f0);
/* f holds f_{t0} on entry and f_{t0+nsteps} on exit. */
int orc_forward_from(const lbm_config* cfg, const double* gamma, double* f, int t0, int nsteps,
                     double* J_steps, double* J_sum);
int orc_forward(const lbm_config* cfg, const double* gamma, const double* macros, int nsteps,
                double* f_out, double* J_steps, double* J_sum);
/* One reverse step at f_t; lam (adjoint of the post-collision state of step t)
 * is replaced by the one of step t-1; sens accumulates. */
int orc_adjoint_step(const lbm_config* cfg, const double* gamma, const double* f_t, int t,
                     double* lam, double* sens);
int orc_gradient(const lbm_config* cfg, const double* gamma, const double* macros, int nsteps,
                 double* J_sum, double* sens);
/* Steady phase without objective, then n_unsteady steps with it; the reverse sweep
 * through both (the library's lbm_gradient_steady). */
int orc_gradient_steady(const lbm_config* cfg, const double* gamma, const double* macros,
                        int max_steady, int check_every, double tol, int n_unsteady,
                        double* J_sum, double* sens, int* steady_steps);
/* Phase of the calls that follow: LBM_TIME_RAMP ramps start after step t_phase
 * (2147483647 = never), the objective counts steps >= obj_from (default 1). */
int orc_set_phase(int t_phase, int obj_from);
int orc_macros(const lbm_config* cfg, const double* f, double* mac);
int orc_collide_cell(const lbm_config* cfg, const double* fin, double gamma, double* fout,
                     double* mac);
int orc_reverse_cell(const lbm_config* cfg, const double* fin, double gamma,
                     const double* lam_out, double* lam_in, double* dgamma);
int orc_objective(const lbm_config* cfg, const double* f, const double* gamma, double* J);
/* The boundary conditions of step t (t >= 1; none at t = 0) applied in place to f. */
int orc_apply_bcs(const lbm_config* cfg, int t, double* f);
int orc_wang_count(int nsteps, int nsnap, int64_t* recomputed, int* ok);
int orc_static_count(int nsteps, int nsnap, int64_t* recomputed, int* ok, int* saved);
/* Wall time of nsteps forward and nsteps reverse steps on nthreads threads (0 = all). */
int orc_time_steps(const lbm_config* cfg, const double* gamma, int nsteps, int nthreads,
                   double* sec_fwd, double* sec_adj);
int orc_max_threads(void);
/* Table of boundary slot k for configs whose boundary k has LBM_PROFILE_TABLE
 * (the library's lbm_set_bc_profile): nt rows of npos cells of ncomp values;
 * table = NULL clears the slot.  Process-wide, like the test that sets it. */
int orc_set_bc_profile(int k, int nt, int ncomp, int64_t npos, const double* table);

#ifdef __cplusplus
}
#endif

#endif
