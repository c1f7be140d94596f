/*
 * lbmgpu.h -- C ABI of the GB300 forward/adjoint lattice-Boltzmann library.
 *
 * One opaque handle owns one lattice (its populations, design field gamma,
 * adjoint populations, FP64 sensitivity field and checkpoint slots) resident
 * in device memory.  A handle is single-threaded, like one PETSc rank of the
 * reference.  Every entry point returns an int status: LBM_OK (0) on
 * success, a negative LBM_ERR_* code otherwise; lbm_last_error() gives the
 * text.  Host arrays crossing this boundary are FP64 in the reference's
 * DMDA order: cell index c = (z*ny + y)*nx + x (x fastest) and, for
 * per-cell vectors, AoS element c*Q + q with the reference's lattice
 * numbering (D2Q9 / D3Q19 / D2Q5 of latticeBoltzmann/lattices{2,3}d.hh).
 *
 * Time-step convention (the reference applications' driver loop, e.g.
 * applications/RobustPump2d/robustPump2d.cc:234-249):
 *   f_0 = feq(initial macros)                       (initializeAtEquilibrium)
 *   f_{t+1} = BC_{t+1}( stream( collide(f_t) ) )     (collide(); stream())
 *   J = sum_{t=1..N} F(macros(f_t))                  (computeMacroFunctional)
 * and the reverse sweep for t = N..1 (robustPump2d.cc:268-276):
 *   adjointCollide(f_t); computeCollideSource(f_t); adjointStream().
 * The "state" a handle holds is f_t: post-stream, post-boundary,
 * pre-collision populations.
 */
#ifndef LBMGPU_H
#define LBMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBMGPU_ABI_VERSION 2
#define LBM_MAX_BC 8
#define LBM_MAX_BATCH 8   /* lattices advanced by one batched launch */

/* Status codes.  PETSc's PetscErrorCode is 0 = ok; the reference's
 * "unsupported" case (PETSC_ERR_SUP, boundaryConditions/LBBoundaryLoop.cc:32-38)
 * maps to LBM_ERR_SUP. */
#define LBM_OK             0
#define LBM_ERR_ARG       -1  /* bad argument: null pointer, bad size, bad box */
#define LBM_ERR_SUP       -2  /* combination not supported */
#define LBM_ERR_CUDA      -3  /* CUDA runtime error, or no CUDA device */
#define LBM_ERR_MEM       -4  /* device or host allocation failed */
#define LBM_ERR_STATE     -5  /* call out of order (e.g. no design set) */
#define LBM_ERR_NONFINITE -6  /* NaN/Inf detected in inputs or results */

/* Lattices (latticeBoltzmann/lattices2d.hh:16-62, lattices3d.hh:141-160). */
#define LBM_D2Q9        0
#define LBM_D3Q19       1
#define LBM_D2Q9_D2Q5   2   /* flow D2Q9 + temperature D2Q5 (double distribution) */

/* Collision operators of the flow lattice. */
#define LBM_BGK 0   /* IncompressibleBGK2d (dynamics/incompressibleBGK2d.hh:94-153) */
#define LBM_MRT 1   /* IncompressibleMRT2d / IncompressibleMRT3d (dynamics/MRT3d.hh:28-200) */

/* Population storage in device memory.  Compute precision is FP64 for
 * LBM_STORE_FP64 and FP32 for the two shifted forms, which store the
 * deviation f_i - w_i. */
#define LBM_STORE_FP64 0
#define LBM_STORE_FP32 1
#define LBM_STORE_FP16 2

/* Boundary condition kinds (applied after streaming on the boundary box).
 * Faces per kind, 2D (D2Q9 and the flow part of the thermal lattice):
 *   LBM_BC_VELOCITY  west, east, north (IncompressibleZouHeVelocityWest/East/
 *                    North2d, ZouHe2d.hh:23-133) and south (the mirror image of
 *                    north; no reference counterpart)
 *   LBM_BC_PRESSURE  west, east (IncompressibleZouHePressureWest/East2d,
 *                    ZouHe2d.hh:241-321) and north, south (the east/west
 *                    operator rotated onto the y faces; no reference counterpart)
 *   LBM_BC_VELOCITY_STANDARD  west (StandardZouHeVelocityWest2d, ZouHe2d.hh:139-178):
 *                    the standard-equilibrium density rho = (...)/(1 - ux)
 *   LBM_BC_PRESSURE_STANDARD  west, east (StandardZouHePressureWest/East2d,
 *                    ZouHe2d.hh:325-391)
 *   LBM_BC_TEMPERATURE west (ThermalZouHeWest2d<.,D2Q5,.>, thermalZouHe2d.hh:63-97)
 * 3D (D3Q19): LBM_BC_VELOCITY west (Hecht3d.hh:62-94), LBM_BC_PRESSURE east
 * (Hecht3d.hh:175-209).  Other combinations return LBM_ERR_SUP, as the
 * reference's boundary descriptors do (ZouHe2d.hh:181-236). */
#define LBM_BC_VELOCITY          1
#define LBM_BC_PRESSURE          2
#define LBM_BC_TEMPERATURE       3
#define LBM_BC_VELOCITY_STANDARD 4
#define LBM_BC_PRESSURE_STANDARD 5

/* Faces.  West = x min, East = x max, South = y min, North = y max.  A
 * boundary box lies on its face (x0 = x1 = 0 for west, y0 = y1 = ny-1 for
 * north, ...) and may cover any segment of it. */
#define LBM_FACE_WEST   0
#define LBM_FACE_EAST   1
#define LBM_FACE_SOUTH  2
#define LBM_FACE_NORTH  3

/* Spatial profile of a boundary value over its box. */
#define LBM_PROFILE_UNIFORM   0
#define LBM_PROFILE_PARABOLIC 1  /* across the lattice along the face: west/east faces
                                    (m^2-(y-m)^2)/m^2, m=(ny-1)/2 (applications/diffuser/
                                    diffuser.cc:22-31), times the same in z on D3Q19;
                                    south/north faces the same across x, m=(nx-1)/2 */
#define LBM_PROFILE_TABLE     2  /* tabulated by the caller with lbm_set_bc_profile */

/* Time law of a boundary value: value(t) = value * T(t). */
#define LBM_TIME_OFFSET_SINE 0  /* T(t) = 1 + amp*sin(2*pi*t/period) (amp = 0: steady) */
#define LBM_TIME_SINE        1  /* T(t) = amp*sin(2*pi*t/period): zero mean, e.g. the
                                   oscillating pump inlet of applications/RobustPump2d/
                                   robustPump2d.cc:13-25 */
#define LBM_TIME_RAMP        2  /* T(t) = amp + r(t - t_s), r(s) = 0 for s <= 0,
                                   sin(pi s / (2 period)) for 0 < s < period, 1 after;
                                   t_s = the step at which the last steady phase ended
                                   (lbm_forward_steady, lbm_gradient_steady), never before
                                   one: the StageTemp input of applications/Regenerator2d/
                                   regenerator2d.cc:53-69 (T0 = value*amp, dT = value) */

/* Objectives (functionals/LBMacroFunctional.hh:6-14). */
#define LBM_OBJ_NONE          0
#define LBM_OBJ_PRESSURE_DROP 1  /* functionals/pressureDrop2d.hh:9-70 */
#define LBM_OBJ_DISSIPATION   2  /* porous + viscous dissipated power (no reference counterpart) */
#define LBM_OBJ_HEAT_FLUX     3  /* functionals/temperatureFlow2d.hh:10-63 */
#define LBM_OBJ_OUTFLOW       4  /* -(mean u_x over obj_out): functionals/outflow2d.hh:10-54 */
#define LBM_OBJ_THROUGH_FLOW  5  /* -(mean u_x over obj_in + mean u_x over obj_out):
                                    functionals/throughFlow2d.hh:17-83 */
#define LBM_OBJ_DOMAIN_TEMPERATURE 6  /* mean T over obj_out (thermal lattice):
                                         functionals/domainTemperature2d.hh:13-40 */
#define LBM_OBJ_REGENERATOR_EFFICIENCY 7  /* sum (1-gamma)(T - Ti) / sum (1-gamma)(Tb - Ti)
                                             over obj_out, Ti = obj_param[0], Tb = obj_param[1]
                                             (thermal lattice): functionals/
                                             regeneratorEfficiency2d.hh:16-88 */

/* One boundary condition: the reference's boundary loop plus its Input
 * functor (ZouHe2d.hh:37: velocity or density as a function of the time step
 * and the boundary cell).  At time step t and box cell i the prescribed value
 * is v = value * T(t) * profile(i), and a velocity boundary imposes u = v * dir
 * (dir = (0,0,0) means (1,0,0)); an LBM_PROFILE_TABLE boundary with a vector
 * table takes u from the table instead. */
typedef struct lbm_bc {
  int kind;        /* LBM_BC_* */
  int face;        /* LBM_FACE_* */
  int profile;     /* LBM_PROFILE_* */
  int box[6];      /* x0,x1,y0,y1,z0,z1 inclusive; z0=z1=0 in 2D */
  double value;    /* u_max (velocity), rho0 (pressure), T (temperature) */
  double amp;      /* relative oscillation amplitude of the time law */
  double period;   /* oscillation period in time steps */
  int time_law;    /* LBM_TIME_* */
  double dir[3];   /* velocity direction (velocity boundaries), (0,0,0) = +x */
} lbm_bc;

typedef struct lbm_config {
  int lattice;     /* LBM_D2Q9, LBM_D3Q19, LBM_D2Q9_D2Q5 */
  int collision;   /* LBM_BGK, LBM_MRT */
  int storage;     /* LBM_STORE_* */
  int nx, ny, nz;  /* nz = 1 in 2D */
  double omega;    /* shear relaxation rate 1/tau */
  /* MRT rates.  D3Q19: s1,s2,s4,s10,s16,we,wej,wxx (MRT3d.hh:9-22);
   * D2Q9: s1 (energy), s2 (eps), s46 (heat flux) (incompressibleMRT2d.hh:88-90). */
  double mrt[8];
  /* Partial bounce-back (dynamics/partialBouncebackCollision.hh:53-65):
   * mixing factor = 0.5 * interp_scale * BP_q(gamma),
   * BP_q(s) = 1 - s(1+q)/(q+s) (core/interpolationFunctions.hh:17-21).
   * interp_scale = 1 is the reference's plain BPInterpolation;
   * interp_scale = 2*alpha_max gives alpha(gamma) = alpha_max*q(1-gamma)/(q+gamma). */
  double interp_scale;
  double interp_q;
  /* Temperature lattice (LBM_D2Q9_D2Q5 only): omega_T(gamma) =
   * 1/(3*diffusivity*RAMP(gamma) + 0.5) (dynamics/thermalObstacleCollision.hh:47-53),
   * RAMP(s) = (s(Ck(1+q)-1)+1)/(Ck(1+q s)) (interpolationFunctions.hh:37-49).
   * Heating of the solid: g_i += (1-gamma) w_i heat_rate (heat_T - T). */
  double diffusivity;
  double ramp_q, ramp_ck;
  double heat_rate, heat_T;
  int nbc;
  lbm_bc bc[LBM_MAX_BC];
  int objective;       /* LBM_OBJ_* */
  int obj_in[6];       /* inflow box of the pressure drop */
  int obj_out[6];      /* outflow box (pressure drop, heat flux) */
  double obj_weight;   /* timeConst: weight of each step's value (1/N for a time average) */
  double obj_param[4]; /* objective parameters (LBM_OBJ_REGENERATOR_EFFICIENCY: Ti, Tb) */
} lbm_config;

typedef struct lbm_handle lbm_handle;

typedef struct lbm_gradient_stats {
  int64_t forward_steps;     /* forward steps of the first sweep */
  int64_t recomputed_steps;  /* forward steps re-run by the checkpoint schedule */
  int64_t adjoint_steps;
  double forward_ms, reverse_ms;  /* device time of the two sweeps (CUDA events) */
} lbm_gradient_stats;

/* Fill a config with the reference defaults: D2Q9 BGK FP64, omega 1,
 * MRT3d_Compile_constants, plain BP (scale 1, q 1), no BCs, no objective. */
void lbm_config_default(lbm_config* cfg);

/* Validate the config and allocate device memory.  Replaces
 * IsothermalLBSolver2d<Op>::make (latticeBoltzmann/isothermalLBSolver2d.hh:20-60)
 * plus addBoundaryCondition, and the adjoint set-up of makeSourceAdjoint
 * (isothermalLBSolver2d.hh:62-110). */
int lbm_create(const lbm_config* cfg, lbm_handle** out);
int lbm_destroy(lbm_handle* h);

/* Text of the last error of h (or of the last failed lbm_create if h is NULL). */
const char* lbm_last_error(const lbm_handle* h);

/* Cells (nx*ny*nz) and populations per cell (9, 19 or 9+5). */
int lbm_get_sizes(const lbm_handle* h, int64_t* ncells, int* npop);

/* Lattice dimensions {nx, ny, nz} (nz = 1 in 2D). */
int lbm_get_dims(const lbm_handle* h, int dims[3]);

/* Tabulated input of boundary k, whose config gives it LBM_PROFILE_TABLE: the
 * reference's Input functor (boundaryConditions/ZouHe2d.hh:37, e.g. the
 * InflowVelocity of applications/RobustPump2d/robustPump2d.cc:13-25) sampled
 * on the boundary cells for nt time steps, reused periodically (step t reads
 * row t mod nt; nt = 1 for a profile that does not change in time).  A row
 * holds npos = (cells of the box) entries, the box cells ordered along the
 * face (y, then z, on west/east faces; x on south/north faces), each of ncomp
 * values:
 *   ncomp = 1       a factor: the cell's value is value * T(t) * entry and a
 *                   velocity boundary imposes that times dir;
 *   ncomp = 2 (2D) / 3 (D3Q19), velocity boundaries only: the velocity
 *                   vector itself (value, time law and dir are not used).
 * The table is copied to the device; calling again replaces it.  Steps that
 * apply a table boundary whose table was never set return LBM_ERR_STATE.
 * Set the tables of a batch's lattices before its first CUDA-graph gradient,
 * or the captured graph keeps reading the old table.  No reference
 * counterpart as an entry point (the reference takes a compiled functor). */
int lbm_set_bc_profile(lbm_handle* h, int k, int nt, int ncomp, const double* table);

/* Design field gamma in [0,1], one double per cell.  Replaces
 * LBSolver::setFieldFromDesignVec (latticeBoltzmann/LBSolver.cc:333-348). */
int lbm_set_design(lbm_handle* h, const double* gamma);

/* lbm_set_design from device memory (ncells FP64 values on the current
 * device, e.g. the output of lbm_topopt_apply's filter chain); waits for the
 * device to finish the caller's work first.  The values are not checked for
 * range.  No reference counterpart (the reference's design vectors are host
 * PETSc Vecs). */
int lbm_set_design_device(lbm_handle* h, const double* gamma_dev);

/* Device address of the handle's FP64 dJ/dgamma (ncells values, valid until
 * the handle is destroyed; its contents change with the next reverse step). */
int lbm_get_sensitivity_device(const lbm_handle* h, const double** sens_dev);

/* f_0 = feq(macros) and t = 0.  macros: NULL for rho=1, u=0 (T=0), else
 * per cell {rho,ux,uy} (D2Q9), {rho,ux,uy,uz} (D3Q19) or {rho,ux,uy,T}.
 * Replaces LBSolver::initializeAtEquilibrium (LBSolver.cc:234-249). */
int lbm_init_equilibrium(lbm_handle* h, const double* macros);

/* Advance the state nsteps time steps from t0 to t0+nsteps; accumulate the
 * objective of each new state: J_steps[k] = weight*F(f_{t0+1+k}).
 * J_steps and J_sum may be NULL.  Replaces the app loop around
 * LBSolver::collide/stream (LBSolver.cc:163-206) and
 * LBSolver::computeMacroFunctional (LBSolver.cc:74-91). */
int lbm_forward(lbm_handle* h, int nsteps, double* J_steps, double* J_sum);

/* Advance until the state is steady: every check_every steps the largest
 * change of any population over the last step, max |f_t - f_{t-1}|, is
 * measured on the device; stop when it is below tol, or after max_steps
 * steps (then the change of the last step is measured as well).  No
 * objective is evaluated.  *steps (may be NULL) = steps taken, *change (may
 * be NULL) = the last change measured.  Replaces the steady-state loop of
 * applications/Regenerator2d/regenerator2d.cc:255-272 (chkFreq, tol,
 * maxSteps); the unsteady part that follows there is lbm_forward. */
int lbm_forward_steady(lbm_handle* h, int max_steps, int check_every, double tol, int* steps,
                       double* change);

/* Current time step t of the state. */
int lbm_get_time(const lbm_handle* h, int* t);

/* Populations of the state f_t, FP64 AoS (post-stream, post-BC). */
int lbm_get_populations(const lbm_handle* h, double* f);
/* Replace the state by host populations f (FP64 AoS) at time step t.
 * Replaces LBSolver::setDistributions + setCurrentTimestep (LBSolver.cc:65-97). */
int lbm_set_populations(lbm_handle* h, const double* f, int t);
/* Macros of the state f_t: {rho,ux,uy}, {rho,ux,uy,uz} or {rho,ux,uy,T}. */
int lbm_get_macros(const lbm_handle* h, double* mac);

/* Zero the adjoint populations and the sensitivity field.
 * Replaces AdjointLBSolver::resetAdjoints (adjointLBSolver.cc:138-145). */
int lbm_adjoint_reset(lbm_handle* h);

/* One reverse time step for the forward state currently held (f_t):
 * adjoint collision at f_t with sensitivity accumulation, objective source
 * weight*dF/df_t, adjoint boundary conditions at t, adjoint stream.  At t = 0
 * only the adjoint collision runs (no objective, no boundary): the design
 * dependence of the first collision, which the reference's reverse loop
 * (applications/RobustPump2d/robustPump2d.cc:268-276) leaves out.
 * Replaces AdjointLBSolver::adjointCollide + computeCollideSource +
 * computeSensitivitySource + adjointStream (adjointLBSolver.cc:28-122). */
int lbm_adjoint_step(lbm_handle* h);

/* Adjoint populations (FP64 AoS) of the post-collision state of the step
 * below the last reverse step, i.e. what adjointGlobal holds after
 * AdjointLBSolver::adjointStream. */
int lbm_get_adjoint(const lbm_handle* h, double* lam);

/* dJ/dgamma accumulated so far, one double per cell.
 * Replaces AdjointLBSolver::getSensitivities (adjointLBSolver.cc:153-157). */
int lbm_get_sensitivity(const lbm_handle* h, double* sens);

/* Full gradient: f_0 from uniform rest (or the macros of the last
 * lbm_init_equilibrium), nsteps forward steps with Wang et al. dynamic
 * checkpointing in nsnapshots device slots, then the reverse sweep, closed by
 * the reverse of the collision of f_0 (see lbm_adjoint_step).
 * Replaces the checkpointed driver of robustPump2d.cc:234-276 with
 * LBDynamicCheckpointing (topOpt/LBCheckpointing.cc:322-351,
 * topOpt/dynamicCheckpointing.cc:9-54, topOpt/WangCheckpointing.cc:36-126).
 * J (may be NULL) gets sum_t weight*F(f_t); dJdgamma (may be NULL) gets
 * the sensitivity field; stats may be NULL. */
int lbm_gradient(lbm_handle* h, int nsteps, int nsnapshots, double* J,
                 double* dJdgamma, lbm_gradient_stats* stats);

/* Checkpoint schedules of lbm_gradient_schedule. */
#define LBM_SCHEDULE_DYNAMIC 0 /* LBDynamicCheckpointing: online Wang placement */
#define LBM_SCHEDULE_STATIC 1  /* LBStaticCheckpointing (topOpt/LBCheckpointing.cc:4-35,
                                  staticCheckpointing.cc:3-63): the placement the online
                                  schedule reaches after nsteps, planned before the sweep */

/* lbm_gradient with the checkpoint schedule chosen: replaces the driver loop
 * with LBStaticCheckpointing(nsnapshots, nsteps + 1, solver) as well
 * (applications/pump2d/pump2d.cc:146, RobustPump2d/robustPump2d.cc:166).  The
 * gradient does not depend on the schedule (recomputation is bit-exact). */
int lbm_gradient_schedule(lbm_handle* h, int nsteps, int nsnapshots, int schedule, double* J,
                          double* dJdgamma, lbm_gradient_stats* stats);

/* The regenerator applications' gradient (applications/Regenerator2d/
 * regenerator2d.cc:266-387, ComputeObjectiveAndSens): from f_0 (uniform rest or
 * the macros of the last lbm_init_equilibrium), run to a steady state -- every
 * check_every steps the largest change of any population over the last step,
 * max |f_t - f_{t-1}|, is measured; the phase ends when it is below tol or
 * after max_steady steps -- then n_unsteady more steps whose states' objective
 * is summed (J = sum_{t=S+1..S+n_unsteady} weight*F(f_t), S = the steady
 * steps).  LBM_TIME_RAMP boundaries start their ramp at step S (StageTemp,
 * regenerator2d.cc:53-69).  The reverse sweep runs through all S + n_unsteady
 * steps, the steady part without objective source (the reference's
 * EmptyFunctional), closed by the reverse of the collision of f_0; the states
 * come from Wang et al. dynamic checkpointing in nsnapshots device slots (the
 * length of the sweep is not known in advance).  *steady_steps (may be NULL)
 * gets S; J, dJdgamma and stats as for lbm_gradient. */
int lbm_gradient_steady(lbm_handle* h, int max_steady, int check_every, double tol,
                        int n_unsteady, int nsnapshots, int* steady_steps, double* J,
                        double* dJdgamma, lbm_gradient_stats* stats);

/* Device-time measurement for benchmarks: run `nsteps` forward steps
 * (which = 0), reverse steps over the current state (which = 1; the forward
 * state is left unchanged) or forward+reverse pairs (which = 2) on the
 * handle's stream, bracketed by CUDA events recorded on that stream.  *ms
 * gets the elapsed time.  The adjoint and sensitivity fields are scratch
 * afterwards. */
int lbm_time_steps(lbm_handle* h, int which, int nsteps, float* ms);

/* Time every candidate thread-block shape of the forward and reverse step
 * kernels (and both register variants of the reverse step) for nsteps steps
 * each on this handle's lattice and keep the fastest (the tile-shape
 * autotuner).  Forward steps are timed with the objective summed over the
 * steps, as a gradient's forward sweep runs them.  Needs a design and a state; the state
 * is left unchanged and the adjoint and sensitivity fields are zeroed. */
int lbm_autotune(lbm_handle* h, int nsteps);

/* Block shape in use for the forward (which = 0) or reverse (which = 1) step. */
int lbm_get_launch_shape(const lbm_handle* h, int which, int* bx, int* by);

/* Set the block shape of the forward (which = 0) or reverse (which = 1) step,
 * e.g. one found by lbm_autotune in an earlier run: bx a multiple of 32,
 * bx * by in {64, 128, 256}.  No reference counterpart (the reference has no
 * launch geometry). */
int lbm_set_launch_shape(lbm_handle* h, int which, int bx, int by);

/* Reverse step kernel variant: 0 the default register budget, 1 one more
 * resident thread block per SM with fewer registers per thread (faster where
 * the extra warps hide more memory latency than the spills cost; lbm_autotune
 * times both).  Results agree to FP32 rounding: under the tighter register
 * budget the compiler may fuse a few multiply-adds differently (measured
 * 9e-10 of max |dJ/dgamma| on a D2Q9 channel; bit-identical on D3Q19 MRT and
 * the thermal model).  Set the variant explicitly for bitwise reproducible
 * FP32 gradients across tuning runs.  FP64 storage has only variant 0 (1
 * returns LBM_ERR_SUP).  No reference counterpart. */
int lbm_set_reverse_variant(lbm_handle* h, int lean);
/* The reverse step variant in use (0 or 1), negative on error. */
int lbm_get_reverse_variant(const lbm_handle* h);

/* Select the CUDA device (ordinal) that handles created afterwards by this
 * thread use (one process per GPU: the rank's local GPU). */
int lbm_select_device(int ordinal);

/* Number of kernel launches issued by this handle since creation. */
int lbm_get_launch_count(const lbm_handle* h, int64_t* launches);

/* Wang et al. checkpoint schedule on the host only: forward-recompute
 * steps needed to reverse nsteps steps with nsnapshots slots
 * (WangCheckpointing.cc:72-162 with DynamicCheckpointing.cc:9-54). */
int lbm_wang_recompute_count(int nsteps, int nsnapshots, int64_t* recomputed);

/* Host-only: recomputed steps and states kept by the forward sweep (saved may
 * be NULL) for a schedule, without a device. */
int lbm_schedule_count(int nsteps, int nsnapshots, int schedule, int64_t* recomputed,
                       int64_t* saved);

/* ------------------------------------------------------------------------
 * Batches.  Up to LBM_MAX_BATCH lattices with the same lattice type, collision
 * and storage (sizes, boundaries, designs and objectives free) advanced
 * together: one launch per time step covers every lattice, its blocks laid
 * over their concatenated blocks.  The one-GPU form of
 * the reference's robust-design ensembles (core/MPISplit.cc:14-59,
 * applications/RobustPump2d/robustPump2d.cc:140-146), where each realisation
 * ran on its own MPI sub-communicator. */
typedef struct lbm_batch lbm_batch;

int lbm_batch_create(const lbm_config* cfgs, int n, lbm_batch** out);
int lbm_batch_destroy(lbm_batch* b);
const char* lbm_batch_last_error(const lbm_batch* b);
/* The handle of lattice i (owned by the batch): set its design, read its state
 * and sensitivities with the single-lattice entry points. */
int lbm_batch_handle(lbm_batch* b, int i, lbm_handle** h);
/* Pick the block shapes of the batched forward and reverse step kernels,
 * each timed on its own, and the reverse step's register variant (states are
 * re-initialised). */
int lbm_batch_autotune(lbm_batch* b, int nsteps);
/* Block shape of the batched forward (and objective) kernels. */
int lbm_batch_get_launch_shape(const lbm_batch* b, int* bx, int* by);
/* Block shape of the batched reverse step kernel. */
int lbm_batch_get_reverse_shape(const lbm_batch* b, int* bx, int* by);
/* Set the block shape of the batched forward and objective kernels
 * (which = 0) or of the batched reverse step (which = 1) to one of
 * lbm_batch_autotune's shapes (256x1, 128x2, 64x4, 32x8, 128x1, 64x2, 32x4,
 * 64x1, 32x2),
 * e.g. one it found in an earlier run.  No reference counterpart. */
int lbm_batch_set_launch_shape(lbm_batch* b, int which, int bx, int by);
/* Register variant of the batched reverse step (as lbm_set_reverse_variant). */
int lbm_batch_set_reverse_variant(lbm_batch* b, int lean);
int lbm_batch_get_reverse_variant(const lbm_batch* b);
/* nsteps forward steps of every lattice from its current state; J[i] (may be
 * NULL) gets lattice i's objective sum as lbm_forward would. */
int lbm_batch_forward(lbm_batch* b, int nsteps, double* J);
/* lbm_gradient for every lattice at once (same nsteps and nsnapshots).  With
 * use_graph the whole sequence (initialisation, forward sweep, checkpoint
 * copies, recomputation, reverse sweep) is captured once as a CUDA graph and
 * replayed by later calls with the same nsteps and nsnapshots.  J (n values)
 * and dJdgamma (n pointers, entries may be NULL) may be NULL. */
int lbm_batch_gradient(lbm_batch* b, int nsteps, int nsnapshots, int use_graph, double* J,
                       double* const* dJdgamma, lbm_gradient_stats* stats);

/* lbm_batch_gradient with the checkpoint schedule chosen (LBM_SCHEDULE_*). */
int lbm_batch_gradient_schedule(lbm_batch* b, int nsteps, int nsnapshots, int schedule,
                                int use_graph, double* J, double* const* dJdgamma,
                                lbm_gradient_stats* stats);
/* As lbm_time_steps, for the batched kernels. */
int lbm_batch_time_steps(lbm_batch* b, int which, int nsteps, float* ms);
int lbm_batch_get_launch_count(const lbm_batch* b, int64_t* launches);

/* ------------------------------------------------------------------------
 * Design update on the device: the reference's optimisation loop around the
 * solver (applications/RobustPump2d/robustPump2d.cc:215-315) without host
 * round trips.  Design variables x live on the cells of a design box
 * (FullToDesignMapping2d, topOpt/fullToDesignMapping2d.cc); the full field
 * (a fixed background outside the box) passes up to two density-filter +
 * tanh-projection stages (DensityFilter2d/3d, ProjectionFilter2d,
 * DoubleProjectionFilter2d) to the physical gamma; sensitivities go back
 * through the transposed chain; a volume constraint (VolumeConstraint,
 * functionals/volumeConstraint.cc) and MMA (Svanberg 1987, with the
 * subproblem of topOpt/MMA.cc) update x.  Several realisations (robust
 * design: the last projection's eta per realisation) give the min-max form
 * of robustPump2d.cc:166-190 (constraints J_r + magic - z <= 0).  FP64
 * throughout.
 * ------------------------------------------------------------------------ */
#define LBM_VOLUME_NONE 0
#define LBM_VOLUME_FLUID 1    /* ConstrainFluid:    mean(gamma) - V <= 0 */
#define LBM_VOLUME_MATERIAL 2 /* ConstrainMaterial: (1 - V) - mean(gamma) <= 0 */
#define LBM_MAX_STAGES 2
#define LBM_MAX_REALISATIONS 8

typedef struct lbm_topopt_config {
  int nx, ny, nz;             /* the lattice (nz = 1 in 2D) */
  int design_box[6];          /* x0,x1,y0,y1,z0,z1 (inclusive): one design variable per cell */
  int nstages;                /* 0, 1 or 2 filter stages */
  int radius[LBM_MAX_STAGES]; /* cone filter radius of each stage (cells) */
  int filter_box[6];          /* rows the filters act on (the reference passes the design box) */
  int project[LBM_MAX_STAGES];/* 1: tanh projection after the stage's filter */
  double beta[LBM_MAX_STAGES], eta[LBM_MAX_STAGES];
  int nreal;                  /* realisations: 1 = minimise J; > 1 = minimise max_r J_r */
  double real_eta[LBM_MAX_REALISATIONS]; /* eta of the last projection per realisation (nreal > 1) */
  int volume_type;            /* LBM_VOLUME_* */
  double volume;              /* V */
  int volume_real;            /* realisation whose physical field the volume is measured on */
  double move_limit;          /* MMA outer move limit (MMA::Update's movlim) */
  double magic;               /* added to every J_r in the min-max form (robustPump2d.cc:182) */
} lbm_topopt_config;

typedef struct lbm_topopt lbm_topopt;

/* Defaults: one stage of radius 2 with projection beta 1, eta 0.5;
 * ConstrainFluid at 0.5; move limit 0.1; magic 5; nreal 1. */
void lbm_topopt_config_default(lbm_topopt_config* c);
/* background: full-grid gamma outside the design box (NULL = 1, fluid);
 * x0: initial design variables (NULL = 0.5). */
int lbm_topopt_create(const lbm_topopt_config* c, const double* background, const double* x0,
                      lbm_topopt** out);
int lbm_topopt_destroy(lbm_topopt* t);
const char* lbm_topopt_last_error(const lbm_topopt* t);
int lbm_topopt_num_variables(const lbm_topopt* t, int64_t* n);
int lbm_topopt_set_variables(lbm_topopt* t, const double* x);
int lbm_topopt_get_variables(const lbm_topopt* t, double* x);
/* ProjectionFilter2d::setBeta / increaseBeta (projectionFilter2d.hh:16-18) */
int lbm_topopt_set_beta(lbm_topopt* t, int stage, double beta);
/* Physical field of realisation r (host copy, nx*ny*nz values). */
int lbm_topopt_physical(lbm_topopt* t, int r, double* gamma);
/* Physical field of realisation r into a handle's design, on the device
 * (filterDesign + setFieldFromDesignVec). */
int lbm_topopt_apply(lbm_topopt* t, int r, lbm_handle* h);
/* Objective J_r and the handle's dJ/dgamma (after lbm_gradient) for
 * realisation r: the chain rule through the filters and the box
 * (filterSensitivities + mapFullToDesign), on the device. */
int lbm_topopt_set_sensitivity(lbm_topopt* t, int r, lbm_handle* h, double J);
/* The same from a host dJ/dgamma (nx*ny*nz values). */
int lbm_topopt_set_sensitivity_host(lbm_topopt* t, int r, const double* dJdgamma, double J);
/* dJ_r/dx (host copy, one value per design variable). */
int lbm_topopt_get_design_sensitivity(const lbm_topopt* t, int r, double* dJdx);
/* Volume constraint and one MMA step (MMA::Update + DesignChange): x is
 * replaced; *change = max |x_new - x_old|; constraints (may be NULL) gets the
 * constraint values handed to MMA (nreal == 1: the volume; else J_r + magic
 * for every r, then the volume). */
int lbm_topopt_update(lbm_topopt* t, double* change, double* constraints);

/* Objective weight*F(f_t) of a state that lives in the caller's own device
 * memory, computed without allocating any device memory.  For callers that
 * cannot call cudaMalloc: an application that reserves all of its device
 * memory up front and forbids later allocations, a real-time loop that cannot
 * pay cudaMalloc's latency and implicit synchronisation, a process held to a
 * fixed device-memory budget.  No counterpart in the reference.
 *   cfg       lattice, storage, boundaries and objective (as for lbm_create)
 *   t         time step of the state (boundary conditions of step t are applied
 *             on load when t >= 1)
 *   f_dev     populations in the handle layout: Q planes of P = ncells rounded
 *             up to 128 elements, storage precision of cfg (FP32/FP16 planes of
 *             the flow lattice hold f_i - w_i)
 *   gamma_dev design, ncells values: double for LBM_STORE_FP64, float otherwise
 *   J_dev     device address of one double receiving the objective
 *   stream    cudaStream_t to run on (NULL: the default stream); the result is
 *             ready when the stream is.
 * Its scratch (block partial sums, a counter, inflow-profile tables) is one
 * fixed 640 KiB array per GPU, held for the life of the process.  Limits:
 * at most 32,768 thread blocks of 256 threads, ceil(nx/bx) * ceil(ny/by) * nz
 * with bx = nx rounded up to a multiple of 32 (at most 256) and by = 256/bx
 * (8,388,608 cells when nx is a multiple of 256, fewer otherwise), and
 * 32,768 tabulated inflow-profile values (one per cell of each parabolic
 * velocity boundary); larger requests return LBM_ERR_ARG before any device
 * call.  Boundaries with LBM_PROFILE_TABLE are refused (LBM_ERR_SUP): their
 * tables live in a handle.  With parabolic velocity boundaries the call
 * copies their profile to the scratch and waits for `stream` before it
 * returns.  Every call shares that array, so calls that overlap on the GPU
 * (other streams, other threads) race and must be serialised by the caller.
 * The first call on each device looks up the array's device address and
 * keeps it for the life of the process; make that call before any stream
 * capture.  A cudaDeviceReset() invalidates the kept address (as it does
 * every handle): do not call this entry point after resetting a device.
 * Errors are reported through lbm_last_error(NULL). */
int lbm_objective_noalloc(const lbm_config* cfg, int t, const void* f_dev,
                          const void* gamma_dev, double* J_dev, void* stream);

/* ------------------------------------------------------------------------
 * Files, on the host (errors through lbm_last_error(NULL)).
 * ------------------------------------------------------------------------ */

/* PETSc binary Vec file, as writeVectorToBinary / loadVectorFromBinary
 * (core/binaryIO.cc:3-33) write and read design vectors: big-endian int32
 * class id 1211214, int32 length, big-endian doubles. */
int lbm_write_petsc_vec(const char* path, const double* v, int64_t n);
/* v may be NULL to query the length only; fails if the file holds more than
 * n_max values. */
int lbm_read_petsc_vec(const char* path, double* v, int64_t n_max, int64_t* n);

/* VTK XML StructuredGrid (.vts) of point fields on an nx*ny*nz lattice (x
 * fastest): field k has ncomp[k] components per point. */
int lbm_write_vts_fields(const char* path, int nx, int ny, int nz, int nfields,
                         const char* const* names, const int* ncomp, const double* const* data);
/* The handle's macros at its current state (rho, velocity, and T for the
 * thermal lattice) and, if gamma is not NULL, the design field, as .vts:
 * LBSolver::outputMacros / outputFields (latticeBoltzmann/LBSolver.cc:251-286). */
int lbm_write_vts(lbm_handle* h, const char* path, const double* gamma);

#ifdef __cplusplus
}
#endif

#endif /* LBMGPU_H */
