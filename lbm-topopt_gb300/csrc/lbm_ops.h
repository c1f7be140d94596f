// lbm_ops.h -- per-lattice kernel launchers (one translation unit per lattice).
#pragma once

#include <cuda_runtime.h>

#include "../../include/lbmgpu.h"

namespace lbm {

struct KParams;
struct BatchParams;
struct DevBC;
struct ObjectiveInfo;

enum {
  K_FORWARD = 0,
  K_ADJOINT,
  K_OBJECTIVE,
  K_INIT,
  K_EXPORT,
  K_IMPORT,
  K_MACROS,
  K_EXPORT_ADJ,
  K_GAMMA,
  K_ADJOINT_LEAN,   // the reverse step with one more resident block per SM
};

typedef void (*LaunchFn)(int kind, dim3 grid, dim3 block, cudaStream_t st, const KParams& p,
                         double* aux);

typedef void (*BatchLaunchFn)(int kind, dim3 grid, dim3 block, cudaStream_t st,
                              const BatchParams& bp);
// max |f_t - f_{t-1}| with each state's boundary conditions (k_max_change_bc)
typedef void (*ChangeFn)(dim3 grid, dim3 block, cudaStream_t st, const KParams& cur,
                         const KParams& prev, unsigned long long* bits);
typedef const void* (*KernelAddressFn)(int kind);

struct BatchOps {
  BatchLaunchFn launch = nullptr;
  KernelAddressFn kernel = nullptr;
};

BatchOps batch_ops_d2q9(int collision, int storage);
BatchOps batch_ops_d3q19(int collision, int storage);
BatchOps batch_ops_thermal(int collision, int storage);

LaunchFn launcher_d2q9(int collision, int storage);
LaunchFn launcher_d3q19(int collision, int storage);
LaunchFn launcher_thermal(int collision, int storage);

ChangeFn change_fn_d2q9(int collision, int storage);
ChangeFn change_fn_d3q19(int collision, int storage);
ChangeFn change_fn_thermal(int collision, int storage);

// Text returned by lbm_last_error(NULL) (errors raised outside a handle).
void set_global_error(const char* msg);
// The checks of lbm_create (message through lbm_last_error(NULL)); 0 = valid.
int validate_config(const lbm_config& c);

// Boundary conditions on the host.  Cells of b's box in table order (along the
// face: y then z on west/east faces, x on south/north faces).
int64_t bc_npos(const lbm_bc& b);
// Whether b lies on a south or north face.
bool bc_on_y_face(const lbm_bc& b);
// T(t) of b's time law; t_start: where LBM_TIME_RAMP ramps begin (INT_MAX: not yet).
double bc_time_factor(const lbm_bc& b, int t, int t_start);
// Parabolic factors of a velocity boundary over its box, bc_npos(b) values.
void bc_parabola(const lbm_config& c, const lbm_bc& b, double* out);
// Device parameters of boundary b at time step t.  tab_d / tab_f: the factor
// (ncomp = 1) or velocity (ncomp = 2, 3) table row of step t, or null.
void fill_devbc(const lbm_bc& b, int t, int t_start, int ncomp, const double* tab_d,
                const float* tab_f, DevBC& d);

// The facts of objective `id` from the kernels' objective list; false if unknown.
bool objective_info(int id, ObjectiveInfo* out);
// 1/|in| and 1/|out| of the boxes the config's objective averages over (0 if unused).
void objective_norms(const lbm_config& c, double* inv_in, double* inv_out);

}  // namespace lbm
