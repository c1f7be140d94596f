// lbm_ops.h -- per-lattice kernel launchers (one translation unit per lattice).
#pragma once

#include <cuda_runtime.h>

#include "../../include/lbmgpu.h"

namespace lbm {

struct KParams;
struct BatchParams;

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

// Text returned by lbm_last_error(NULL) (errors raised outside a handle).
void set_global_error(const char* msg);
// The checks of lbm_create (message through lbm_last_error(NULL)); 0 = valid.
int validate_config(const lbm_config& c);

}  // namespace lbm
