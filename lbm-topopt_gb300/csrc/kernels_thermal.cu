// kernels_thermal.cu -- instantiation of the step kernels for one lattice.
#include "lbm_kernels.cuh"

namespace lbm {

#define LAT LAT_D2Q9_D2Q5
LaunchFn launcher_thermal(int collision, int storage) {
  if (collision == LBM_BGK) {
    if (storage == LBM_STORE_FP64) return &OpsImpl<LAT, LBM_BGK, double>::launch;
    if (storage == LBM_STORE_FP32) return &OpsImpl<LAT, LBM_BGK, float>::launch;
  }
  return nullptr;
}
#undef LAT

}  // namespace lbm
