// kernels_d2q9.cu -- instantiation of the step kernels for one lattice.
#include "lbm_kernels.cuh"

namespace lbm {

#define LAT LAT_D2Q9
LaunchFn launcher_d2q9(int collision, int storage) {
  if (collision == LBM_BGK) {
    if (storage == LBM_STORE_FP64) return &OpsImpl<LAT, LBM_BGK, double>::launch;
    if (storage == LBM_STORE_FP32) return &OpsImpl<LAT, LBM_BGK, float>::launch;
    if (storage == LBM_STORE_FP16) return &OpsImpl<LAT, LBM_BGK, __half>::launch;
  } else if (collision == LBM_MRT) {
    if (storage == LBM_STORE_FP64) return &OpsImpl<LAT, LBM_MRT, double>::launch;
    if (storage == LBM_STORE_FP32) return &OpsImpl<LAT, LBM_MRT, float>::launch;
    if (storage == LBM_STORE_FP16) return &OpsImpl<LAT, LBM_MRT, __half>::launch;
  }
  return nullptr;
}

ChangeFn change_fn_d2q9(int collision, int storage) {
  if (collision == LBM_BGK) {
    if (storage == LBM_STORE_FP64) return &OpsImpl<LAT, LBM_BGK, double>::max_change;
    if (storage == LBM_STORE_FP32) return &OpsImpl<LAT, LBM_BGK, float>::max_change;
    if (storage == LBM_STORE_FP16) return &OpsImpl<LAT, LBM_BGK, __half>::max_change;
  } else if (collision == LBM_MRT) {
    if (storage == LBM_STORE_FP64) return &OpsImpl<LAT, LBM_MRT, double>::max_change;
    if (storage == LBM_STORE_FP32) return &OpsImpl<LAT, LBM_MRT, float>::max_change;
    if (storage == LBM_STORE_FP16) return &OpsImpl<LAT, LBM_MRT, __half>::max_change;
  }
  return nullptr;
}

BatchOps batch_ops_d2q9(int collision, int storage) {
  BatchOps o;
  if (collision == LBM_BGK && storage == LBM_STORE_FP64) {
    o.launch = &OpsImpl<LAT, LBM_BGK, double>::launch_batch;
    o.kernel = &OpsImpl<LAT, LBM_BGK, double>::kernel_address;
  }
  if (collision == LBM_BGK && storage == LBM_STORE_FP32) {
    o.launch = &OpsImpl<LAT, LBM_BGK, float>::launch_batch;
    o.kernel = &OpsImpl<LAT, LBM_BGK, float>::kernel_address;
  }
  if (collision == LBM_BGK && storage == LBM_STORE_FP16) {
    o.launch = &OpsImpl<LAT, LBM_BGK, __half>::launch_batch;
    o.kernel = &OpsImpl<LAT, LBM_BGK, __half>::kernel_address;
  }
  if (collision == LBM_MRT && storage == LBM_STORE_FP64) {
    o.launch = &OpsImpl<LAT, LBM_MRT, double>::launch_batch;
    o.kernel = &OpsImpl<LAT, LBM_MRT, double>::kernel_address;
  }
  if (collision == LBM_MRT && storage == LBM_STORE_FP32) {
    o.launch = &OpsImpl<LAT, LBM_MRT, float>::launch_batch;
    o.kernel = &OpsImpl<LAT, LBM_MRT, float>::kernel_address;
  }
  if (collision == LBM_MRT && storage == LBM_STORE_FP16) {
    o.launch = &OpsImpl<LAT, LBM_MRT, __half>::launch_batch;
    o.kernel = &OpsImpl<LAT, LBM_MRT, __half>::kernel_address;
  }
  return o;
}
#undef LAT

}  // namespace lbm
