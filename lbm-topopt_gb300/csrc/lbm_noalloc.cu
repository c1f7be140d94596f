// lbm_noalloc.cu -- objective evaluation that allocates no device memory.
//
// Callers that manage every byte of device memory themselves (a solver embedded
// in a larger simulation that reserves its arena up front, a real-time loop that
// cannot afford the latency and implicit synchronisation of cudaMalloc, a
// process held to a fixed device-memory budget where a late allocation may
// fail) can still ask for the objective of a state they own.  The state, the
// design and the result buffer are theirs; the scratch this kernel needs (one
// FP64 partial sum per thread block, the last-block counter and the inflow
// profile tables) lives in the fixed array below, which every GPU that loads
// the library keeps until the process exits.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/lbmgpu.h"
#include "lbm_device.cuh"
#include "lbm_ops.h"

using namespace lbm;

namespace {

// Scratch limits: at most kMaxBlocks 256-thread blocks (8,388,608 cells when
// nx is a multiple of 256; the launch pads each row of blocks) and kMaxProfile
// tabulated inflow-profile entries over all parabolic velocity boundaries.
constexpr int kMaxBlocks = 32768;
constexpr int kMaxProfile = 32768;
constexpr size_t kCounterBytes = 256;
constexpr size_t kPartialBytes = sizeof(double) * kMaxBlocks;
constexpr size_t kProfDBytes = sizeof(double) * kMaxProfile;
constexpr size_t kProfFBytes = sizeof(float) * kMaxProfile;
constexpr size_t kScratchBytes = kCounterBytes + kPartialBytes + kProfDBytes + kProfFBytes;

// 640 KiB + 256 B per device: counter | block partials | FP64 profile | FP32 profile
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
// Device address of the array per device, looked up by the first call on that
// device.  A cudaDeviceReset() of the device would leave a stale address here
// (the array gets a new one in the new context); the library is not used
// across device resets.
void* g_scratch_ptr[kMaxDevices] = {};
// host-side staging of the profile tables (static storage: no heap allocation)
double g_prof_d[kMaxProfile];
float g_prof_f[kMaxProfile];

// A velocity boundary whose factors this path tabulates into its scratch.
bool parabolic(const lbm_bc& b) {
  return (b.kind == LBM_BC_VELOCITY || b.kind == LBM_BC_VELOCITY_STANDARD) &&
         b.profile == LBM_PROFILE_PARABOLIC;
}

int fail(int code, const std::string& msg) {
  lbm::set_global_error(msg.c_str());   // read back with lbm_last_error(NULL)
  return code;
}

}  // namespace

extern "C" int lbm_objective_noalloc(const lbm_config* cfg, int t, const void* f_dev,
                                     const void* gamma_dev, double* J_dev, void* stream) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!cfg || !f_dev || !gamma_dev || !J_dev) return fail(LBM_ERR_ARG, "null argument");
  if (t < 0) return fail(LBM_ERR_ARG, "time step < 0");
  const lbm_config& c = *cfg;
  int vrc = validate_config(c);   // same checks as lbm_create (boxes, faces, kinds)
  if (vrc) return vrc;
  if (c.objective == LBM_OBJ_NONE) return fail(LBM_ERR_ARG, "config has no objective");
  const int dim = c.lattice == LBM_D3Q19 ? 3 : 2;
  const int nz = dim == 3 ? c.nz : 1;
  if (c.nx < 3 || c.ny < 3 || nz < 1) return fail(LBM_ERR_ARG, "lattice too small");
  const int Q = c.lattice == LBM_D2Q9 ? 9 : c.lattice == LBM_D3Q19 ? 19 : 14;
  const long long ncell = (long long)c.nx * c.ny * nz;
  const long long P = (ncell + 127) / 128 * 128;
  if ((long long)Q * P >= (long long)INT32_MAX) return fail(LBM_ERR_SUP, "lattice too large");

  // launch geometry: 256-thread x-major blocks, as the handle's default
  int bx = c.nx >= 256 ? 256 : ((c.nx + 31) / 32) * 32;
  if (bx > 256) bx = 256;
  int by = 256 / bx;
  dim3 block(bx, by, 1), grid((c.nx + bx - 1) / bx, (c.ny + by - 1) / by, nz);
  const long long nblocks = (long long)grid.x * grid.y * grid.z;
  if (nblocks > kMaxBlocks)
    return fail(LBM_ERR_ARG, "lattice needs " + std::to_string(nblocks) +
                                 " thread blocks; the allocation-free path holds scratch for " +
                                 std::to_string(kMaxBlocks));
  long long nprof = 0;
  for (int k = 0; k < c.nbc; ++k) {
    const lbm_bc& b = c.bc[k];
    if (b.profile == LBM_PROFILE_TABLE)
      return fail(LBM_ERR_SUP, "boundary " + std::to_string(k) +
                                   ": tabulated profiles live in a handle; the allocation-free "
                                   "path takes uniform and parabolic profiles only");
    if (b.time_law == LBM_TIME_RAMP)
      return fail(LBM_ERR_SUP, "boundary " + std::to_string(k) +
                                   ": ramps start after a handle's steady phase; the allocation-"
                                   "free path has none");
    if (parabolic(b)) nprof += bc_npos(b);
  }
  if (c.objective == LBM_OBJ_REGENERATOR_EFFICIENCY)
    return fail(LBM_ERR_SUP, "the regenerator efficiency's denominator comes from a handle's design");
  if (nprof > kMaxProfile)
    return fail(LBM_ERR_ARG, "inflow profiles need " + std::to_string(nprof) +
                                 " entries; the allocation-free path holds " +
                                 std::to_string(kMaxProfile));
  LaunchFn launch = c.lattice == LBM_D2Q9    ? launcher_d2q9(c.collision, c.storage)
                    : c.lattice == LBM_D3Q19 ? launcher_d3q19(c.collision, c.storage)
                                             : launcher_thermal(c.collision, c.storage);
  if (!launch) return fail(LBM_ERR_SUP, "no kernel for this lattice/collision/storage");

  // Set-up once per device, with that device current: the host-side name of
  // the array is not a device address, so ask the runtime for it.
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(LBM_ERR_CUDA, "device ordinal out of range");
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(LBM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = ptr;
  }
  unsigned char* base = (unsigned char*)g_scratch_ptr[dev];
  unsigned* counter = (unsigned*)base;
  double* partial = (double*)(base + kCounterBytes);
  double* prof_d = (double*)(base + kCounterBytes + kPartialBytes);
  float* prof_f = (float*)(base + kCounterBytes + kPartialBytes + kProfDBytes);
  cudaStream_t st = (cudaStream_t)stream;

  KParams p;
  memset(&p, 0, sizeof(p));
  p.nx = c.nx;
  p.ny = c.ny;
  p.nz = nz;
  p.P = P;
  p.step = (unsigned)t;
  p.key_fwd = step_key(p.step, kSaltForward);
  p.key_adj = step_key(p.step, kSaltAdjoint);
  ModelParams<double>& md = p.md;
  md.omega = c.omega;
  for (int i = 0; i < 8; ++i) md.mrt[i] = c.mrt[i];
  md.pbb_scale = c.interp_scale;
  md.pbb_q = c.interp_q;
  md.obj_weight = c.obj_weight;
  {
    double nu = (1. / c.omega - 0.5) / 3.;
    md.cv_diss = 4.5 * nu * c.omega * c.omega;
  }
  p.objective = c.objective;
  p.obj_weight = c.obj_weight;
  for (int i = 0; i < 6; ++i) {
    p.obj_in[i] = c.obj_in[i];
    p.obj_out[i] = c.obj_out[i];
  }
  objective_norms(c, &p.inv_in, &p.inv_out);
  md.w_in = p.inv_in * c.obj_weight;
  md.w_out = p.inv_out * c.obj_weight;
  ModelParams<float>& mf = p.mf;
  mf.omega = (float)md.omega;
  for (int i = 0; i < 8; ++i) mf.mrt[i] = (float)md.mrt[i];
  mf.pbb_scale = (float)md.pbb_scale;
  mf.pbb_q = (float)md.pbb_q;
  mf.obj_weight = (float)md.obj_weight;
  mf.w_in = (float)md.w_in;
  mf.w_out = (float)md.w_out;
  mf.cv_diss = (float)md.cv_diss;
  // boundary conditions of time t, with the inflow profiles tabulated into the scratch
  p.nbc = c.nbc;
  p.apply_bc = t >= 1;
  long long off = 0;
  for (int k = 0; k < c.nbc; ++k) {
    const lbm_bc& b = c.bc[k];
    const bool par = parabolic(b);
    if (par) {
      bc_parabola(c, b, g_prof_d + off);
      for (long long i = 0; i < bc_npos(b); ++i) g_prof_f[off + i] = (float)g_prof_d[off + i];
    }
    fill_devbc(b, t, INT_MAX, 1, par ? prof_d + off : nullptr, par ? prof_f + off : nullptr,
               p.bc[k]);
    if (bc_on_y_face(b)) p.bc_y = 1;
    if (par) off += bc_npos(b);
  }
  if (off > 0) {
    e = cudaMemcpyAsync(prof_d, g_prof_d, sizeof(double) * off, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(prof_f, g_prof_f, sizeof(float) * off, cudaMemcpyHostToDevice, st);
    // the host tables are reused by the next call: wait until they are on the device
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("profile upload: ") + cudaGetErrorString(e));
  }
  // the counter must start at zero whatever the previous call left behind
  e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  p.partial = partial;
  p.counter = counter;
  p.result = J_dev;
  p.fin = f_dev;
  p.gamma = gamma_dev;
  p.eval_obj = 1;
  launch(K_OBJECTIVE, grid, block, st, p, nullptr);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return LBM_OK;
}
