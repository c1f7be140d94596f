// lbm_capi.cu -- the C ABI of include/lbmgpu.h: handle life cycle, argument
// checking, device memory, the time-stepping drivers and the checkpointed
// gradient.  All numerical work is done by the kernels of kernels_*.cu; there
// is no host fallback.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_device.cuh"
#include "lbm_ops.h"
#include "state_pool.hpp"
#include "wang.hpp"

using namespace lbm;

namespace lbm {

bool bc_on_y_face(const lbm_bc& b) { return b.face == LBM_FACE_SOUTH || b.face == LBM_FACE_NORTH; }

int64_t bc_npos(const lbm_bc& b) {
  if (bc_on_y_face(b)) return (int64_t)(b.box[1] - b.box[0] + 1) * (b.box[5] - b.box[4] + 1);
  return (int64_t)(b.box[3] - b.box[2] + 1) * (b.box[5] - b.box[4] + 1);
}

double bc_time_factor(const lbm_bc& b, int t, int t_start) {
  if (b.time_law == LBM_TIME_SINE)
    return b.amp == 0. ? 0. : b.amp * sin(2. * M_PI * (double)t / b.period);
  if (b.time_law == LBM_TIME_RAMP) {
    // StageTemp (applications/Regenerator2d/regenerator2d.cc:53-69)
    if (t_start == INT_MAX || t <= t_start) return b.amp;
    const long long s = (long long)t - t_start;
    return b.amp + ((double)s < b.period ? sin(M_PI * (double)s / (2. * b.period)) : 1.);
  }
  return (b.amp == 0.) ? 1. : 1. + b.amp * sin(2. * M_PI * (double)t / b.period);
}

// (m^2 - (s-m)^2)/m^2 across the lattice along the face (m = (n-1)/2 of the
// tangential axis; applications/diffuser/diffuser.cc:22-31), times the same
// in z on D3Q19.
void bc_parabola(const lbm_config& c, const lbm_bc& b, double* out) {
  const bool yface = bc_on_y_face(b);
  const int n = yface ? c.nx : c.ny;
  const int s0 = yface ? b.box[0] : b.box[2], s1 = yface ? b.box[1] : b.box[3];
  const int ns = s1 - s0 + 1;
  for (int z = b.box[4]; z <= b.box[5]; ++z)
    for (int s = s0; s <= s1; ++s) {
      double mid = (double)(n - 1) / 2.;
      double pr = (mid * mid - (s - mid) * (s - mid)) / (mid * mid);
      if (c.lattice == LBM_D3Q19) {
        double mz = (double)(c.nz - 1) / 2.;
        pr *= (mz * mz - (z - mz) * (z - mz)) / (mz * mz);
      }
      out[(size_t)(z - b.box[4]) * ns + (s - s0)] = pr;
    }
}

void fill_devbc(const lbm_bc& b, int t, int t_start, int ncomp, const double* tab_d,
                const float* tab_f, DevBC& d) {
  d.kind = b.kind;
  d.face = b.face;
  d.profile = b.profile;
  for (int i = 0; i < 6; ++i) d.box[i] = b.box[i];
  d.tang_x = bc_on_y_face(b) ? 1 : 0;
  d.n_t = d.tang_x ? b.box[1] - b.box[0] + 1 : b.box[3] - b.box[2] + 1;
  d.ncomp = tab_d ? ncomp : 0;
  // value(t) = value * T(t), evaluated here once per launch
  d.value = b.value * bc_time_factor(b, t, t_start);
  d.value_f = (float)d.value;
  d.vshift = d.value - 1.;
  d.vshift_f = (float)d.vshift;
  const bool nodir = b.dir[0] == 0. && b.dir[1] == 0. && b.dir[2] == 0.;
  for (int a = 0; a < 3; ++a) {
    d.dir[a] = nodir ? (a == 0 ? 1. : 0.) : b.dir[a];
    d.dir_f[a] = (float)d.dir[a];
  }
  d.prof = tab_d;
  d.prof_f = tab_f;
}

bool objective_info(int id, ObjectiveInfo* out) {
  for (int k = 0; k < objective_count(ObjectiveList{}); ++k) {
    const ObjectiveInfo oi = objective_info_at(ObjectiveList{}, k);
    if (oi.id == id) {
      if (out) *out = oi;
      return true;
    }
  }
  return false;
}

void objective_norms(const lbm_config& c, double* inv_in, double* inv_out) {
  *inv_in = *inv_out = 0.;
  ObjectiveInfo oi;
  if (c.objective == LBM_OBJ_NONE || !objective_info(c.objective, &oi)) return;
  if (oi.uses & kUsesIn) {
    const int* a = c.obj_in;
    *inv_in = (double)(1. / ((a[1] - a[0] + 1) * (a[3] - a[2] + 1) * (a[5] - a[4] + 1)));
  }
  if (oi.uses & kUsesOut) {
    const int* b = c.obj_out;
    *inv_out = (double)(1. / ((b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1)));
  }
}

}  // namespace lbm

namespace {

thread_local std::string g_create_error;

const int kBlockThreads = 256;

struct Geometry {
  dim3 grid, block;
  unsigned nblocks;
};

Geometry make_geometry(int nx, int ny, int nz, int bx, int by) {
  Geometry g;
  g.block = dim3(bx, by, 1);
  g.grid = dim3((nx + bx - 1) / bx, (ny + by - 1) / by, nz);
  g.nblocks = g.grid.x * g.grid.y * g.grid.z;
  return g;
}

// Thread-block shapes the autotuner tries (x-major rows; 64, 128 or 256
// threads: the 64-thread ones spread lattices of a few thousand blocks more
// evenly over the SMs, e.g. the 128x64 FP64 channel's steps 6.2 -> 5.6 us
// forward and 12.3 -> 11.4 us reverse).
const int kShapes[][2] = {{256, 1}, {128, 2}, {64, 4}, {32, 8}, {128, 1}, {64, 2}, {32, 4},
                          {64, 1}, {32, 2}};

}  // namespace

struct lbm_handle {
  lbm_config cfg;
  int Q = 0, QF = 0, nmac = 0, dim = 2;
  int64_t ncell = 0;
  long long P = 0;       // plane stride (elements)
  size_t pop_bytes = 0;  // bytes per population value
  size_t adj_bytes = 0;  // bytes per adjoint value
  size_t gam_bytes = 0;  // bytes per design value
  LaunchFn launch = nullptr;
  ChangeFn change = nullptr;   // max |f_t - f_{t-1}| of two states (steady runs)
  cudaStream_t stream = nullptr;
  Geometry geo;       // initialisation / export kernels
  Geometry geo_fwd;   // forward step (autotuned)
  Geometry geo_adj;   // reverse step (autotuned)
  bool adj_lean = false;   // reverse step: the register-lean variant (autotuned)
  bool sens_atomic = false;   // reverse step adds to dJ/dgamma atomically (fits in L2)
  bool tuned = false;
  size_t partial_cap = 0;
  void* f[2] = {nullptr, nullptr};
  int cur = 0;
  void* gamma = nullptr;
  void* lam[2] = {nullptr, nullptr};
  int lcur = 0;
  double* sens = nullptr;
  double* partial = nullptr;
  unsigned* counter = nullptr;
  double* jdev = nullptr;
  size_t jcap = 0;
  double* stage = nullptr;     // FP64 AoS staging (ncell*Q)
  double* init_mac = nullptr;  // initial macros kept for lbm_gradient (device, may be null)
  std::vector<void*> slots;
  // per boundary: parabolic factors or the caller's table (lbm_set_bc_profile),
  // tab_nt rows of bc_npos * tab_ncomp values (device, FP64 and FP32 copies)
  double* bcprof_d[LBM_MAX_BC] = {};
  float* bcprof_f[LBM_MAX_BC] = {};
  int tab_nt[LBM_MAX_BC] = {};
  int tab_ncomp[LBM_MAX_BC] = {};
  int64_t table_gen = 0;   // bumped when a table moves to a new device buffer
  // first step whose state's objective counts (a steady phase before it adds none)
  int obj_from = 1;
  // step at which the last steady phase ended (start of LBM_TIME_RAMP ramps)
  int t_phase = INT_MAX;
  // 1/D of the regenerator efficiency, D = sum (1-gamma)(Tb - Ti) over obj_out
  double regen_invD = 0.;
  int t = 0;
  bool have_design = false, have_state = false, have_adjoint = false;
  bool accumulate = false;   // objective sums over steps into the warp partials
  int64_t launches = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::string err;
};

namespace {

int fail(lbm_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h)
    h->err = buf;
  else
    g_create_error = buf;
  return code;
}

#define CUDA_OR_FAIL(h, call)                                                              \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail((h), LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// *out = sum of partial[0..n) in a fixed order (one block of 1024 threads):
// the objective summed over time steps by the accumulating reductions.
__global__ void __launch_bounds__(1024) k_sum_partials(const double* __restrict__ partial,
                                                       long long n, double* __restrict__ out) {
  __shared__ double sh[32];
  double acc = 0.;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) tot += sh[w];
    *out = tot;
  }
}

// sens[c] += coef * (*J) over the cells of box b (x fastest): the design
// term every box cell shares (the regenerator efficiency's 1/D derivative).
__global__ void k_box_add_scaled(double* __restrict__ sens, int nx, int ny, int x0, int x1, int y0,
                                 int y1, int z0, int z1, const double* __restrict__ J, double coef) {
  const int bx = x1 - x0 + 1, by = y1 - y0 + 1;
  const long long n = (long long)bx * by * (z1 - z0 + 1);
  const double v = coef * (*J);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = x0 + (int)(i % bx);
    const int y = y0 + (int)((i / bx) % by);
    const int z = z0 + (int)(i / ((long long)bx * by));
    sens[((long long)z * ny + y) * nx + x] += v;
  }
}

size_t state_bytes(const lbm_handle* h) { return (size_t)h->Q * h->P * h->pop_bytes; }
size_t adjoint_bytes(const lbm_handle* h) { return (size_t)h->Q * h->P * h->adj_bytes; }
// Bytes one reverse step moves: the state, the adjoint in and out, the design
// and the FP64 dJ/dgamma read and written.
size_t reverse_step_bytes(const lbm_handle* h) {
  return state_bytes(h) + 2 * adjoint_bytes(h) + (size_t)h->P * (h->gam_bytes + 16);
}
// Whether a reverse step of that many bytes stays in this device's L2.
bool fits_in_l2(size_t bytes) {
  int dev = 0, l2 = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess) return false;
  return bytes <= (size_t)l2;
}

int check_box(const lbm_config& c, const int* b, int dim, const char* what) {
  int nz = dim == 3 ? c.nz : 1;
  if (b[0] < 0 || b[1] >= c.nx || b[0] > b[1] || b[2] < 0 || b[3] >= c.ny || b[2] > b[3] ||
      b[4] < 0 || b[5] >= nz || b[4] > b[5])
    return fail(nullptr, LBM_ERR_ARG, "%s box [%d,%d]x[%d,%d]x[%d,%d] outside the %dx%dx%d lattice",
                what, b[0], b[1], b[2], b[3], b[4], b[5], c.nx, c.ny, nz);
  return 0;
}

int validate(const lbm_config& c) {
  if (c.lattice != LBM_D2Q9 && c.lattice != LBM_D3Q19 && c.lattice != LBM_D2Q9_D2Q5)
    return fail(nullptr, LBM_ERR_ARG, "unknown lattice %d", c.lattice);
  if (c.collision != LBM_BGK && c.collision != LBM_MRT)
    return fail(nullptr, LBM_ERR_ARG, "unknown collision %d", c.collision);
  if (c.storage != LBM_STORE_FP64 && c.storage != LBM_STORE_FP32 && c.storage != LBM_STORE_FP16)
    return fail(nullptr, LBM_ERR_ARG, "unknown storage %d", c.storage);
  if (c.lattice == LBM_D2Q9_D2Q5 && c.collision != LBM_BGK)
    return fail(nullptr, LBM_ERR_SUP, "the thermal lattice supports BGK flow only");
  int dim = c.lattice == LBM_D3Q19 ? 3 : 2;
  if (c.nx < 3 || c.ny < 3 || (dim == 3 && c.nz < 3))
    return fail(nullptr, LBM_ERR_ARG, "lattice %dx%dx%d too small (>= 3 cells per axis)", c.nx,
                c.ny, c.nz);
  if ((double)c.nx * c.ny * (dim == 3 ? c.nz : 1) > 2.0e9)
    return fail(nullptr, LBM_ERR_ARG, "lattice too large");
  if (!(c.omega > 0. && c.omega < 2.))
    return fail(nullptr, LBM_ERR_ARG, "omega %g outside (0,2)", c.omega);
  if (!(c.interp_q > 0.) || !std::isfinite(c.interp_scale))
    return fail(nullptr, LBM_ERR_ARG, "interpolation q must be > 0");
  if (c.lattice == LBM_D2Q9_D2Q5 && (!(c.diffusivity > 0.) || !(c.ramp_ck > 0.) || !(c.ramp_q >= 0.)))
    return fail(nullptr, LBM_ERR_ARG, "thermal lattice needs diffusivity > 0, ramp_ck > 0, ramp_q >= 0");
  if (c.nbc < 0 || c.nbc > LBM_MAX_BC)
    return fail(nullptr, LBM_ERR_ARG, "nbc %d outside [0,%d]", c.nbc, LBM_MAX_BC);
  for (int k = 0; k < c.nbc; ++k) {
    const lbm_bc& b = c.bc[k];
    int rc = check_box(c, b.box, dim, "boundary");
    if (rc) return rc;
    if (b.face < LBM_FACE_WEST || b.face > LBM_FACE_NORTH)
      return fail(nullptr, LBM_ERR_ARG, "boundary %d: unknown face %d", k, b.face);
    // the operators each kind has per face (the reference's descriptors give
    // PETSC_ERR_SUP for the others, boundaryConditions/ZouHe2d.hh:181-236)
    const int w = 1 << LBM_FACE_WEST, e = 1 << LBM_FACE_EAST, all = 15;
    int faces = 0;
    if (dim == 3) {
      faces = b.kind == LBM_BC_VELOCITY ? w : b.kind == LBM_BC_PRESSURE ? e : 0;
      if (!((1 << b.face) & faces))
        return fail(nullptr, LBM_ERR_SUP,
                    "D3Q19 supports the Hecht velocity west and pressure east faces only");
    } else {
      switch (b.kind) {
        case LBM_BC_VELOCITY:
        case LBM_BC_PRESSURE:
          faces = all;
          break;
        case LBM_BC_VELOCITY_STANDARD:
          faces = w;
          break;
        case LBM_BC_PRESSURE_STANDARD:
          faces = w | e;
          break;
        case LBM_BC_TEMPERATURE:
          if (c.lattice != LBM_D2Q9_D2Q5)
            return fail(nullptr, LBM_ERR_SUP, "temperature boundary needs the thermal lattice");
          faces = w;
          break;
        default:
          return fail(nullptr, LBM_ERR_SUP, "boundary kind %d not supported", b.kind);
      }
      if (!((1 << b.face) & faces))
        return fail(nullptr, LBM_ERR_SUP, "boundary %d: kind %d has no operator on face %d", k,
                    b.kind, b.face);
    }
    bool ok = false;
    switch (b.face) {
      case LBM_FACE_WEST: ok = b.box[0] == 0 && b.box[1] == 0; break;
      case LBM_FACE_EAST: ok = b.box[0] == c.nx - 1 && b.box[1] == c.nx - 1; break;
      case LBM_FACE_SOUTH: ok = b.box[2] == 0 && b.box[3] == 0; break;
      default: ok = b.box[2] == c.ny - 1 && b.box[3] == c.ny - 1; break;
    }
    if (!ok) return fail(nullptr, LBM_ERR_ARG, "boundary %d: box does not lie on its face", k);
    if (b.profile != LBM_PROFILE_UNIFORM && b.profile != LBM_PROFILE_PARABOLIC &&
        b.profile != LBM_PROFILE_TABLE)
      return fail(nullptr, LBM_ERR_ARG, "boundary %d: unknown profile %d", k, b.profile);
    if (b.time_law != LBM_TIME_OFFSET_SINE && b.time_law != LBM_TIME_SINE &&
        b.time_law != LBM_TIME_RAMP)
      return fail(nullptr, LBM_ERR_ARG, "boundary %d: unknown time law %d", k, b.time_law);
    if (b.time_law == LBM_TIME_RAMP && !(b.period > 0.))
      return fail(nullptr, LBM_ERR_ARG, "boundary %d: a ramp needs period > 0", k);
    if (b.amp != 0. && !(b.period > 0.))
      return fail(nullptr, LBM_ERR_ARG, "boundary %d: oscillation needs period > 0", k);
    if (!std::isfinite(b.value) || !std::isfinite(b.amp))
      return fail(nullptr, LBM_ERR_ARG, "boundary %d: bad value", k);
    for (int a = 0; a < 3; ++a)
      if (!std::isfinite(b.dir[a])) return fail(nullptr, LBM_ERR_ARG, "boundary %d: bad direction", k);
  }
  for (int i = 0; i < 4; ++i)
    if (!std::isfinite(c.obj_param[i]))
      return fail(nullptr, LBM_ERR_ARG, "objective parameter %d is not finite", i);
  if (c.objective == LBM_OBJ_REGENERATOR_EFFICIENCY && c.obj_param[1] == c.obj_param[0])
    return fail(nullptr, LBM_ERR_ARG, "regenerator efficiency needs Tb != Ti (obj_param[1], [0])");
  if (c.objective != LBM_OBJ_NONE) {
    ObjectiveInfo oi;
    if (!objective_info(c.objective, &oi))
      return fail(nullptr, LBM_ERR_ARG, "unknown objective %d", c.objective);
    if (oi.thermal && c.lattice != LBM_D2Q9_D2Q5)
      return fail(nullptr, LBM_ERR_SUP, "objective %d needs the thermal lattice", c.objective);
    if (oi.uses & kUsesIn) {
      int rc = check_box(c, c.obj_in, dim, "objective inflow");
      if (rc) return rc;
    }
    if (oi.uses & kUsesOut) {
      int rc = check_box(c, c.obj_out, dim, "objective outflow");
      if (rc) return rc;
    }
  }
  return 0;
}

void destroy_buffers(lbm_handle* h) {
  for (void*& p : h->f) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  for (void*& p : h->lam) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  for (void* s : h->slots)
    if (s) cudaFree(s);
  h->slots.clear();
  void* ps[] = {h->gamma, h->sens, h->partial, h->counter, h->jdev, h->stage, h->init_mac};
  for (void* p : ps)
    if (p) cudaFree(p);
  for (int k = 0; k < LBM_MAX_BC; ++k) {
    if (h->bcprof_d[k]) cudaFree(h->bcprof_d[k]);
    if (h->bcprof_f[k]) cudaFree(h->bcprof_f[k]);
    h->bcprof_d[k] = nullptr;
    h->bcprof_f[k] = nullptr;
  }
  h->gamma = h->sens = h->partial = nullptr;
  h->counter = nullptr;
  h->jdev = h->stage = h->init_mac = nullptr;
  for (cudaEvent_t& e : h->ev)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  if (h->stream) cudaStreamDestroy(h->stream);
  h->stream = nullptr;
}

KParams base_params(const lbm_handle* h, int t) {
  const lbm_config& c = h->cfg;
  KParams p;
  memset(&p, 0, sizeof(p));
  p.nx = c.nx;
  p.ny = c.ny;
  p.nz = h->dim == 3 ? c.nz : 1;
  p.P = h->P;
  p.step = (unsigned)t;
  p.key_fwd = step_key(p.step, kSaltForward);
  p.key_adj = step_key(p.step, kSaltAdjoint);
  p.omega = c.omega;
  for (int i = 0; i < 8; ++i) p.mrt[i] = c.mrt[i];
  p.pbb_scale = c.interp_scale;
  p.pbb_q = c.interp_q;
  p.diff = c.diffusivity;
  p.ramp_q = c.ramp_q;
  p.ramp_ck = c.ramp_ck;
  p.heat_rate = c.heat_rate;
  p.heat_T = c.heat_T;
  p.nbc = c.nbc;
  p.apply_bc = t >= 1;
  for (int k = 0; k < c.nbc; ++k) {
    const lbm_bc& b = c.bc[k];
    // a table row per time step (t mod nt); parabolic factors have one row
    const int64_t row = h->tab_nt[k] > 0 ? (int64_t)(t % h->tab_nt[k]) * bc_npos(b) *
                                               (h->tab_ncomp[k] > 0 ? h->tab_ncomp[k] : 1)
                                         : 0;
    fill_devbc(b, t, h->t_phase, h->tab_ncomp[k] > 0 ? h->tab_ncomp[k] : 1,
               h->bcprof_d[k] ? h->bcprof_d[k] + row : nullptr,
               h->bcprof_f[k] ? h->bcprof_f[k] + row : nullptr, p.bc[k]);
    if (bc_on_y_face(b)) p.bc_y = 1;
  }
  p.objective = c.objective;
  p.obj_weight = c.obj_weight;
  for (int i = 0; i < 6; ++i) {
    p.obj_in[i] = c.obj_in[i];
    p.obj_out[i] = c.obj_out[i];
  }
  objective_norms(c, &p.inv_in, &p.inv_out);
  ModelParams<double>& md = p.md;
  md.omega = c.omega;
  for (int i = 0; i < 8; ++i) md.mrt[i] = c.mrt[i];
  md.pbb_scale = c.interp_scale;
  md.pbb_q = c.interp_q;
  md.diff = c.diffusivity;
  md.ramp_q = c.ramp_q;
  md.ramp_ck = c.ramp_ck;
  md.heat_rate = c.heat_rate;
  md.heat_T = c.heat_T;
  md.obj_weight = c.obj_weight;
  md.w_in = p.inv_in * c.obj_weight;
  md.w_out = p.inv_out * c.obj_weight;
  {
    double nu = (1. / c.omega - 0.5) / 3.;
    md.cv_diss = 4.5 * nu * c.omega * c.omega;
  }
  md.obj_p[0] = c.obj_param[0];
  md.obj_p[1] = c.objective == LBM_OBJ_REGENERATOR_EFFICIENCY ? c.obj_weight * h->regen_invD : 0.;
  ModelParams<float>& mf = p.mf;
  mf.omega = (float)md.omega;
  for (int i = 0; i < 8; ++i) mf.mrt[i] = (float)md.mrt[i];
  mf.pbb_scale = (float)md.pbb_scale;
  mf.pbb_q = (float)md.pbb_q;
  mf.diff = (float)md.diff;
  mf.ramp_q = (float)md.ramp_q;
  mf.ramp_ck = (float)md.ramp_ck;
  mf.heat_rate = (float)md.heat_rate;
  mf.heat_T = (float)md.heat_T;
  mf.obj_weight = (float)md.obj_weight;
  mf.w_in = (float)md.w_in;
  mf.w_out = (float)md.w_out;
  mf.cv_diss = (float)md.cv_diss;
  mf.obj_p[0] = (float)md.obj_p[0];
  mf.obj_p[1] = (float)md.obj_p[1];
  p.partial = h->partial;
  p.counter = h->counter;
  p.accumulate = h->accumulate ? 1 : 0;
  p.gamma = h->gamma;
  p.sens = h->sens;
  p.sens_atomic = h->sens_atomic ? 1 : 0;
  return p;
}

// A boundary with LBM_PROFILE_TABLE whose table lbm_set_bc_profile never set
// (-1 if none).
int missing_table(const lbm_handle* h) {
  for (int k = 0; k < h->cfg.nbc; ++k)
    if (h->cfg.bc[k].profile == LBM_PROFILE_TABLE && !h->bcprof_d[k]) return k;
  return -1;
}

int launch(lbm_handle* h, int kind, const KParams& p, double* aux) {
  if (p.apply_bc) {
    const int k = missing_table(h);
    if (k >= 0)
      return fail(h, LBM_ERR_STATE, "boundary %d has LBM_PROFILE_TABLE but no table "
                  "(lbm_set_bc_profile)", k);
  }
  const Geometry& g = kind == K_FORWARD                              ? h->geo_fwd
                      : (kind == K_ADJOINT || kind == K_ADJOINT_LEAN) ? h->geo_adj
                                                                       : h->geo;
  h->launch(kind, g.grid, g.block, h->stream, p, aux);
  h->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, "kernel launch %d: %s", kind, cudaGetErrorString(e));
  return 0;
}

int ensure_jcap(lbm_handle* h, size_t n) {
  if (n <= h->jcap) return 0;
  if (h->jdev) cudaFree(h->jdev);
  h->jdev = nullptr;
  size_t cap = n < 1024 ? 1024 : n;
  CUDA_OR_FAIL(h, cudaMalloc(&h->jdev, cap * sizeof(double)));
  h->jcap = cap;
  return 0;
}

int ensure_stage(lbm_handle* h) {
  if (h->stage) return 0;
  CUDA_OR_FAIL(h, cudaMalloc(&h->stage, (size_t)h->ncell * h->Q * sizeof(double)));
  return 0;
}

// Objective summed over time steps without a per-step reduction: zero the
// warp partials, let every step's reduction add into them, sum them once.
int begin_accumulate(lbm_handle* h, cudaStream_t st) {
  CUDA_OR_FAIL(h, cudaMemsetAsync(h->partial, 0, h->partial_cap * sizeof(double), st));
  h->accumulate = true;
  return 0;
}
int begin_accumulate(lbm_handle* h) { return begin_accumulate(h, h->stream); }

int end_accumulate(lbm_handle* h, double* out, cudaStream_t st) {
  h->accumulate = false;
  k_sum_partials<<<1, 1024, 0, st>>>(h->partial, (long long)h->partial_cap, out);
  h->launches++;
  CUDA_OR_FAIL(h, cudaGetLastError());
  return 0;
}
int end_accumulate(lbm_handle* h, double* out) { return end_accumulate(h, out, h->stream); }

// Buffer b of a handle's state pool: 0 and 1 are the state buffers, 2 .. K+1
// the checkpoint slots' (see StatePool).
void* pool_buffer(lbm_handle* h, int b) { return b < 2 ? h->f[b] : h->slots[b - 2]; }

// One forward step f~_t (in) -> f~_{t+1} (out); result (may be null) receives F(f_t).
int forward_launch(lbm_handle* h, const void* in, void* out, double* result) {
  KParams p = base_params(h, h->t);
  p.fin = in;
  p.fout = out;
  p.eval_obj = (result != nullptr && h->cfg.objective != LBM_OBJ_NONE) ? 1 : 0;
  p.result = result;
  int rc = launch(h, K_FORWARD, p, nullptr);
  if (rc) return rc;
  h->t += 1;
  return 0;
}

int forward_step(lbm_handle* h, double* result) {
  int rc = forward_launch(h, h->f[h->cur], h->f[1 - h->cur], result);
  if (rc) return rc;
  h->cur ^= 1;
  return 0;
}

int objective_at(lbm_handle* h, const void* f, double* result) {
  KParams p = base_params(h, h->t);
  p.fin = f;
  p.eval_obj = 1;
  p.result = result;
  return launch(h, K_OBJECTIVE, p, nullptr);
}

int objective_only(lbm_handle* h, double* result) { return objective_at(h, h->f[h->cur], result); }

// One reverse step at the forward state f_t held in `f`.
int adjoint_at(lbm_handle* h, const void* f) {
  KParams p = base_params(h, h->t);
  p.fin = f;
  p.lam_in = h->lam[h->lcur];
  p.lam_out = h->lam[1 - h->lcur];
  p.eval_obj = (h->t >= h->obj_from && h->cfg.objective != LBM_OBJ_NONE) ? 1 : 0;
  int rc = launch(h, h->adj_lean ? K_ADJOINT_LEAN : K_ADJOINT, p, nullptr);
  if (rc) return rc;
  h->lcur ^= 1;
  return 0;
}

int adjoint_step(lbm_handle* h) { return adjoint_at(h, h->f[h->cur]); }

int sync(lbm_handle* h) {
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, "device error: %s", cudaGetErrorString(e));
  return 0;
}

int zero_adjoint(lbm_handle* h) {
  for (void* p : h->lam) CUDA_OR_FAIL(h, cudaMemsetAsync(p, 0, adjoint_bytes(h), h->stream));
  CUDA_OR_FAIL(h, cudaMemsetAsync(h->sens, 0, (size_t)h->ncell * sizeof(double), h->stream));
  h->lcur = 0;
  return 0;
}

int init_into(lbm_handle* h, void* out) {
  KParams p = base_params(h, 0);
  p.fout = out;
  int rc = launch(h, K_INIT, p, h->init_mac);
  if (rc) return rc;
  h->t = 0;
  h->have_state = true;
  return 0;
}

int init_state(lbm_handle* h) { return init_into(h, h->f[h->cur]); }

// *out = max |f_t - f_{t-1}| over every population, the state `cur` of step
// t_cur and `prev` of step t_cur - 1 each with its step's boundary conditions
// (the reference's steady test compares post-boundary states).  bits: one
// device word of scratch.  Waits for the result.
int measure_change(lbm_handle* h, const void* cur, const void* prev, int t_cur,
                   unsigned long long* bits, double* out) {
  KParams pc = base_params(h, t_cur), pp = base_params(h, t_cur - 1);
  pc.fin = cur;
  pp.fin = prev;
  CUDA_OR_FAIL(h, cudaMemsetAsync(bits, 0, sizeof(unsigned long long), h->stream));
  h->change(h->geo.grid, h->geo.block, h->stream, pc, pp, bits);
  h->launches++;
  CUDA_OR_FAIL(h, cudaGetLastError());
  unsigned long long hb = 0;
  CUDA_OR_FAIL(h, cudaMemcpyAsync(&hb, bits, sizeof(hb), cudaMemcpyDeviceToHost, h->stream));
  CUDA_OR_FAIL(h, cudaStreamSynchronize(h->stream));
  memcpy(out, &hb, sizeof(double));
  return 0;
}

// D = sum over obj_out of (1 - gamma)(Tb - Ti) of the regenerator efficiency,
// from the design on the host.
void set_regen_denominator(lbm_handle* h, const double* gamma) {
  const lbm_config& c = h->cfg;
  if (c.objective != LBM_OBJ_REGENERATOR_EFFICIENCY) return;
  const int* b = c.obj_out;
  double d = 0.;
  for (int z = b[4]; z <= b[5]; ++z)
    for (int y = b[2]; y <= b[3]; ++y)
      for (int x = b[0]; x <= b[1]; ++x)
        d += (1. - gamma[((int64_t)z * c.ny + y) * c.nx + x]) * (c.obj_param[1] - c.obj_param[0]);
  h->regen_invD = 1. / d;   // no solid in the box: inf, and the objective is reported non-finite
}

// The objective's design term shared by every box cell, from the objective
// value *J (device): the regenerator efficiency's d(1/D)/dgamma part,
// J (Tb - Ti) / D.  Nothing for the other objectives.
int add_design_term(lbm_handle* h, const double* J) {
  const lbm_config& c = h->cfg;
  if (c.objective != LBM_OBJ_REGENERATOR_EFFICIENCY) return 0;
  const int* b = c.obj_out;
  const double coef = (c.obj_param[1] - c.obj_param[0]) * h->regen_invD;
  const long long n = (long long)(b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1);
  const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 1024);
  k_box_add_scaled<<<blocks, 256, 0, h->stream>>>(h->sens, c.nx, c.ny, b[0], b[1], b[2], b[3], b[4],
                                                  b[5], J, coef);
  h->launches++;
  CUDA_OR_FAIL(h, cudaGetLastError());
  return 0;
}

}  // namespace

namespace lbm {
void set_global_error(const char* msg) { g_create_error = msg ? msg : ""; }
int validate_config(const lbm_config& c) { return validate(c); }
}  // namespace lbm

// ===========================================================================

extern "C" {

void lbm_config_default(lbm_config* c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->lattice = LBM_D2Q9;
  c->collision = LBM_BGK;
  c->storage = LBM_STORE_FP64;
  c->nx = c->ny = c->nz = 1;
  c->omega = 1.;
  const double d3[8] = {1.19, 1.4, 1.2, 1.4, 1.4, 3., -5.5, -0.5};
  for (int i = 0; i < 8; ++i) c->mrt[i] = d3[i];
  c->interp_scale = 1.;
  c->interp_q = 1.;
  c->ramp_q = 1.;
  c->ramp_ck = 1.;
  c->heat_T = 1.;
  c->obj_weight = 1.;
}

const char* lbm_last_error(const lbm_handle* h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

int lbm_create(const lbm_config* cfg, lbm_handle** out) {
  if (!cfg || !out) return fail(nullptr, LBM_ERR_ARG, "null argument");
  *out = nullptr;
  int rc = validate(*cfg);
  if (rc) return rc;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, LBM_ERR_CUDA, "no CUDA device available (%s)",
                e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
  lbm_handle* h = new (std::nothrow) lbm_handle();
  if (!h) return fail(nullptr, LBM_ERR_MEM, "host allocation failed");
  h->cfg = *cfg;
  const lbm_config& c = h->cfg;
  h->dim = c.lattice == LBM_D3Q19 ? 3 : 2;
  if (h->dim == 2) h->cfg.nz = 1;
  h->Q = c.lattice == LBM_D2Q9 ? 9 : c.lattice == LBM_D3Q19 ? 19 : 14;
  h->QF = c.lattice == LBM_D3Q19 ? 19 : 9;
  h->nmac = c.lattice == LBM_D2Q9 ? 3 : 4;
  h->ncell = (int64_t)c.nx * c.ny * h->cfg.nz;
  h->P = (h->ncell + 127) / 128 * 128;
  if ((int64_t)h->Q * h->P >= (int64_t)INT32_MAX) {
    const long long ncell = (long long)h->ncell;
    delete h;
    return fail(nullptr, LBM_ERR_SUP, "lattice of %lld cells too large for 32-bit population offsets",
                ncell);
  }
  h->pop_bytes = c.storage == LBM_STORE_FP64 ? 8 : c.storage == LBM_STORE_FP32 ? 4 : 2;
  h->adj_bytes = c.storage == LBM_STORE_FP64 ? 8 : 4;
  h->gam_bytes = c.storage == LBM_STORE_FP64 ? 8 : 4;
  h->sens_atomic = fits_in_l2(reverse_step_bytes(h));
  h->launch = c.lattice == LBM_D2Q9    ? launcher_d2q9(c.collision, c.storage)
              : c.lattice == LBM_D3Q19 ? launcher_d3q19(c.collision, c.storage)
                                       : launcher_thermal(c.collision, c.storage);
  h->change = c.lattice == LBM_D2Q9    ? change_fn_d2q9(c.collision, c.storage)
              : c.lattice == LBM_D3Q19 ? change_fn_d3q19(c.collision, c.storage)
                                       : change_fn_thermal(c.collision, c.storage);
  if (!h->launch || !h->change) {
    const int lat = c.lattice, coll = c.collision, stor = c.storage;   // c is h->cfg
    delete h;
    return fail(nullptr, LBM_ERR_SUP, "no kernel for lattice %d collision %d storage %d", lat, coll,
                stor);
  }
  // thread blocks: 256 threads, x-major rows
  int bx = c.nx >= 256 ? 256 : ((c.nx + 31) / 32) * 32;
  if (bx > 256) bx = 256;
  int by = kBlockThreads / bx;
  if (by < 1) by = 1;
  h->geo = make_geometry(c.nx, c.ny, h->cfg.nz, bx, by);
  h->geo_fwd = h->geo;
  h->geo_adj = h->geo;
  // partial sums: one slot per warp of the largest grid any tuned shape gives
  for (const auto& sh : kShapes) {
    Geometry g = make_geometry(c.nx, c.ny, h->cfg.nz, sh[0], sh[1]);
    const size_t slots = (size_t)g.nblocks * (size_t)(sh[0] * sh[1] / 32);
    if (slots > h->partial_cap) h->partial_cap = slots;
  }

#define ALLOC(ptr, bytes)                                                                  \
  do {                                                                                     \
    const size_t nbytes_ = (bytes);                                                        \
    cudaError_t ee = cudaMalloc((void**)&(ptr), nbytes_);                                  \
    if (ee != cudaSuccess) {                                                               \
      destroy_buffers(h);                                                                  \
      delete h;                                                                            \
      return fail(nullptr, ee == cudaErrorMemoryAllocation ? LBM_ERR_MEM : LBM_ERR_CUDA,   \
                  "cudaMalloc(%zu bytes): %s", nbytes_, cudaGetErrorString(ee));           \
    }                                                                                      \
  } while (0)

  e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return fail(nullptr, LBM_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  for (int i = 0; i < 4; ++i) {
    e = cudaEventCreate(&h->ev[i]);
    if (e != cudaSuccess) {
      h->ev[i] = nullptr;
      destroy_buffers(h);
      delete h;
      return fail(nullptr, LBM_ERR_CUDA, "cudaEventCreate: %s", cudaGetErrorString(e));
    }
  }
  ALLOC(h->f[0], state_bytes(h));
  ALLOC(h->f[1], state_bytes(h));
  ALLOC(h->lam[0], adjoint_bytes(h));
  ALLOC(h->lam[1], adjoint_bytes(h));
  ALLOC(h->gamma, (size_t)h->P * h->gam_bytes);
  ALLOC(h->sens, (size_t)h->P * sizeof(double));
  ALLOC(h->partial, h->partial_cap * sizeof(double));
  ALLOC(h->counter, sizeof(unsigned));
  // Inflow profile factors over each parabolic velocity boundary box,
  // tabulated once (tables of LBM_PROFILE_TABLE boundaries come from
  // lbm_set_bc_profile).
  for (int k = 0; k < c.nbc; ++k) {
    const lbm_bc& b = c.bc[k];
    if ((b.kind != LBM_BC_VELOCITY && b.kind != LBM_BC_VELOCITY_STANDARD) ||
        b.profile != LBM_PROFILE_PARABOLIC)
      continue;
    std::vector<double> pd((size_t)bc_npos(b));
    bc_parabola(c, b, pd.data());
    std::vector<float> pf(pd.begin(), pd.end());
    ALLOC(h->bcprof_d[k], pd.size() * sizeof(double));
    ALLOC(h->bcprof_f[k], pf.size() * sizeof(float));
    cudaMemcpy(h->bcprof_d[k], pd.data(), pd.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(h->bcprof_f[k], pf.data(), pf.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
#undef ALLOC
  cudaMemsetAsync(h->counter, 0, sizeof(unsigned), h->stream);
  cudaMemsetAsync(h->f[0], 0, state_bytes(h), h->stream);
  cudaMemsetAsync(h->f[1], 0, state_bytes(h), h->stream);
  if (zero_adjoint(h) || sync(h)) {
    std::string msg = h->err;
    destroy_buffers(h);
    delete h;
    return fail(nullptr, LBM_ERR_CUDA, "initialisation failed: %s", msg.c_str());
  }
  *out = h;
  return LBM_OK;
}

int lbm_destroy(lbm_handle* h) {
  if (!h) return LBM_OK;
  cudaStreamSynchronize(h->stream);
  destroy_buffers(h);
  delete h;
  return LBM_OK;
}

int lbm_get_dims(const lbm_handle* h, int dims[3]) {
  if (!h || !dims) return fail(nullptr, LBM_ERR_ARG, "null argument");
  dims[0] = h->cfg.nx;
  dims[1] = h->cfg.ny;
  dims[2] = h->dim == 3 ? h->cfg.nz : 1;
  return LBM_OK;
}

int lbm_get_sizes(const lbm_handle* h, int64_t* ncells, int* npop) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (ncells) *ncells = h->ncell;
  if (npop) *npop = h->Q;
  return LBM_OK;
}

int lbm_set_bc_profile(lbm_handle* h, int k, int nt, int ncomp, const double* table) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (k < 0 || k >= h->cfg.nbc) return fail(h, LBM_ERR_ARG, "boundary %d outside [0,%d)", k, h->cfg.nbc);
  const lbm_bc& b = h->cfg.bc[k];
  if (b.profile != LBM_PROFILE_TABLE)
    return fail(h, LBM_ERR_STATE, "boundary %d was not configured with LBM_PROFILE_TABLE", k);
  if (!table) return fail(h, LBM_ERR_ARG, "null table");
  if (nt < 1) return fail(h, LBM_ERR_ARG, "table needs nt >= 1 rows");
  const bool vel = b.kind == LBM_BC_VELOCITY || b.kind == LBM_BC_VELOCITY_STANDARD;
  if (!(ncomp == 1 || (vel && ncomp == h->dim)))
    return fail(h, LBM_ERR_ARG, "boundary %d: %d values per cell (1, or %d for a velocity)", k,
                ncomp, h->dim);
  const size_t n = (size_t)nt * (size_t)bc_npos(b) * (size_t)ncomp;
  if (n > ((size_t)1 << 31)) return fail(h, LBM_ERR_ARG, "table of %zu values too large", n);
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(table[i])) return fail(h, LBM_ERR_NONFINITE, "table value %zu is not finite", i);
  std::vector<float> tf(table, table + n);
  const size_t old_n = h->bcprof_d[k] ? (size_t)(h->tab_nt[k] > 0 ? h->tab_nt[k] : 1) *
                                            (size_t)bc_npos(b) *
                                            (size_t)(h->tab_ncomp[k] > 0 ? h->tab_ncomp[k] : 1)
                                      : 0;
  // finish whatever still reads the old table before it changes (the handle's
  // own stream, or the stream of a batch it belongs to)
  CUDA_OR_FAIL(h, cudaDeviceSynchronize());
  // captured graphs hold the table's address and layout: a new one needs a new capture
  if (old_n != n || h->tab_nt[k] != nt || h->tab_ncomp[k] != ncomp) h->table_gen++;
  if (old_n != n) {
    if (h->bcprof_d[k]) cudaFree(h->bcprof_d[k]);
    if (h->bcprof_f[k]) cudaFree(h->bcprof_f[k]);
    h->bcprof_d[k] = nullptr;
    h->bcprof_f[k] = nullptr;
    h->tab_nt[k] = h->tab_ncomp[k] = 0;
    cudaError_t e = cudaMalloc((void**)&h->bcprof_d[k], n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->bcprof_f[k], n * sizeof(float));
    if (e != cudaSuccess) {
      if (h->bcprof_d[k]) cudaFree(h->bcprof_d[k]);
      h->bcprof_d[k] = nullptr;
      h->bcprof_f[k] = nullptr;
      return fail(h, e == cudaErrorMemoryAllocation ? LBM_ERR_MEM : LBM_ERR_CUDA,
                  "table allocation: %s", cudaGetErrorString(e));
    }
  }
  CUDA_OR_FAIL(h, cudaMemcpy(h->bcprof_d[k], table, n * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_OR_FAIL(h, cudaMemcpy(h->bcprof_f[k], tf.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  h->tab_nt[k] = nt;
  h->tab_ncomp[k] = ncomp;
  return LBM_OK;
}

int lbm_set_design(lbm_handle* h, const double* gamma) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!gamma) return fail(h, LBM_ERR_ARG, "null design pointer");
  for (int64_t i = 0; i < h->ncell; ++i) {
    double g = gamma[i];
    if (!std::isfinite(g)) return fail(h, LBM_ERR_NONFINITE, "design value %lld is not finite", (long long)i);
    if (g < 0. || g > 1.) return fail(h, LBM_ERR_ARG, "design value %lld = %g outside [0,1]", (long long)i, g);
  }
  int rc = ensure_stage(h);
  if (rc) return rc;
  set_regen_denominator(h, gamma);
  CUDA_OR_FAIL(h, cudaMemcpyAsync(h->stage, gamma, (size_t)h->ncell * sizeof(double),
                                  cudaMemcpyHostToDevice, h->stream));
  KParams p = base_params(h, 0);
  rc = launch(h, K_GAMMA, p, h->stage);
  if (rc) return rc;
  rc = sync(h);
  if (rc) return rc;
  h->have_design = true;
  return LBM_OK;
}

int lbm_set_design_device(lbm_handle* h, const double* gamma_dev) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!gamma_dev) return fail(h, LBM_ERR_ARG, "null design pointer");
  // the caller's producing work must be complete before this stream reads it
  CUDA_OR_FAIL(h, cudaDeviceSynchronize());
  if (h->cfg.objective == LBM_OBJ_REGENERATOR_EFFICIENCY) {
    std::vector<double> g((size_t)h->ncell);
    CUDA_OR_FAIL(h, cudaMemcpy(g.data(), gamma_dev, g.size() * sizeof(double), cudaMemcpyDeviceToHost));
    set_regen_denominator(h, g.data());
  }
  KParams p = base_params(h, 0);
  int rc = launch(h, K_GAMMA, p, const_cast<double*>(gamma_dev));
  if (rc) return rc;
  rc = sync(h);
  if (rc) return rc;
  h->have_design = true;
  return LBM_OK;
}

int lbm_get_sensitivity_device(const lbm_handle* h, const double** sens_dev) {
  if (!h || !sens_dev) return fail(nullptr, LBM_ERR_ARG, "null argument");
  *sens_dev = h->sens;
  return LBM_OK;
}

int lbm_init_equilibrium(lbm_handle* h, const double* macros) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (macros) {
    size_t n = (size_t)h->ncell * h->nmac;
    for (size_t i = 0; i < n; ++i)
      if (!std::isfinite(macros[i])) return fail(h, LBM_ERR_NONFINITE, "initial macro %zu not finite", i);
    if (!h->init_mac) CUDA_OR_FAIL(h, cudaMalloc(&h->init_mac, n * sizeof(double)));
    CUDA_OR_FAIL(h, cudaMemcpyAsync(h->init_mac, macros, n * sizeof(double), cudaMemcpyHostToDevice,
                                    h->stream));
  } else if (h->init_mac) {
    cudaFree(h->init_mac);
    h->init_mac = nullptr;
  }
  h->t_phase = INT_MAX;   // a new run: no steady phase yet
  h->obj_from = 1;
  int rc = init_state(h);
  if (rc) return rc;
  return sync(h);
}

int lbm_forward_steady(lbm_handle* h, int max_steps, int check_every, double tol, int* steps,
                       double* change) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (max_steps < 1 || check_every < 1) return fail(h, LBM_ERR_ARG, "need max_steps >= 1 and check_every >= 1");
  if (!(tol >= 0.)) return fail(h, LBM_ERR_ARG, "tol must be >= 0");
  if (!h->have_design) return fail(h, LBM_ERR_STATE, "no design set (lbm_set_design)");
  if (!h->have_state) return fail(h, LBM_ERR_STATE, "no state (lbm_init_equilibrium)");
  int rc = ensure_jcap(h, 1);
  if (rc) return rc;
  unsigned long long* bits = (unsigned long long*)h->jdev;
  double last = -1.;
  int k = 0;
  while (k < max_steps) {
    if ((rc = forward_step(h, nullptr))) return rc;
    ++k;
    if (k % check_every == 0 || k == max_steps) {
      // the step's input is intact in the other state buffer
      if ((rc = measure_change(h, h->f[h->cur], h->f[1 - h->cur], h->t, bits, &last))) return rc;
      if (!std::isfinite(last)) return fail(h, LBM_ERR_NONFINITE, "state is not finite at step %d", h->t);
      if (last < tol) break;
    }
  }
  if ((rc = sync(h))) return rc;
  h->t_phase = h->t;   // LBM_TIME_RAMP boundaries start from here
  if (steps) *steps = k;
  if (change) *change = last;
  return LBM_OK;
}

int lbm_forward(lbm_handle* h, int nsteps, double* J_steps, double* J_sum) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (nsteps < 0) return fail(h, LBM_ERR_ARG, "nsteps %d < 0", nsteps);
  if (!h->have_design) return fail(h, LBM_ERR_STATE, "no design set (lbm_set_design)");
  if (!h->have_state) return fail(h, LBM_ERR_STATE, "no state (lbm_init_equilibrium)");
  if (J_sum) *J_sum = 0.;
  if (nsteps == 0) return LBM_OK;
  bool obj = h->cfg.objective != LBM_OBJ_NONE;
  int rc = ensure_jcap(h, (size_t)nsteps);
  if (rc) return rc;
  const bool sum_only = obj && !J_steps;
  if (sum_only && (rc = begin_accumulate(h))) return rc;
  for (int k = 0; k < nsteps; ++k) {
    rc = forward_step(h, (obj && k > 0) ? h->jdev + (k - 1) : nullptr);
    if (rc) {
      h->accumulate = false;
      return rc;
    }
  }
  if (obj) {
    rc = objective_only(h, h->jdev + (nsteps - 1));
    if (!rc && sum_only) rc = end_accumulate(h, h->jdev);
    h->accumulate = false;
    if (rc) return rc;
  }
  rc = sync(h);
  if (rc) return rc;
  if (sum_only) {
    double acc = 0.;
    CUDA_OR_FAIL(h, cudaMemcpy(&acc, h->jdev, sizeof(double), cudaMemcpyDeviceToHost));
    if (!std::isfinite(acc)) return fail(h, LBM_ERR_NONFINITE, "objective is not finite");
    if (J_sum) *J_sum = acc;
  } else if (obj) {
    std::vector<double> js((size_t)nsteps);
    CUDA_OR_FAIL(h, cudaMemcpy(js.data(), h->jdev, js.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double acc = 0.;
    for (int k = 0; k < nsteps; ++k) acc += js[k];
    if (!std::isfinite(acc)) return fail(h, LBM_ERR_NONFINITE, "objective is not finite");
    if (J_steps) memcpy(J_steps, js.data(), js.size() * sizeof(double));
    if (J_sum) *J_sum = acc;
  } else if (J_steps) {
    memset(J_steps, 0, sizeof(double) * nsteps);
  }
  return LBM_OK;
}

int lbm_get_time(const lbm_handle* h, int* t) {
  if (!h || !t) return fail(nullptr, LBM_ERR_ARG, "null argument");
  *t = h->t;
  return LBM_OK;
}

int lbm_get_populations(const lbm_handle* hc, double* f) {
  lbm_handle* h = const_cast<lbm_handle*>(hc);
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!f) return fail(h, LBM_ERR_ARG, "null output");
  if (!h->have_state) return fail(h, LBM_ERR_STATE, "no state");
  int rc = ensure_stage(h);
  if (rc) return rc;
  KParams p = base_params(h, h->t);
  p.fin = h->f[h->cur];
  rc = launch(h, K_EXPORT, p, h->stage);
  if (rc) return rc;
  CUDA_OR_FAIL(h, cudaMemcpyAsync(f, h->stage, (size_t)h->ncell * h->Q * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int lbm_set_populations(lbm_handle* h, const double* f, int t) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!f) return fail(h, LBM_ERR_ARG, "null input");
  if (t < 0) return fail(h, LBM_ERR_ARG, "time step %d < 0", t);
  int rc = ensure_stage(h);
  if (rc) return rc;
  CUDA_OR_FAIL(h, cudaMemcpyAsync(h->stage, f, (size_t)h->ncell * h->Q * sizeof(double),
                                  cudaMemcpyHostToDevice, h->stream));
  KParams p = base_params(h, t);
  p.fout = h->f[h->cur];
  rc = launch(h, K_IMPORT, p, h->stage);
  if (rc) return rc;
  h->t = t;
  h->have_state = true;
  return sync(h);
}

int lbm_get_macros(const lbm_handle* hc, double* mac) {
  lbm_handle* h = const_cast<lbm_handle*>(hc);
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!mac) return fail(h, LBM_ERR_ARG, "null output");
  if (!h->have_state) return fail(h, LBM_ERR_STATE, "no state");
  int rc = ensure_stage(h);
  if (rc) return rc;
  KParams p = base_params(h, h->t);
  p.fin = h->f[h->cur];
  rc = launch(h, K_MACROS, p, h->stage);
  if (rc) return rc;
  CUDA_OR_FAIL(h, cudaMemcpyAsync(mac, h->stage, (size_t)h->ncell * h->nmac * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int lbm_adjoint_reset(lbm_handle* h) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  int rc = zero_adjoint(h);
  if (rc) return rc;
  h->have_adjoint = true;
  return sync(h);
}

int lbm_adjoint_step(lbm_handle* h) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!h->have_design || !h->have_state) return fail(h, LBM_ERR_STATE, "no design or state");
  if (!h->have_adjoint) return fail(h, LBM_ERR_STATE, "adjoint not reset (lbm_adjoint_reset)");
  int rc;
  if (h->cfg.objective == LBM_OBJ_REGENERATOR_EFFICIENCY && h->t >= h->obj_from) {
    // this step's share of the 1/D design term needs the step's objective
    if ((rc = ensure_jcap(h, 1))) return rc;
    if ((rc = objective_only(h, h->jdev))) return rc;
    if ((rc = add_design_term(h, h->jdev))) return rc;
  }
  rc = adjoint_step(h);
  if (rc) return rc;
  return sync(h);
}

int lbm_get_adjoint(const lbm_handle* hc, double* lam) {
  lbm_handle* h = const_cast<lbm_handle*>(hc);
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!lam) return fail(h, LBM_ERR_ARG, "null output");
  int rc = ensure_stage(h);
  if (rc) return rc;
  KParams p = base_params(h, h->t);
  p.lam_in = h->lam[h->lcur];
  rc = launch(h, K_EXPORT_ADJ, p, h->stage);
  if (rc) return rc;
  CUDA_OR_FAIL(h, cudaMemcpyAsync(lam, h->stage, (size_t)h->ncell * h->Q * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int lbm_get_sensitivity(const lbm_handle* hc, double* sens) {
  lbm_handle* h = const_cast<lbm_handle*>(hc);
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!sens) return fail(h, LBM_ERR_ARG, "null output");
  CUDA_OR_FAIL(h, cudaMemcpyAsync(sens, h->sens, (size_t)h->ncell * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int lbm_gradient(lbm_handle* h, int nsteps, int nsnap, double* J, double* dJdgamma,
                 lbm_gradient_stats* stats) {
  return lbm_gradient_schedule(h, nsteps, nsnap, LBM_SCHEDULE_DYNAMIC, J, dJdgamma, stats);
}

}  // extern "C"

namespace {

// The steady phase of a regenerator-style gradient: run until the largest
// one-step change of any population, measured every check_every steps, is
// below tol (or max_steps steps).
struct SteadyPhase {
  int max_steps, check_every;
  double tol;
  int steps = 0;        // taken
  double change = -1.;  // last measured
};

// The checkpointed forward sweep, reverse sweep and t = 0 term of
// lbm_gradient_schedule and lbm_gradient_steady.  With `sp`, a steady phase
// without objective comes first and nsteps objective steps follow it.
int gradient_run(lbm_handle* h, int nsteps, int nsnap, int schedule, SteadyPhase* sp, double* J,
                 double* dJdgamma, lbm_gradient_stats* stats) {
  int rc;
  // snapshot slots in device memory
  if ((int)h->slots.size() != nsnap) {
    for (void* s : h->slots)
      if (s) cudaFree(s);
    h->slots.assign(nsnap, nullptr);
    for (int i = 0; i < nsnap; ++i) {
      cudaError_t e = cudaMalloc(&h->slots[i], state_bytes(h));
      if (e != cudaSuccess) {
        for (void* s : h->slots)
          if (s) cudaFree(s);
        h->slots.clear();
        return fail(h, LBM_ERR_MEM, "%d snapshot slots of %zu bytes: %s", nsnap, state_bytes(h),
                    cudaGetErrorString(e));
      }
    }
  }
  if ((rc = ensure_jcap(h, (size_t)nsteps + 1))) return rc;
  const bool obj = h->cfg.objective != LBM_OBJ_NONE;
  const size_t sb = state_bytes(h);
  WangSchedule ws(nsnap);
  const bool planned = schedule == LBM_SCHEDULE_STATIC;
  if (planned) ws.plan_static(nsteps);
  auto place = [&](int index) { return planned ? ws.make_checkpoint_static(index) : ws.make_checkpoint(index); };
  // Checkpoints without copies: every state lives in one of the pool's K+2
  // buffers and saves/restores only move labels (StatePool).
  StatePool pool;
  pool.reset(nsnap, h->cur);
  auto cur_buf = [&]() { return pool_buffer(h, pool.current()); };
  auto advance = [&](double* result) -> int {
    const int out = pool.scratch();
    int r = forward_launch(h, cur_buf(), pool_buffer(h, out), result);
    if (!r) pool.set_current(out);
    return r;
  };
  auto save = [&](int slot) -> int {
    if (slot < 0) return 0;   // a state the static plan does not keep
    const int dst = pool.save(slot);
    if (dst >= 0)
      CUDA_OR_FAIL(h, cudaMemcpyAsync(pool_buffer(h, dst), cur_buf(), sb, cudaMemcpyDeviceToDevice,
                                      h->stream));
    return 0;
  };
  WangSchedule::Actions act;
  act.advance = [&]() { return advance(nullptr); };
  act.restore = [&](int step, int slot) -> int {
    pool.restore(slot);
    h->t = step;
    return 0;
  };
  act.save = save;

  h->t_phase = INT_MAX;   // a new run: ramps wait for the steady phase
  h->obj_from = 1;
  cudaEventRecord(h->ev[0], h->stream);
  {
    const int out = pool.scratch();
    if ((rc = init_into(h, pool_buffer(h, out)))) return rc;
    pool.set_current(out);
  }
  if ((rc = save(place(0)))) return rc;
  int steady = 0;
  if (sp) {
    // regenerator2d.cc:282-310: no objective; the states are checkpointed too
    // (the reverse sweep runs through them with an empty objective)
    unsigned long long* bits = (unsigned long long*)(h->jdev + nsteps);
    while (steady < sp->max_steps) {
      const int prev = pool.current();
      if ((rc = advance(nullptr))) return rc;
      ++steady;
      if ((rc = save(place(steady)))) return rc;
      if (steady % sp->check_every == 0 || steady == sp->max_steps) {
        // the step's input is still intact in its buffer (the next step writes later)
        if ((rc = measure_change(h, cur_buf(), pool_buffer(h, prev), h->t, bits, &sp->change)))
          return rc;
        if (!std::isfinite(sp->change))
          return fail(h, LBM_ERR_NONFINITE, "state is not finite at step %d", h->t);
        if (sp->change < sp->tol) break;
      }
    }
    sp->steps = steady;
    h->t_phase = steady;      // StageTemp: the ramp starts after the steady phase
    h->obj_from = steady + 1; // the objective counts the states after it
  }
  // J = sum_t F(f_t) over t = obj_from .. steady + nsteps, summed in the warp
  // partials across the sweep
  if (obj && (rc = begin_accumulate(h))) return rc;
  for (int s = steady; s < steady + nsteps; ++s) {
    if ((rc = advance((obj && s >= h->obj_from) ? h->jdev : nullptr))) break;
    if ((rc = save(place(s + 1)))) break;
  }
  if (!rc && obj && !(rc = objective_at(h, cur_buf(), h->jdev))) rc = end_accumulate(h, h->jdev);
  h->accumulate = false;
  if (rc) return rc;
  cudaEventRecord(h->ev[1], h->stream);
  if ((rc = zero_adjoint(h))) return rc;
  h->have_adjoint = true;
  const int total = steady + nsteps;
  for (int s = total; s >= 1; --s) {
    try {
      rc = ws.get_forward_solution(s, act);
    } catch (const std::exception& ex) {
      return fail(h, LBM_ERR_STATE, "checkpoint schedule: %s", ex.what());
    }
    if (rc) return rc;
    if ((rc = adjoint_at(h, cur_buf()))) return rc;
  }
  // The collision of f_0 depends on the design too; the reference's reverse loop stops
  // at step 1 (robustPump2d.cc:268-276).  Reverse it as well: no objective and no
  // boundary at t = 0.  The term is exactly zero for isothermal flows started at rest.
  // Every checkpoint has been consumed, so f_0 goes back into state buffer 0.
  h->cur = 0;
  if ((rc = init_state(h))) return rc;
  if ((rc = adjoint_step(h))) return rc;
  // the objective's design term shared by the box cells, from J
  if (obj && (rc = add_design_term(h, h->jdev))) return rc;
  cudaEventRecord(h->ev[2], h->stream);
  if ((rc = sync(h))) return rc;
  double acc = 0.;
  if (obj) {
    CUDA_OR_FAIL(h, cudaMemcpy(&acc, h->jdev, sizeof(double), cudaMemcpyDeviceToHost));
    if (!std::isfinite(acc)) return fail(h, LBM_ERR_NONFINITE, "objective is not finite");
  }
  if (J) *J = acc;
  if (dJdgamma) {
    CUDA_OR_FAIL(h, cudaMemcpy(dJdgamma, h->sens, (size_t)h->ncell * sizeof(double), cudaMemcpyDeviceToHost));
  }
  if (stats) {
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
    stats->forward_steps = total;
    stats->recomputed_steps = ws.recomputed();
    stats->adjoint_steps = total;
    stats->forward_ms = a;
    stats->reverse_ms = b;
  }
  return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_gradient_schedule(lbm_handle* h, int nsteps, int nsnap, int schedule, double* J,
                          double* dJdgamma, lbm_gradient_stats* stats) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (nsteps < 1) return fail(h, LBM_ERR_ARG, "nsteps %d < 1", nsteps);
  if (nsnap < 2) return fail(h, LBM_ERR_ARG, "nsnapshots %d < 2", nsnap);
  if (schedule != LBM_SCHEDULE_DYNAMIC && schedule != LBM_SCHEDULE_STATIC)
    return fail(h, LBM_ERR_ARG, "unknown checkpoint schedule %d", schedule);
  if (!h->have_design) return fail(h, LBM_ERR_STATE, "no design set (lbm_set_design)");
  return gradient_run(h, nsteps, nsnap, schedule, nullptr, J, dJdgamma, stats);
}

int lbm_gradient_steady(lbm_handle* h, int max_steady, int check_every, double tol,
                        int n_unsteady, int nsnap, int* steady_steps, double* J, double* dJdgamma,
                        lbm_gradient_stats* stats) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (max_steady < 1 || check_every < 1)
    return fail(h, LBM_ERR_ARG, "need max_steady >= 1 and check_every >= 1");
  if (!(tol >= 0.)) return fail(h, LBM_ERR_ARG, "tol must be >= 0");
  if (n_unsteady < 1) return fail(h, LBM_ERR_ARG, "n_unsteady %d < 1", n_unsteady);
  if (nsnap < 2) return fail(h, LBM_ERR_ARG, "nsnapshots %d < 2", nsnap);
  if (!h->have_design) return fail(h, LBM_ERR_STATE, "no design set (lbm_set_design)");
  SteadyPhase sp{max_steady, check_every, tol};
  int rc = gradient_run(h, n_unsteady, nsnap, LBM_SCHEDULE_DYNAMIC, &sp, J, dJdgamma, stats);
  if (steady_steps) *steady_steps = sp.steps;
  return rc;
}

int lbm_time_steps(lbm_handle* h, int which, int nsteps, float* ms) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!ms || nsteps < 1 || which < 0 || which > 2) return fail(h, LBM_ERR_ARG, "bad arguments");
  if (!h->have_design || !h->have_state) return fail(h, LBM_ERR_STATE, "no design or state");
  int rc;
  if (which >= 1 && !h->have_adjoint) {
    if ((rc = zero_adjoint(h))) return rc;
    h->have_adjoint = true;
  }
  int t_keep = h->t;
  if (which == 1 && h->t < 1) h->t = 1;
  cudaEventRecord(h->ev[0], h->stream);
  for (int k = 0; k < nsteps; ++k) {
    if (which == 0) {
      rc = forward_step(h, nullptr);
    } else if (which == 1) {
      rc = adjoint_step(h);
    } else {
      rc = forward_step(h, nullptr);
      if (!rc) rc = adjoint_step(h);
    }
    if (rc) return rc;
  }
  cudaEventRecord(h->ev[1], h->stream);
  if ((rc = sync(h))) return rc;
  if (which == 1) h->t = t_keep;
  cudaEventElapsedTime(ms, h->ev[0], h->ev[1]);
  return LBM_OK;
}

int lbm_autotune(lbm_handle* h, int nsteps) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (!h->have_design || !h->have_state) return fail(h, LBM_ERR_STATE, "no design or state");
  if (nsteps < 1) nsteps = 5;
  int rc;
  // keep the state: the trial steps run on a copy
  void* keep = nullptr;
  CUDA_OR_FAIL(h, cudaMalloc(&keep, state_bytes(h)));
  CUDA_OR_FAIL(h, cudaMemcpyAsync(keep, h->f[h->cur], state_bytes(h), cudaMemcpyDeviceToDevice, h->stream));
  const int t_keep = h->t, cur_keep = h->cur;
  if (!h->have_adjoint) {
    if ((rc = zero_adjoint(h))) { cudaFree(keep); return rc; }
    h->have_adjoint = true;
  }
  if (h->t < 1) h->t = 1;
  float best_f = 1e30f, best_a = 1e30f;
  Geometry bf = h->geo_fwd, ba = h->geo_adj;
  bool blean = h->adj_lean;
  const int nx = h->cfg.nx;
  const int nlean = h->cfg.storage == LBM_STORE_FP64 ? 1 : 2;   // FP64 has no lean variant
  // Forward steps are timed as a gradient's forward sweep runs them, with the
  // objective summed into the warp partials (scratch here; the next sweep
  // zeroes them): the shapes differ most in that reduction.
  const bool obj = h->cfg.objective != LBM_OBJ_NONE;
  if (obj && (rc = ensure_jcap(h, 1))) { cudaFree(keep); return rc; }
  double* jres = obj ? h->jdev : nullptr;
  for (const auto& sh : kShapes) {
    if (sh[0] > ((nx + 31) / 32) * 32 && sh[0] > 32) continue;
    Geometry g = make_geometry(nx, h->cfg.ny, h->cfg.nz, sh[0], sh[1]);
    for (int which = 0; which < 1 + nlean; ++which) {
      // which: 0 forward, 1 reverse, 2 reverse (lean variant)
      (which == 0 ? h->geo_fwd : h->geo_adj) = g;
      if (which >= 1) h->adj_lean = which == 2;
      h->accumulate = which == 0 && obj;
      // one untimed launch, then nsteps timed
      rc = which == 0 ? forward_step(h, jres) : adjoint_step(h);
      if (rc) { h->accumulate = false; cudaFree(keep); return rc; }
      cudaEventRecord(h->ev[0], h->stream);
      for (int k = 0; k < nsteps && !rc; ++k) rc = which == 0 ? forward_step(h, jres) : adjoint_step(h);
      cudaEventRecord(h->ev[1], h->stream);
      h->accumulate = false;
      if (rc || (rc = sync(h))) { cudaFree(keep); return rc; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
      if (which == 0 && ms < best_f) { best_f = ms; bf = g; }
      if (which >= 1 && ms < best_a) { best_a = ms; ba = g; blean = which == 2; }
    }
  }
  h->geo_fwd = bf;
  h->geo_adj = ba;
  h->adj_lean = blean;
  h->tuned = true;
  h->cur = cur_keep;
  h->t = t_keep;
  CUDA_OR_FAIL(h, cudaMemcpyAsync(h->f[h->cur], keep, state_bytes(h), cudaMemcpyDeviceToDevice, h->stream));
  rc = zero_adjoint(h);
  if (!rc) rc = sync(h);
  cudaFree(keep);
  return rc;
}

int lbm_set_launch_shape(lbm_handle* h, int which, int bx, int by) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (which < 0 || which > 1) return fail(h, LBM_ERR_ARG, "which must be 0 (forward) or 1 (reverse)");
  if (bx < 32 || bx % 32 != 0 || by < 1 || (bx * by != 64 && bx * by != 128 && bx * by != 256))
    return fail(h, LBM_ERR_ARG, "block %dx%d: bx must be a multiple of 32 and bx*by 64, 128 or 256", bx,
                by);
  Geometry g = make_geometry(h->cfg.nx, h->cfg.ny, h->cfg.nz, bx, by);
  if ((size_t)g.nblocks * (size_t)(bx * by / 32) > h->partial_cap)
    return fail(h, LBM_ERR_ARG, "block %dx%d gives too many blocks", bx, by);
  (which == 0 ? h->geo_fwd : h->geo_adj) = g;
  return LBM_OK;
}

int lbm_get_launch_shape(const lbm_handle* h, int which, int* bx, int* by) {
  if (!h || !bx || !by || which < 0 || which > 1) return fail(nullptr, LBM_ERR_ARG, "bad arguments");
  const Geometry& g = which == 0 ? h->geo_fwd : h->geo_adj;
  *bx = g.block.x;
  *by = g.block.y;
  return LBM_OK;
}

int lbm_set_reverse_variant(lbm_handle* h, int lean) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  if (lean != 0 && lean != 1) return fail(h, LBM_ERR_ARG, "variant %d is neither 0 nor 1", lean);
  if (lean && h->cfg.storage == LBM_STORE_FP64)
    return fail(h, LBM_ERR_SUP, "FP64 storage has no register-lean reverse variant");
  h->adj_lean = lean == 1;
  return LBM_OK;
}

int lbm_get_reverse_variant(const lbm_handle* h) {
  if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
  return h->adj_lean ? 1 : 0;
}

int lbm_select_device(int ordinal) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return fail(nullptr, LBM_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
  if (ordinal < 0 || ordinal >= n) return fail(nullptr, LBM_ERR_ARG, "device %d of %d", ordinal, n);
  e = cudaSetDevice(ordinal);
  if (e != cudaSuccess) return fail(nullptr, LBM_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  return LBM_OK;
}

int lbm_get_launch_count(const lbm_handle* h, int64_t* n) {
  if (!h || !n) return fail(nullptr, LBM_ERR_ARG, "null argument");
  *n = h->launches;
  return LBM_OK;
}

int lbm_wang_recompute_count(int nsteps, int nsnap, int64_t* recomputed) {
  return lbm_schedule_count(nsteps, nsnap, LBM_SCHEDULE_DYNAMIC, recomputed, nullptr);
}

int lbm_schedule_count(int nsteps, int nsnap, int schedule, int64_t* recomputed, int64_t* saved) {
  if (!recomputed || nsteps < 1 || nsnap < 2)
    return fail(nullptr, LBM_ERR_ARG, "need nsteps >= 1, nsnapshots >= 2");
  if (schedule != LBM_SCHEDULE_DYNAMIC && schedule != LBM_SCHEDULE_STATIC)
    return fail(nullptr, LBM_ERR_ARG, "unknown checkpoint schedule %d", schedule);
  WangSchedule ws(nsnap);
  const bool planned = schedule == LBM_SCHEDULE_STATIC;
  if (planned) ws.plan_static(nsteps);
  std::vector<int> slot_step(nsnap, -1);
  int state = 0;
  int64_t kept = 0;
  for (int s = 0; s <= nsteps; ++s) {
    const int slot = planned ? ws.make_checkpoint_static(s) : ws.make_checkpoint(s);
    if (slot >= 0) {
      slot_step[slot] = s;
      ++kept;
    }
  }
  if (saved) *saved = kept;
  WangSchedule::Actions act;
  act.advance = [&]() { ++state; return 0; };
  act.restore = [&](int step, int slot) {
    if (slot_step[slot] != step) return -1;
    state = step;
    return 0;
  };
  act.save = [&](int slot) { slot_step[slot] = state; return 0; };
  for (int s = nsteps; s >= 1; --s) {
    int rc = ws.get_forward_solution(s, act);
    if (rc || state != s) return fail(nullptr, LBM_ERR_STATE, "schedule did not reverse at step %d", s);
  }
  *recomputed = ws.recomputed();
  return LBM_OK;
}

}  // extern "C"

// ===========================================================================
// Batches: several lattices (uneven sizes, own boundaries, designs and
// objectives; same lattice type, collision and storage) advanced together, one
// launch per time step, with the whole checkpointed gradient optionally
// captured in a CUDA graph and replayed.  This is the one-GPU form of the
// reference's MPISplit ensembles (core/MPISplit.cc:14-59: one realisation per
// sub-communicator) plus uneven extra instances.

namespace {

struct CopyBatch {
  int n;
  const uint4* src[LBM_MAX_BATCH];
  uint4* dst[LBM_MAX_BATCH];
  long long nvec[LBM_MAX_BATCH];   // 16-byte vectors per buffer
};

// dst_i <- src_i for every buffer of the batch, 16 bytes per thread and step.
__global__ void __launch_bounds__(256) k_copy_batch(const __grid_constant__ CopyBatch cb) {
  for (int i = 0; i < cb.n; ++i) {
    const uint4* __restrict__ s = cb.src[i];
    uint4* __restrict__ d = cb.dst[i];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < cb.nvec[i];
         k += (long long)gridDim.x * blockDim.x)
      d[k] = s[k];
  }
}

}  // namespace

struct lbm_batch {
  int n = 0;
  lbm_handle* h[LBM_MAX_BATCH] = {};
  BatchOps ops;
  cudaStream_t stream = nullptr;
  int bx = 128, by = 2;     // block shape of the forward and objective kernels
  int abx = 128, aby = 2;   // block shape of the reverse step kernel
  bool adj_lean = false;    // reverse step: the register-lean variant
  bool sens_atomic = false; // the batched reverse step fits in L2 (see lbm_handle)
  int nsm = 1;
  int grid_fwd = 1, grid_adj = 1, grid_obj = 1, grid_copy = 1;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = -1, graph_snap = -1, graph_schedule = -1;
  int64_t graph_table_gen = -1;          // the lattices' table generations at capture
  int64_t graph_recomputed = 0;
  int64_t graph_launches = 0;            // kernels in the captured sequence
  int end_cur[LBM_MAX_BATCH] = {}, end_lcur[LBM_MAX_BATCH] = {};   // host state after it
  int64_t launches = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::string err;
};

namespace {

int bfail(lbm_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b)
    b->err = buf;
  else
    g_create_error = buf;
  return code;
}

#define BCUDA(b, call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return bfail((b), LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Persistent grid: resident blocks of kernel `kind` times SMs, at most the work.
// Block shape of a batched kernel: the reverse step has its own.
dim3 batch_block(const lbm_batch* b, int kind) {
  return (kind == K_ADJOINT || kind == K_ADJOINT_LEAN) ? dim3(b->abx, b->aby) : dim3(b->bx, b->by);
}

// Grid of a batched kernel over `total` virtual blocks.  The step kernels get
// one CTA per virtual block, as a single lattice's launch does, so that
// programmatic dependent launch can schedule the next step's CTAs into the
// previous step's last wave (a resident-CTA grid striding over the virtual
// blocks cannot: measured on the 8-channel D2Q9 batch, 43.2 / 64.9 us per
// forward / reverse step that way against 38.8 / 62.0 us with one CTA per
// virtual block).  The objective kernel keeps a grid of resident CTAs
// striding over the blocks.
int batch_grid(lbm_batch* b, int kind, int total) {
  if (kind == K_FORWARD || kind == K_ADJOINT || kind == K_ADJOINT_LEAN) return total;
  int per_sm = 1;
  const void* k = b->ops.kernel(kind);
  const dim3 blk = batch_block(b, kind);
  if (k) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, blk.x * blk.y, 0);
  if (per_sm < 1) per_sm = 1;
  int g = per_sm * b->nsm;
  return g < total ? g : total;
}

void batch_layout(lbm_batch* b, BatchParams& bp, int kind) {
  const dim3 blk = batch_block(b, kind);
  // rows of cells per virtual block
  const int rows = (int)blk.y * (kind == K_FORWARD                             ? kBatchRowsForward
                                 : (kind == K_ADJOINT || kind == K_ADJOINT_LEAN) ? kBatchRowsReverse
                                                                                 : 1);
  bp.n = b->n;
  int start = 0;
  for (int i = 0; i < b->n; ++i) {
    const lbm_handle* h = b->h[i];
    bp.gx[i] = (h->cfg.nx + (int)blk.x - 1) / (int)blk.x;
    bp.gy[i] = (h->cfg.ny + rows - 1) / rows;
    // multiply-high divisors (batch_div): the numerators stay below the
    // lattice's block count gx*gy*nz (for gx) and gy*nz (for gy)
    const uint64_t nblk = (uint64_t)bp.gx[i] * bp.gy[i] * h->cfg.nz;
    bp.gxm[i] = batch_div_magic((uint64_t)bp.gx[i], nblk);
    bp.gym[i] = batch_div_magic((uint64_t)bp.gy[i], nblk / (uint64_t)bp.gx[i]);
    bp.start[i] = start;
    start += bp.gx[i] * bp.gy[i] * h->cfg.nz;
  }
  // slots past the batch start at the total (the kernels count the starts
  // at or below a block)
  for (int i = b->n; i <= kMaxBatch; ++i) bp.start[i] = start;
}

// Persistent grids of the batched kernels for the current block shapes.
void batch_set_grids(lbm_batch* b) {
  BatchParams bp;
  batch_layout(b, bp, K_FORWARD);
  b->grid_fwd = batch_grid(b, K_FORWARD, bp.start[b->n]);
  batch_layout(b, bp, K_OBJECTIVE);
  b->grid_obj = batch_grid(b, K_OBJECTIVE, bp.start[b->n]);
  batch_layout(b, bp, K_ADJOINT);
  b->grid_adj = batch_grid(b, b->adj_lean ? K_ADJOINT_LEAN : K_ADJOINT, bp.start[b->n]);
}

int batch_launch(lbm_batch* b, int kind, const BatchParams& bp, int grid) {
  for (int i = 0; i < b->n; ++i) {
    const int k = bp.p[i].apply_bc ? missing_table(b->h[i]) : -1;
    if (k >= 0)
      return bfail(b, LBM_ERR_STATE, "lattice %d: boundary %d has LBM_PROFILE_TABLE but no table "
                   "(lbm_set_bc_profile)", i, k);
  }
  b->ops.launch(kind, dim3(grid), batch_block(b, kind), b->stream, bp);
  b->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "batched launch %d: %s", kind, cudaGetErrorString(e));
  return 0;
}

// Buffers are named by StatePool index, or per lattice as its current state
// buffer / its other state buffer.
constexpr int kCurState = -1, kOtherState = -2;

void* batch_buffer(lbm_handle* h, int b) {
  return b == kCurState ? h->f[h->cur] : b == kOtherState ? h->f[1 - h->cur] : pool_buffer(h, b);
}

// One forward step of every lattice from buffer `in` into buffer `out`;
// results[i] (may be null) gets F of lattice i.
int batch_forward_bufs(lbm_batch* b, int in, int out, double* const* results) {
  BatchParams bp;
  batch_layout(b, bp, K_FORWARD);
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    KParams& p = bp.p[i];
    p = base_params(h, h->t);
    p.fin = batch_buffer(h, in);
    p.fout = batch_buffer(h, out);
    p.eval_obj = (results && results[i] && h->cfg.objective != LBM_OBJ_NONE) ? 1 : 0;
    p.result = results ? results[i] : nullptr;
  }
  int rc = batch_launch(b, K_FORWARD, bp, b->grid_fwd);
  if (rc) return rc;
  for (int i = 0; i < b->n; ++i) b->h[i]->t += 1;
  return 0;
}

// One forward step of every lattice between its two state buffers.
int batch_forward(lbm_batch* b, double* const* results) {
  int rc = batch_forward_bufs(b, kCurState, kOtherState, results);
  if (rc) return rc;
  for (int i = 0; i < b->n; ++i) b->h[i]->cur ^= 1;
  return 0;
}

int batch_objective(lbm_batch* b, int buf, double* const* results) {
  BatchParams bp;
  batch_layout(b, bp, K_OBJECTIVE);
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    KParams& p = bp.p[i];
    p = base_params(h, h->t);
    p.fin = batch_buffer(h, buf);
    p.eval_obj = h->cfg.objective != LBM_OBJ_NONE ? 1 : 0;
    p.result = results[i];
  }
  return batch_launch(b, K_OBJECTIVE, bp, b->grid_obj);
}

int batch_adjoint(lbm_batch* b, int buf) {
  BatchParams bp;
  batch_layout(b, bp, K_ADJOINT);
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    KParams& p = bp.p[i];
    p = base_params(h, h->t);
    p.fin = batch_buffer(h, buf);
    p.lam_in = h->lam[h->lcur];
    p.lam_out = h->lam[1 - h->lcur];
    p.eval_obj = (h->t >= 1 && h->cfg.objective != LBM_OBJ_NONE) ? 1 : 0;
    p.sens_atomic = b->sens_atomic ? 1 : 0;
  }
  int rc = batch_launch(b, b->adj_lean ? K_ADJOINT_LEAN : K_ADJOINT, bp, b->grid_adj);
  if (rc) return rc;
  for (int i = 0; i < b->n; ++i) b->h[i]->lcur ^= 1;
  return 0;
}

// dst <- src for every lattice (pool-buffer indices), one launch
int batch_copy(lbm_batch* b, int src, int dst) {
  CopyBatch cb;
  cb.n = b->n;
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    cb.src[i] = (const uint4*)batch_buffer(h, src);
    cb.dst[i] = (uint4*)batch_buffer(h, dst);
    cb.nvec[i] = (long long)(state_bytes(h) / 16);
  }
  k_copy_batch<<<b->grid_copy, 256, 0, b->stream>>>(cb);
  b->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "batched copy: %s", cudaGetErrorString(e));
  return 0;
}

int batch_init(lbm_batch* b, int buf) {
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    KParams p = base_params(h, 0);
    p.fout = batch_buffer(h, buf);
    h->launch(K_INIT, h->geo.grid, h->geo.block, b->stream, p, h->init_mac);
    b->launches++;
    h->t = 0;
    h->have_state = true;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "init: %s", cudaGetErrorString(e));
  return 0;
}

// The checkpointed forward + reverse sequence of lbm_batch_gradient, issued on
// the batch stream (and so capturable as one graph).  All lattices follow one
// schedule, so one StatePool labels the buffers of every lattice alike.
int batch_sequence(lbm_batch* b, int nsteps, int nsnap, int schedule, int64_t* recomputed) {
  int rc;
  for (int i = 0; i < b->n; ++i) {
    b->h[i]->cur = 0;
    b->h[i]->lcur = 0;
  }
  WangSchedule ws(nsnap);
  const bool planned = schedule == LBM_SCHEDULE_STATIC;
  if (planned) ws.plan_static(nsteps);
  auto place = [&](int index) { return planned ? ws.make_checkpoint_static(index) : ws.make_checkpoint(index); };
  StatePool pool;
  pool.reset(nsnap, 0);
  double* res[LBM_MAX_BATCH];
  auto advance = [&](double* const* results) -> int {
    const int out = pool.scratch();
    int r = batch_forward_bufs(b, pool.current(), out, results);
    if (!r) pool.set_current(out);
    return r;
  };
  auto save = [&](int slot) -> int {
    if (slot < 0) return 0;   // a state the static plan does not keep
    const int dst = pool.save(slot);
    return dst >= 0 ? batch_copy(b, pool.current(), dst) : 0;
  };
  {
    const int out = pool.scratch();
    if ((rc = batch_init(b, out))) return rc;
    pool.set_current(out);
  }
  // J of every lattice summed in its warp partials across the sweep
  for (int i = 0; i < b->n; ++i)
    if (b->h[i]->cfg.objective != LBM_OBJ_NONE && (rc = begin_accumulate(b->h[i], b->stream)))
      return bfail(b, rc, "%s", b->h[i]->err.c_str());
  auto stop_accumulating = [&]() {
    for (int i = 0; i < b->n; ++i) b->h[i]->accumulate = false;
  };
  if ((rc = save(place(0)))) {
    stop_accumulating();
    return rc;
  }
  for (int s = 0; s < nsteps; ++s) {
    for (int i = 0; i < b->n; ++i) res[i] = s >= 1 ? b->h[i]->jdev : nullptr;
    if ((rc = advance(res)) || (rc = save(place(s + 1)))) {
      stop_accumulating();
      return rc;
    }
  }
  for (int i = 0; i < b->n; ++i) res[i] = b->h[i]->jdev;
  rc = batch_objective(b, pool.current(), res);
  for (int i = 0; i < b->n && !rc; ++i)
    if (b->h[i]->cfg.objective != LBM_OBJ_NONE &&
        (rc = end_accumulate(b->h[i], b->h[i]->jdev, b->stream)))
      rc = bfail(b, rc, "%s", b->h[i]->err.c_str());
  stop_accumulating();
  if (rc) return rc;
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    for (void* p : h->lam) BCUDA(b, cudaMemsetAsync(p, 0, adjoint_bytes(h), b->stream));
    BCUDA(b, cudaMemsetAsync(h->sens, 0, (size_t)h->ncell * sizeof(double), b->stream));
    h->lcur = 0;
    h->have_adjoint = true;
  }
  WangSchedule::Actions act;
  act.advance = [&]() { return advance(nullptr); };
  act.restore = [&](int step, int slot) -> int {
    for (int i = 0; i < b->n; ++i) b->h[i]->t = step;
    pool.restore(slot);
    return 0;
  };
  act.save = save;
  for (int s = nsteps; s >= 1; --s) {
    try {
      rc = ws.get_forward_solution(s, act);
    } catch (const std::exception& ex) {
      return bfail(b, LBM_ERR_STATE, "checkpoint schedule: %s", ex.what());
    }
    if (rc) return rc;
    if ((rc = batch_adjoint(b, pool.current()))) return rc;
  }
  // reverse of the collision of f_0 (see lbm_gradient), from state buffer 0
  if ((rc = batch_init(b, 0))) return rc;
  if ((rc = batch_adjoint(b, 0))) return rc;
  *recomputed = ws.recomputed();
  return 0;
}

void batch_destroy_graph(lbm_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_steps = b->graph_snap = b->graph_schedule = -1;
  b->graph_table_gen = -1;
}

}  // namespace

extern "C" {

int lbm_batch_create(const lbm_config* cfgs, int n, lbm_batch** out) {
  if (!cfgs || !out) return bfail(nullptr, LBM_ERR_ARG, "null argument");
  *out = nullptr;
  if (n < 1 || n > LBM_MAX_BATCH) return bfail(nullptr, LBM_ERR_ARG, "batch of %d lattices outside [1,%d]", n, LBM_MAX_BATCH);
  for (int i = 1; i < n; ++i)
    if (cfgs[i].lattice != cfgs[0].lattice || cfgs[i].collision != cfgs[0].collision ||
        cfgs[i].storage != cfgs[0].storage)
      return bfail(nullptr, LBM_ERR_SUP, "batched lattices must share lattice, collision and storage");
  for (int i = 0; i < n; ++i)
    if (cfgs[i].objective == LBM_OBJ_REGENERATOR_EFFICIENCY)
      return bfail(nullptr, LBM_ERR_SUP,
                   "lattice %d: the regenerator efficiency runs on single handles only", i);
  lbm_batch* b = new (std::nothrow) lbm_batch();
  if (!b) return bfail(nullptr, LBM_ERR_MEM, "host allocation failed");
  for (int i = 0; i < n; ++i) {
    int rc = lbm_create(&cfgs[i], &b->h[i]);
    if (rc) {
      std::string msg = g_create_error;
      for (int j = 0; j < i; ++j) lbm_destroy(b->h[j]);
      delete b;
      return bfail(nullptr, rc, "lattice %d: %s", i, msg.c_str());
    }
    b->n = i + 1;
  }
  const lbm_config& c = cfgs[0];
  b->ops = c.lattice == LBM_D2Q9    ? batch_ops_d2q9(c.collision, c.storage)
           : c.lattice == LBM_D3Q19 ? batch_ops_d3q19(c.collision, c.storage)
                                    : batch_ops_thermal(c.collision, c.storage);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
  if (b->nsm < 1) b->nsm = 1;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess || !b->ops.launch) {
    for (int i = 0; i < b->n; ++i) lbm_destroy(b->h[i]);
    delete b;
    return bfail(nullptr, LBM_ERR_CUDA, "batch set-up failed");
  }
  for (cudaEvent_t& ev : b->ev) {
    if (cudaEventCreate(&ev) != cudaSuccess) {
      ev = nullptr;
      lbm_batch_destroy(b);
      return bfail(nullptr, LBM_ERR_CUDA, "batch set-up failed: cudaEventCreate");
    }
  }
  // default shapes: 128x2, one of the autotuner's shapes (partial sums are sized for all)
  b->bx = b->abx = 128;
  b->by = b->aby = 2;
  batch_set_grids(b);
  b->grid_copy = 4 * b->nsm;
  size_t rev = 0;
  for (int i = 0; i < b->n; ++i) rev += reverse_step_bytes(b->h[i]);
  b->sens_atomic = fits_in_l2(rev);
  *out = b;
  return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* b) {
  if (!b) return LBM_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_destroy_graph(b);
  for (int i = 0; i < b->n; ++i) lbm_destroy(b->h[i]);
  for (cudaEvent_t e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return LBM_OK;
}

const char* lbm_batch_last_error(const lbm_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

int lbm_batch_handle(lbm_batch* b, int i, lbm_handle** h) {
  if (!b || !h || i < 0 || i >= b->n) return bfail(b, LBM_ERR_ARG, "lattice index %d", i);
  *h = b->h[i];
  return LBM_OK;
}

int lbm_batch_autotune(lbm_batch* b, int nsteps) {
  if (!b) return bfail(nullptr, LBM_ERR_ARG, "null batch");
  for (int i = 0; i < b->n; ++i)
    if (!b->h[i]->have_design) return bfail(b, LBM_ERR_STATE, "lattice %d has no design", i);
  if (nsteps < 1) nsteps = 3;
  batch_destroy_graph(b);
  int rc;
  if ((rc = batch_init(b, kCurState))) return rc;
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    for (void* p : h->lam) BCUDA(b, cudaMemsetAsync(p, 0, adjoint_bytes(h), b->stream));
    h->have_adjoint = true;
    h->t = 1;
  }
  // each kernel on its own: every shape for the forward step, then every
  // shape and both register variants for the reverse step
  float best_f = 1e30f, best_a = 1e30f;
  int fbx = b->bx, fby = b->by, abx = b->abx, aby = b->aby;
  bool alean = b->adj_lean;
  const int nlean = b->h[0]->cfg.storage == LBM_STORE_FP64 ? 1 : 2;
  // forward steps timed with the objectives summed into the warp partials, as
  // a gradient's forward sweep runs them (the partials are scratch here)
  double* res[LBM_MAX_BATCH] = {};
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    if (h->cfg.objective == LBM_OBJ_NONE) continue;
    if ((rc = ensure_jcap(h, 1))) return bfail(b, rc, "%s", h->err.c_str());
    res[i] = h->jdev;
  }
  auto accumulate_all = [&](bool on) {
    for (int i = 0; i < b->n; ++i) b->h[i]->accumulate = on && res[i] != nullptr;
  };
  for (int which = 0; which < 1 + nlean; ++which) {
    for (const auto& sh : kShapes) {
      if (which == 0) {
        b->bx = sh[0];
        b->by = sh[1];
      } else {
        b->abx = sh[0];
        b->aby = sh[1];
        b->adj_lean = which == 2;
      }
      batch_set_grids(b);
      accumulate_all(which == 0);
      rc = which == 0 ? batch_forward(b, res) : batch_adjoint(b, kCurState);
      if (rc) {
        accumulate_all(false);
        return rc;
      }
      cudaEventRecord(b->ev[0], b->stream);
      for (int k = 0; k < nsteps && !rc; ++k)
        rc = which == 0 ? batch_forward(b, res) : batch_adjoint(b, kCurState);
      cudaEventRecord(b->ev[1], b->stream);
      accumulate_all(false);
      if (rc) return rc;
      BCUDA(b, cudaStreamSynchronize(b->stream));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
      if (which == 0 && ms < best_f) {
        best_f = ms;
        fbx = sh[0];
        fby = sh[1];
      }
      if (which >= 1 && ms < best_a) {
        best_a = ms;
        abx = sh[0];
        aby = sh[1];
        alean = which == 2;
      }
    }
    if (which == 0) {
      b->bx = fbx;
      b->by = fby;
    }
  }
  b->adj_lean = alean;
  b->abx = abx;
  b->aby = aby;
  batch_set_grids(b);
  if ((rc = batch_init(b, kCurState))) return rc;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

int lbm_batch_get_launch_shape(const lbm_batch* b, int* bx, int* by) {
  if (!b || !bx || !by) return bfail(nullptr, LBM_ERR_ARG, "null argument");
  *bx = b->bx;
  *by = b->by;
  return LBM_OK;
}

int lbm_batch_get_reverse_shape(const lbm_batch* b, int* bx, int* by) {
  if (!b || !bx || !by) return bfail(nullptr, LBM_ERR_ARG, "null argument");
  *bx = b->abx;
  *by = b->aby;
  return LBM_OK;
}

int lbm_batch_set_reverse_variant(lbm_batch* b, int lean) {
  if (!b) return bfail(nullptr, LBM_ERR_ARG, "null batch");
  if (lean != 0 && lean != 1) return bfail(b, LBM_ERR_ARG, "variant %d is neither 0 nor 1", lean);
  if (lean && b->h[0]->cfg.storage == LBM_STORE_FP64)
    return bfail(b, LBM_ERR_SUP, "FP64 storage has no register-lean reverse variant");
  batch_destroy_graph(b);
  b->adj_lean = lean == 1;
  batch_set_grids(b);
  return LBM_OK;
}

int lbm_batch_set_launch_shape(lbm_batch* b, int which, int bx, int by) {
  if (!b) return bfail(nullptr, LBM_ERR_ARG, "null batch");
  if (which < 0 || which > 1) return bfail(b, LBM_ERR_ARG, "which must be 0 (forward) or 1 (reverse)");
  // the per-warp partial sums of every lattice are sized for the tuner's shapes
  bool known = false;
  for (const auto& sh : kShapes) known = known || (sh[0] == bx && sh[1] == by);
  if (!known) return bfail(b, LBM_ERR_ARG, "block %dx%d is not one of the tuner's shapes", bx, by);
  batch_destroy_graph(b);
  if (which == 0) {
    b->bx = bx;
    b->by = by;
  } else {
    b->abx = bx;
    b->aby = by;
  }
  batch_set_grids(b);
  return LBM_OK;
}

int lbm_batch_get_reverse_variant(const lbm_batch* b) {
  if (!b) return bfail(nullptr, LBM_ERR_ARG, "null batch");
  return b->adj_lean ? 1 : 0;
}

int lbm_batch_forward(lbm_batch* b, int nsteps, double* J) {
  if (!b) return bfail(nullptr, LBM_ERR_ARG, "null batch");
  if (nsteps < 1) return bfail(b, LBM_ERR_ARG, "nsteps %d < 1", nsteps);
  for (int i = 0; i < b->n; ++i) {
    if (!b->h[i]->have_design || !b->h[i]->have_state)
      return bfail(b, LBM_ERR_STATE, "lattice %d has no design or state", i);
    if (ensure_jcap(b->h[i], (size_t)nsteps)) return bfail(b, LBM_ERR_MEM, "%s", b->h[i]->err.c_str());
  }
  int rc;
  double* res[LBM_MAX_BATCH];
  for (int s = 0; s < nsteps; ++s) {
    for (int i = 0; i < b->n; ++i) res[i] = s >= 1 ? b->h[i]->jdev + (s - 1) : nullptr;
    if ((rc = batch_forward(b, res))) return rc;
  }
  for (int i = 0; i < b->n; ++i) res[i] = b->h[i]->jdev + (nsteps - 1);
  if ((rc = batch_objective(b, kCurState, res))) return rc;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  if (J) {
    std::vector<double> js((size_t)nsteps);
    for (int i = 0; i < b->n; ++i) {
      BCUDA(b, cudaMemcpy(js.data(), b->h[i]->jdev, js.size() * sizeof(double), cudaMemcpyDeviceToHost));
      double acc = 0.;
      for (double v : js) acc += v;
      J[i] = acc;
    }
  }
  return LBM_OK;
}

int lbm_batch_gradient(lbm_batch* b, int nsteps, int nsnap, int use_graph, double* J,
                       double* const* dJdgamma, lbm_gradient_stats* stats) {
  return lbm_batch_gradient_schedule(b, nsteps, nsnap, LBM_SCHEDULE_DYNAMIC, use_graph, J,
                                     dJdgamma, stats);
}

int lbm_batch_gradient_schedule(lbm_batch* b, int nsteps, int nsnap, int schedule, int use_graph,
                                double* J, double* const* dJdgamma, lbm_gradient_stats* stats) {
  if (!b) return bfail(nullptr, LBM_ERR_ARG, "null batch");
  if (nsteps < 1 || nsnap < 2) return bfail(b, LBM_ERR_ARG, "need nsteps >= 1 and nsnapshots >= 2");
  if (schedule != LBM_SCHEDULE_DYNAMIC && schedule != LBM_SCHEDULE_STATIC)
    return bfail(b, LBM_ERR_ARG, "unknown checkpoint schedule %d", schedule);
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    if (!h->have_design) return bfail(b, LBM_ERR_STATE, "lattice %d has no design", i);
    if (ensure_jcap(h, (size_t)nsteps)) return bfail(b, LBM_ERR_MEM, "%s", h->err.c_str());
    if ((int)h->slots.size() != nsnap) {
      batch_destroy_graph(b);
      for (void* s : h->slots)
        if (s) cudaFree(s);
      h->slots.assign(nsnap, nullptr);
      for (int k = 0; k < nsnap; ++k) {
        if (cudaMalloc(&h->slots[k], state_bytes(h)) != cudaSuccess) {
          for (void* s : h->slots)
            if (s) cudaFree(s);
          h->slots.clear();
          return bfail(b, LBM_ERR_MEM, "lattice %d: %d snapshot slots", i, nsnap);
        }
      }
    }
  }
  int rc;
  int64_t recomputed = 0;
  cudaEventRecord(b->ev[0], b->stream);
  if (use_graph) {
    int64_t table_gen = 0;
    for (int i = 0; i < b->n; ++i) table_gen += b->h[i]->table_gen;
    if (!(b->graph && b->graph_steps == nsteps && b->graph_snap == nsnap &&
          b->graph_schedule == schedule && b->graph_table_gen == table_gen)) {
      batch_destroy_graph(b);
      cudaGraph_t g = nullptr;
      const int64_t l0 = b->launches;
      BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      rc = batch_sequence(b, nsteps, nsnap, schedule, &recomputed);
      b->graph_launches = b->launches - l0;
      cudaError_t e = cudaStreamEndCapture(b->stream, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (e != cudaSuccess) return bfail(b, LBM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        b->graph = nullptr;
        return bfail(b, LBM_ERR_CUDA, "graph instantiation: %s", cudaGetErrorString(e));
      }
      b->graph_steps = nsteps;
      b->graph_snap = nsnap;
      b->graph_schedule = schedule;
      b->graph_table_gen = table_gen;
      b->graph_recomputed = recomputed;
      for (int i = 0; i < b->n; ++i) {
        b->end_cur[i] = b->h[i]->cur;
        b->end_lcur[i] = b->h[i]->lcur;
      }
      b->launches -= b->graph_launches;   // counted again below, per replay
      cudaEventRecord(b->ev[0], b->stream);
    } else {
      recomputed = b->graph_recomputed;
    }
    BCUDA(b, cudaGraphLaunch(b->graph, b->stream));
    b->launches += b->graph_launches;
    // the replayed sequence starts from f_0 in buffer 0 whatever the handles held
    // before, and leaves them as the captured sequence did
    for (int i = 0; i < b->n; ++i) {
      lbm_handle* h = b->h[i];
      h->cur = b->end_cur[i];
      h->lcur = b->end_lcur[i];
      h->t = 0;
      h->have_state = h->have_adjoint = true;
    }
  } else {
    if ((rc = batch_sequence(b, nsteps, nsnap, schedule, &recomputed))) return rc;
  }
  cudaEventRecord(b->ev[1], b->stream);
  BCUDA(b, cudaStreamSynchronize(b->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    if (J) {
      double acc = 0.;
      if (h->cfg.objective != LBM_OBJ_NONE)
        BCUDA(b, cudaMemcpy(&acc, h->jdev, sizeof(double), cudaMemcpyDeviceToHost));
      if (!std::isfinite(acc)) return bfail(b, LBM_ERR_NONFINITE, "lattice %d: objective not finite", i);
      J[i] = acc;
    }
    if (dJdgamma && dJdgamma[i])
      BCUDA(b, cudaMemcpy(dJdgamma[i], h->sens, (size_t)h->ncell * sizeof(double), cudaMemcpyDeviceToHost));
  }
  if (stats) {
    stats->forward_steps = nsteps;
    stats->recomputed_steps = recomputed;
    stats->adjoint_steps = nsteps;
    stats->forward_ms = ms;   // whole sequence (one graph launch when use_graph)
    stats->reverse_ms = 0.;
  }
  return LBM_OK;
}

int lbm_batch_time_steps(lbm_batch* b, int which, int nsteps, float* ms) {
  if (!b || !ms || nsteps < 1 || which < 0 || which > 2) return bfail(b, LBM_ERR_ARG, "bad arguments");
  for (int i = 0; i < b->n; ++i)
    if (!b->h[i]->have_design || !b->h[i]->have_state)
      return bfail(b, LBM_ERR_STATE, "lattice %d has no design or state", i);
  int rc;
  for (int i = 0; i < b->n; ++i) {
    lbm_handle* h = b->h[i];
    if (which >= 1 && !h->have_adjoint) {
      for (void* p : h->lam) BCUDA(b, cudaMemsetAsync(p, 0, adjoint_bytes(h), b->stream));
      h->have_adjoint = true;
    }
    if (which >= 1 && h->t < 1) h->t = 1;
  }
  cudaEventRecord(b->ev[0], b->stream);
  for (int k = 0; k < nsteps; ++k) {
    if (which != 1 && (rc = batch_forward(b, nullptr))) return rc;
    if (which != 0 && (rc = batch_adjoint(b, kCurState))) return rc;
  }
  cudaEventRecord(b->ev[1], b->stream);
  BCUDA(b, cudaStreamSynchronize(b->stream));
  cudaEventElapsedTime(ms, b->ev[0], b->ev[1]);
  return LBM_OK;
}

int lbm_batch_get_launch_count(const lbm_batch* b, int64_t* n) {
  if (!b || !n) return bfail(nullptr, LBM_ERR_ARG, "null argument");
  *n = b->launches;
  return LBM_OK;
}

}  // extern "C"
