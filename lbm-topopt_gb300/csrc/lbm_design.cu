// lbm_design.cu -- the design update of the optimisation loop on the device:
// design box <-> full field, density filter + tanh projection stages and
// their transposes, volume constraint, and MMA, all in FP64.
//
// Reference behaviour followed (each restated, none compiled in):
//   box mapping       topOpt/fullToDesignMapping2d.cc (design box cells <-> full grid)
//   density filter    topOpt/densityFilter2d.cc:33-146, densityFilter3d.cc:60-139:
//                     rows of the filter box carry the cone weights R - |d| of their
//                     neighbours inside the grid, other rows are identity rows;
//                     filter = H x / rowsum(H), sensitivities H^T (s / rowsum(H))
//   projection        topOpt/projectionFilter2d.cc:27-88 (on the filter box only)
//   two stages        topOpt/doubleProjectionFilter2d.cc
//   volume            functionals/volumeConstraint.cc
//   MMA               Svanberg (1987), with the subproblem of topOpt/MMA.cc (GenSub):
//                     asymptotes 0.5/0.7/1.2 clamped to [0.01, 10] x range, bounds
//                     0.9 L + 0.1 x / 0.9 U + 0.1 x, p/q with 0.001|df| + 0.5e-6/(U-L)
//                     for the objective, plain for the constraints, y and z penalties
//                     c = 1000 (c y + y^2/2) and z + z^2/20, outer move limit in [0,1].
//                     Its dual (m <= 9 multipliers) is solved by a primal-dual Newton
//                     method with a barrier reduced tenfold down to 1e-9 sqrt(n + m):
//                     every dual evaluation is one pass over the n variables on the
//                     device with a fixed-order reduction, the m x m Newton step runs
//                     on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_ops.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxM = LBM_MAX_REALISATIONS + 1;                 // MMA constraints
constexpr int kMaxVals = kMaxM + kMaxM * (kMaxM + 1) / 2;      // dual gradient + upper Hessian
constexpr int kMaxBlocks = 1024;

struct Grid {
  int nx, ny, nz;
  long long n;
};

// One filter stage as the kernels see it.
struct StageDev {
  int project, ntaps;
  int box[6];
  double beta, eta, pden;   // pden = tanh(beta eta) + tanh(beta (1 - eta))
  const int* tap;           // ntaps x (dx, dy, dz), dz then dy then dx ascending
  const double* w;          // weights R - |d| > 0
  const double* den;        // row sums of the filter matrix (1 outside the box)
};

__device__ __forceinline__ bool in_box(const int* b, int x, int y, int z) {
  return x >= b[0] && x <= b[1] && y >= b[2] && y <= b[3] && z >= b[4] && z <= b[5];
}

__device__ __forceinline__ void cell_xyz(const Grid& g, long long c, int& x, int& y, int& z) {
  x = (int)(c % g.nx);
  long long r = c / g.nx;
  y = (int)(r % g.ny);
  z = (int)(r / g.ny);
}

__global__ void k_den(Grid g, StageDev s, double* den) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    if (!in_box(s.box, x, y, z)) {
      den[c] = 1.;
      continue;
    }
    double acc = 0.;
    for (int k = 0; k < s.ntaps; ++k) {
      const int xx = x + s.tap[3 * k], yy = y + s.tap[3 * k + 1], zz = z + s.tap[3 * k + 2];
      if (xx < 0 || yy < 0 || zz < 0 || xx >= g.nx || yy >= g.ny || zz >= g.nz) continue;
      acc += s.w[k];
    }
    den[c] = acc;
  }
}

// xfull = background, with the design variables on the box
__global__ void k_scatter_box(Grid g, const int* __restrict__ b, const double* __restrict__ x,
                              const double* __restrict__ bg, double* __restrict__ xfull) {
  const int nxb = b[1] - b[0] + 1, nyb = b[3] - b[2] + 1;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int cx, cy, cz;
    cell_xyz(g, c, cx, cy, cz);
    if (in_box(b, cx, cy, cz))
      xfull[c] = x[((long long)(cz - b[4]) * nyb + (cy - b[2])) * nxb + (cx - b[0])];
    else
      xfull[c] = bg[c];
  }
}

// out[i] = full[cell of design variable i]
__global__ void k_gather_box(Grid g, const int* __restrict__ b, long long n,
                             const double* __restrict__ full, double* __restrict__ out) {
  const int nxb = b[1] - b[0] + 1, nyb = b[3] - b[2] + 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nxb) + b[0];
    const long long r = i / nxb;
    const int y = (int)(r % nyb) + b[2];
    const int z = (int)(r / nyb) + b[4];
    out[i] = full[((long long)z * g.ny + y) * g.nx + x];
  }
}

__global__ void k_stage_forward(Grid g, StageDev s, const double* __restrict__ in,
                                double* __restrict__ keep, double* __restrict__ out) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    const bool ib = in_box(s.box, x, y, z);
    double v;
    if (!ib) {
      v = in[c];
    } else {
      double acc = 0.;
      for (int k = 0; k < s.ntaps; ++k) {
        const int xx = x + s.tap[3 * k], yy = y + s.tap[3 * k + 1], zz = z + s.tap[3 * k + 2];
        if (xx < 0 || yy < 0 || zz < 0 || xx >= g.nx || yy >= g.ny || zz >= g.nz) continue;
        acc += s.w[k] * in[((long long)zz * g.ny + yy) * g.nx + xx];
      }
      v = acc / s.den[c];
    }
    keep[c] = v;
    if (s.project && ib) v = (tanh(s.beta * s.eta) + tanh(s.beta * (v - s.eta))) / s.pden;
    out[c] = v;
  }
}

// t = (projection derivative at keep) * s / rowsum
__global__ void k_stage_scale(Grid g, StageDev s, const double* __restrict__ keep,
                              const double* __restrict__ sin, double* __restrict__ t) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    double v = sin[c];
    if (s.project && in_box(s.box, x, y, z)) {
      const double th = tanh(s.beta * (keep[c] - s.eta));
      v *= (1. - th * th) * s.beta / s.pden;
    }
    t[c] = v / s.den[c];
  }
}

// sout = H^T t: column c gathers the filter rows that hold it (the cone is symmetric)
__global__ void k_stage_transpose(Grid g, StageDev s, const double* __restrict__ t,
                                  double* __restrict__ sout) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    double acc = in_box(s.box, x, y, z) ? 0. : t[c];
    for (int k = 0; k < s.ntaps; ++k) {
      const int xx = x + s.tap[3 * k], yy = y + s.tap[3 * k + 1], zz = z + s.tap[3 * k + 2];
      if (xx < 0 || yy < 0 || zz < 0 || xx >= g.nx || yy >= g.ny || zz >= g.nz) continue;
      if (!in_box(s.box, xx, yy, zz)) continue;
      acc += s.w[k] * t[((long long)zz * g.ny + yy) * g.nx + xx];
    }
    sout[c] = acc;
  }
}

__global__ void k_fill(double* v, long long n, double a) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = a;
}

// ---------------------------------------------------------------------------
// Fixed-order reductions: every thread accumulates its own elements in index
// order, warps and blocks combine in a fixed order, a last single-block pass
// adds the block partials in order.  Results do not depend on timing.

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// part[blockIdx.x * nv + k] = block sum of v[k] (max when use_max)
__device__ void block_store(double* v, int nv, double* part, bool use_max) {
  __shared__ double sh[kThreads / 32][kMaxVals];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < nv; ++k) {
    const double r = use_max ? warp_max_d(v[k]) : warp_sum_d(v[k]);
    if (lane == 0) sh[wid][k] = r;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double acc = sh[0][threadIdx.x];
    for (int w = 1; w < (int)(blockDim.x / 32); ++w)
      acc = use_max ? fmax(acc, sh[w][threadIdx.x]) : acc + sh[w][threadIdx.x];
    part[blockIdx.x * nv + threadIdx.x] = acc;
  }
}

__global__ void k_finish(const double* __restrict__ part, int nblk, int nv, double* __restrict__ out,
                         int use_max) {
  for (int k = threadIdx.x; k < nv; k += blockDim.x) {
    double acc = part[k];
    for (int b = 1; b < nblk; ++b) acc = use_max ? fmax(acc, part[b * nv + k]) : acc + part[b * nv + k];
    out[k] = acc;
  }
}

__global__ void k_sum(const double* __restrict__ v, long long n, double* part) {
  double acc[1] = {0.};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    acc[0] += v[i];
  block_store(acc, 1, part, false);
}

__global__ void k_max_abs_diff(const double* __restrict__ a, const double* __restrict__ b,
                               long long n, double* part) {
  double acc[1] = {0.};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    acc[0] = fmax(acc[0], fabs(a[i] - b[i]));
  block_store(acc, 1, part, true);
}

// ---------------------------------------------------------------------------
// MMA on the device.

struct MmaDev {
  long long n;
  int m;
  double *x, *x1, *x2, *L, *U, *al, *be, *p0, *q0, *P, *Q;   // P, Q: m x n
  const double* df0;
  const double* dg;                                           // m x n
};

struct MmaScalars {
  int k;
  double asyminit, asymdec, asyminc, movlim;
  double lam[kMaxM];
  int hess;
};

// Subproblem at the expansion point x (GenSub), the history shift, and the
// block sums of sum_i (P_ji/(U-x) + Q_ji/(x-L)) for b_j.
__global__ void k_mma_gensub(MmaDev d, MmaScalars s, double* part) {
  const double feps = 1.0e-6;
  double acc[kMaxM];
  for (int j = 0; j < d.m; ++j) acc[j] = 0.;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.n;
       i += (long long)gridDim.x * blockDim.x) {
    const double x = d.x[i], x1 = d.x1[i], x2 = d.x2[i];
    const double xmin = fmax(0., x - s.movlim), xmax = fmin(1., x + s.movlim);
    double L, U;
    if (s.k < 3) {
      L = x - s.asyminit * (xmax - xmin);
      U = x + s.asyminit * (xmax - xmin);
    } else {
      const double sg = (x - x1) * (x1 - x2);
      const double gm = sg < 0. ? s.asymdec : sg > 0. ? s.asyminc : 1.;
      L = x - gm * (x1 - d.L[i]);
      U = x + gm * (d.U[i] - x1);
      const double w = fmax(1.0e-5, xmax - xmin);
      L = fmin(fmax(L, x - 10. * w), x - 0.01 * w);
      U = fmin(fmax(U, x + 0.01 * w), x + 10. * w);
    }
    d.L[i] = L;
    d.U[i] = U;
    d.al[i] = fmax(xmin, 0.9 * L + 0.1 * x);
    d.be[i] = fmin(xmax, 0.9 * U + 0.1 * x);
    const double ux = U - x, xl = x - L, reg = 0.5 * feps / (U - L), df = d.df0[i];
    d.p0[i] = ux * ux * (fmax(0., df) + 0.001 * fabs(df) + reg);
    d.q0[i] = xl * xl * (fmax(0., -df) + 0.001 * fabs(df) + reg);
    for (int j = 0; j < d.m; ++j) {
      const double gj = d.dg[(long long)j * d.n + i];
      const double P = ux * ux * fmax(0., gj), Q = xl * xl * fmax(0., -gj);
      d.P[(long long)j * d.n + i] = P;
      d.Q[(long long)j * d.n + i] = Q;
      acc[j] += P / ux + Q / xl;
    }
    d.x2[i] = x1;
    d.x1[i] = x;
  }
  block_store(acc, d.m, part, false);
}

// x(lam) into d.x, and the block sums of the dual gradient terms and (hess)
// of the dual Hessian's upper triangle.
__global__ void k_mma_dual(MmaDev d, MmaScalars s, double* part) {
  const int m = d.m;
  const int nv = s.hess ? m + m * (m + 1) / 2 : m;
  double acc[kMaxVals];
  for (int k = 0; k < nv; ++k) acc[k] = 0.;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.n;
       i += (long long)gridDim.x * blockDim.x) {
    double p = d.p0[i], q = d.q0[i];
    for (int j = 0; j < m; ++j) {
      p += d.P[(long long)j * d.n + i] * s.lam[j];
      q += d.Q[(long long)j * d.n + i] * s.lam[j];
    }
    const double L = d.L[i], U = d.U[i];
    const double sp = sqrt(p), sq = sqrt(q);
    const double xf = (sp * L + sq * U) / (sp + sq);
    const double x = fmin(fmax(xf, d.al[i]), d.be[i]);
    d.x[i] = x;
    const double ux = U - x, xl = x - L;
    for (int j = 0; j < m; ++j)
      acc[j] += d.P[(long long)j * d.n + i] / ux + d.Q[(long long)j * d.n + i] / xl;
    if (s.hess && !(xf < d.al[i] || xf > d.be[i])) {
      const double d2 = -1. / (2. * p / (ux * ux * ux) + 2. * q / (xl * xl * xl));
      double pq[kMaxM];
      for (int j = 0; j < m; ++j)
        pq[j] = d.P[(long long)j * d.n + i] / (ux * ux) - d.Q[(long long)j * d.n + i] / (xl * xl);
      int k = m;
      for (int j = 0; j < m; ++j)
        for (int l = j; l < m; ++l) acc[k++] += pq[j] * d2 * pq[l];
    }
  }
  block_store(acc, nv, part, false);
}

void solve_small(double* A, double* r, int m) {
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int k = c + 1; k < m; ++k)
      if (std::fabs(A[k * m + c]) > std::fabs(A[piv * m + c])) piv = k;
    if (piv != c) {
      for (int k = 0; k < m; ++k) std::swap(A[c * m + k], A[piv * m + k]);
      std::swap(r[c], r[piv]);
    }
    for (int k = c + 1; k < m; ++k) {
      const double f = A[k * m + c] / A[c * m + c];
      for (int l = c; l < m; ++l) A[k * m + l] -= f * A[c * m + l];
      r[k] -= f * r[c];
    }
  }
  for (int c = m - 1; c >= 0; --c) {
    double acc = r[c];
    for (int l = c + 1; l < m; ++l) acc -= A[c * m + l] * r[l];
    r[c] = acc / A[c * m + c];
  }
}

int grid_for(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  if (b > kMaxBlocks) b = kMaxBlocks;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

// ---------------------------------------------------------------------------

struct lbm_topopt {
  lbm_topopt_config cfg;
  Grid g;
  long long n = 0;                 // design variables
  int nstages = 0, nreal = 1, m = 0;
  cudaStream_t st = nullptr;
  int* box_d = nullptr;            // design box on the device
  double *bg = nullptr, *xfull = nullptr, *tmp = nullptr, *tmp2 = nullptr;
  struct Stage {
    int radius = 0, ntaps = 0;
    int* tap = nullptr;
    double* w = nullptr;
    double* den = nullptr;
  } stage[LBM_MAX_STAGES];
  double* keep[LBM_MAX_REALISATIONS][LBM_MAX_STAGES] = {};
  double* gamma[LBM_MAX_REALISATIONS] = {};
  double* df[LBM_MAX_REALISATIONS] = {};   // dJ_r/dx
  double J[LBM_MAX_REALISATIONS] = {};
  bool have_sens[LBM_MAX_REALISATIONS] = {};
  // MMA
  double *x = nullptr, *x1 = nullptr, *x2 = nullptr, *L = nullptr, *U = nullptr, *al = nullptr,
         *be = nullptr, *p0 = nullptr, *q0 = nullptr, *P = nullptr, *Q = nullptr, *df0 = nullptr,
         *dg = nullptr, *zero = nullptr;
  double *part = nullptr, *sums = nullptr;
  double a[kMaxM] = {}, c[kMaxM] = {};
  int k = 0;
  int dual_iterations = 0;
  std::vector<void*> allocs;
  std::string err;
};

namespace {

int tfail(lbm_topopt* t, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (t)
    t->err = buf;
  else
    lbm::set_global_error(buf);
  return code;
}

#define TCUDA(t, call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return tfail((t), LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

int talloc(lbm_topopt* t, double** p, long long count) {
  cudaError_t e = cudaMalloc((void**)p, sizeof(double) * (size_t)(count > 0 ? count : 1));
  if (e != cudaSuccess)
    return tfail(t, e == cudaErrorMemoryAllocation ? LBM_ERR_MEM : LBM_ERR_CUDA, "cudaMalloc: %s",
                 cudaGetErrorString(e));
  t->allocs.push_back(*p);
  return 0;
}

void tfree(lbm_topopt* t) {
  for (void* p : t->allocs) cudaFree(p);
  t->allocs.clear();
  if (t->st) cudaStreamDestroy(t->st);
  t->st = nullptr;
}

// stage k as seen by realisation r
StageDev stage_dev(const lbm_topopt* t, int k, int r) {
  StageDev s;
  memset(&s, 0, sizeof(s));
  const lbm_topopt_config& c = t->cfg;
  s.project = c.project[k];
  s.ntaps = t->stage[k].ntaps;
  for (int i = 0; i < 6; ++i) s.box[i] = c.filter_box[i];
  s.beta = c.beta[k];
  s.eta = (k == t->nstages - 1 && t->nreal > 1) ? c.real_eta[r] : c.eta[k];
  s.pden = std::tanh(s.beta * s.eta) + std::tanh(s.beta * (1. - s.eta));
  s.tap = t->stage[k].tap;
  s.w = t->stage[k].w;
  s.den = t->stage[k].den;
  return s;
}

int check_launch(lbm_topopt* t) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfail(t, LBM_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
  return 0;
}

// physical field of realisation r (and each stage's filtered field) from x
int forward_chain(lbm_topopt* t, int r) {
  const int gb = grid_for(t->g.n);
  k_scatter_box<<<gb, kThreads, 0, t->st>>>(t->g, t->box_d, t->x, t->bg, t->xfull);
  const double* in = t->xfull;
  if (t->nstages == 0) {
    TCUDA(t, cudaMemcpyAsync(t->gamma[r], t->xfull, sizeof(double) * t->g.n,
                             cudaMemcpyDeviceToDevice, t->st));
  }
  for (int k = 0; k < t->nstages; ++k) {
    double* out = (k == t->nstages - 1) ? t->gamma[r] : t->tmp2;
    k_stage_forward<<<gb, kThreads, 0, t->st>>>(t->g, stage_dev(t, k, r), in, t->keep[r][k], out);
    in = out;
  }
  return check_launch(t);
}

// design sensitivity (n) from a full-grid sensitivity in t->tmp, realisation r
int transpose_chain(lbm_topopt* t, int r, double* out_design) {
  const int gb = grid_for(t->g.n);
  for (int k = t->nstages - 1; k >= 0; --k) {
    StageDev s = stage_dev(t, k, r);
    k_stage_scale<<<gb, kThreads, 0, t->st>>>(t->g, s, t->keep[r][k], t->tmp, t->tmp2);
    k_stage_transpose<<<gb, kThreads, 0, t->st>>>(t->g, s, t->tmp2, t->tmp);
  }
  k_gather_box<<<grid_for(t->n), kThreads, 0, t->st>>>(t->g, t->box_d, t->n, t->tmp, out_design);
  return check_launch(t);
}

// fixed-order sum (or max) into host values
int reduce_to_host(lbm_topopt* t, int nblk, int nv, bool use_max, double* host) {
  k_finish<<<1, 64, 0, t->st>>>(t->part, nblk, nv, t->sums, use_max ? 1 : 0);
  TCUDA(t, cudaGetLastError());
  TCUDA(t, cudaMemcpyAsync(host, t->sums, sizeof(double) * nv, cudaMemcpyDeviceToHost, t->st));
  TCUDA(t, cudaStreamSynchronize(t->st));
  return 0;
}

int validate_topopt(const lbm_topopt_config& c) {
  if (c.nx < 1 || c.ny < 1 || c.nz < 1) return tfail(nullptr, LBM_ERR_ARG, "lattice must be >= 1 cell per axis");
  if ((double)c.nx * c.ny * c.nz > 2.0e9) return tfail(nullptr, LBM_ERR_ARG, "lattice too large");
  auto bad_box = [&](const int* b) {
    return b[0] < 0 || b[1] >= c.nx || b[0] > b[1] || b[2] < 0 || b[3] >= c.ny || b[2] > b[3] ||
           b[4] < 0 || b[5] >= c.nz || b[4] > b[5];
  };
  if (bad_box(c.design_box)) return tfail(nullptr, LBM_ERR_ARG, "design box outside the lattice");
  if (c.nstages < 0 || c.nstages > LBM_MAX_STAGES)
    return tfail(nullptr, LBM_ERR_ARG, "nstages must be 0..%d", LBM_MAX_STAGES);
  if (c.nstages > 0 && bad_box(c.filter_box)) return tfail(nullptr, LBM_ERR_ARG, "filter box outside the lattice");
  for (int k = 0; k < c.nstages; ++k) {
    const int rmax = c.nz > 1 ? 12 : 32;
    if (c.radius[k] < 1 || c.radius[k] > rmax)
      return tfail(nullptr, LBM_ERR_ARG, "filter radius %d outside 1..%d", c.radius[k], rmax);
    if (c.project[k] && !(c.beta[k] > 0. && c.eta[k] >= 0. && c.eta[k] <= 1.))
      return tfail(nullptr, LBM_ERR_ARG, "projection needs beta > 0 and eta in [0,1]");
  }
  if (c.nreal < 1 || c.nreal > LBM_MAX_REALISATIONS)
    return tfail(nullptr, LBM_ERR_ARG, "nreal must be 1..%d", LBM_MAX_REALISATIONS);
  if (c.nreal > 1 && c.nstages > 0 && !c.project[c.nstages - 1])
    return tfail(nullptr, LBM_ERR_ARG, "several realisations need a last stage with projection");
  if (c.volume_type != LBM_VOLUME_NONE && c.volume_type != LBM_VOLUME_FLUID &&
      c.volume_type != LBM_VOLUME_MATERIAL)
    return tfail(nullptr, LBM_ERR_ARG, "unknown volume constraint %d", c.volume_type);
  if (c.nreal == 1 && c.volume_type == LBM_VOLUME_NONE)
    return tfail(nullptr, LBM_ERR_ARG, "a single realisation needs a volume constraint");
  if (c.volume_real < 0 || c.volume_real >= c.nreal)
    return tfail(nullptr, LBM_ERR_ARG, "volume_real outside 0..nreal-1");
  if (!(c.move_limit > 0. && c.move_limit <= 1.)) return tfail(nullptr, LBM_ERR_ARG, "move limit must be in (0,1]");
  return 0;
}

}  // namespace

extern "C" {

void lbm_topopt_config_default(lbm_topopt_config* c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->nx = c->ny = c->nz = 1;
  c->nstages = 1;
  c->radius[0] = c->radius[1] = 2;
  c->project[0] = 1;
  c->beta[0] = c->beta[1] = 1.;
  c->eta[0] = c->eta[1] = 0.5;
  c->nreal = 1;
  for (int r = 0; r < LBM_MAX_REALISATIONS; ++r) c->real_eta[r] = 0.5;
  c->volume_type = LBM_VOLUME_FLUID;
  c->volume = 0.5;
  c->move_limit = 0.1;
  c->magic = 5.;
}

int lbm_topopt_create(const lbm_topopt_config* cfg, const double* background, const double* x0,
                      lbm_topopt** out) {
  if (!cfg || !out) return tfail(nullptr, LBM_ERR_ARG, "null argument");
  *out = nullptr;
  int rc = validate_topopt(*cfg);
  if (rc) return rc;
  lbm_topopt* t = new lbm_topopt;
  t->cfg = *cfg;
  const lbm_topopt_config& c = t->cfg;
  t->g = Grid{c.nx, c.ny, c.nz, (long long)c.nx * c.ny * c.nz};
  const int* b = c.design_box;
  t->n = (long long)(b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1);
  t->nstages = c.nstages;
  t->nreal = c.nreal;
  const bool vol = c.volume_type != LBM_VOLUME_NONE;
  t->m = (c.nreal > 1 ? c.nreal : 0) + (vol ? 1 : 0);
  for (int j = 0; j < kMaxM; ++j) {
    t->a[j] = (c.nreal > 1 && j < c.nreal) ? 1. : 0.;   // robust constants (SetRobustConstants)
    t->c[j] = 1000.;
  }
  auto bail = [&](int code) {
    tfree(t);
    std::string msg = t->err;
    delete t;
    lbm::set_global_error(msg.c_str());
    return code;
  };
  if (cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking) != cudaSuccess) {
    t->err = "no CUDA device (cudaStreamCreate failed)";
    return bail(LBM_ERR_CUDA);
  }
  const long long N = t->g.n, n = t->n;
  if ((rc = talloc(t, &t->bg, N)) || (rc = talloc(t, &t->xfull, N)) || (rc = talloc(t, &t->tmp, N)) ||
      (rc = talloc(t, &t->tmp2, N)))
    return bail(rc);
  for (int r = 0; r < t->nreal; ++r) {
    if ((rc = talloc(t, &t->gamma[r], N)) || (rc = talloc(t, &t->df[r], n))) return bail(rc);
    for (int k = 0; k < t->nstages; ++k)
      if ((rc = talloc(t, &t->keep[r][k], N))) return bail(rc);
  }
  double** mm[] = {&t->x, &t->x1, &t->x2, &t->L, &t->U, &t->al, &t->be, &t->p0, &t->q0, &t->df0, &t->zero};
  for (double** p : mm)
    if ((rc = talloc(t, p, n))) return bail(rc);
  if ((rc = talloc(t, &t->P, (long long)t->m * n)) || (rc = talloc(t, &t->Q, (long long)t->m * n)) ||
      (rc = talloc(t, &t->dg, (long long)t->m * n)) ||
      (rc = talloc(t, &t->part, (long long)kMaxBlocks * kMaxVals)) || (rc = talloc(t, &t->sums, kMaxVals)))
    return bail(rc);
  int* bx = nullptr;
  if (cudaMalloc((void**)&bx, 6 * sizeof(int)) != cudaSuccess) {
    t->err = "cudaMalloc failed";
    return bail(LBM_ERR_MEM);
  }
  t->allocs.push_back(bx);
  t->box_d = bx;
  cudaMemcpyAsync(bx, c.design_box, 6 * sizeof(int), cudaMemcpyHostToDevice, t->st);
  // background and initial design
  std::vector<double> h(N);
  if (background) {
    for (long long i = 0; i < N; ++i) {
      if (!(background[i] >= 0. && background[i] <= 1.)) {
        t->err = "background value outside [0,1]";
        return bail(LBM_ERR_ARG);
      }
      h[i] = background[i];
    }
  } else {
    std::fill(h.begin(), h.end(), 1.);
  }
  cudaMemcpyAsync(t->bg, h.data(), sizeof(double) * N, cudaMemcpyHostToDevice, t->st);
  cudaStreamSynchronize(t->st);
  std::vector<double> hx(n, 0.5);
  if (x0)
    for (long long i = 0; i < n; ++i) {
      if (!(x0[i] >= 0. && x0[i] <= 1.)) {
        t->err = "initial design variable outside [0,1]";
        return bail(LBM_ERR_ARG);
      }
      hx[i] = x0[i];
    }
  cudaMemcpyAsync(t->x, hx.data(), sizeof(double) * n, cudaMemcpyHostToDevice, t->st);
  cudaMemcpyAsync(t->x1, hx.data(), sizeof(double) * n, cudaMemcpyHostToDevice, t->st);
  cudaMemcpyAsync(t->x2, hx.data(), sizeof(double) * n, cudaMemcpyHostToDevice, t->st);
  k_fill<<<grid_for(n), kThreads, 0, t->st>>>(t->zero, n, 0.);
  cudaStreamSynchronize(t->st);
  // filter taps and row sums
  for (int k = 0; k < t->nstages; ++k) {
    const int R = c.radius[k], R3 = c.nz > 1 ? R : 0;
    std::vector<int> taps;
    std::vector<double> w;
    for (int dz = -R3; dz <= R3; ++dz)
      for (int dy = -R; dy <= R; ++dy)
        for (int dx = -R; dx <= R; ++dx) {
          const double d = std::sqrt((double)(dx * dx + dy * dy + dz * dz));
          if (d < (double)R) {   // weight R - d > 0; the d = R entries carry weight 0
            taps.push_back(dx);
            taps.push_back(dy);
            taps.push_back(dz);
            w.push_back((double)R - d);
          }
        }
    lbm_topopt::Stage& s = t->stage[k];
    s.radius = R;
    s.ntaps = (int)w.size();
    int* tp = nullptr;
    if (cudaMalloc((void**)&tp, sizeof(int) * taps.size()) != cudaSuccess) {
      t->err = "cudaMalloc failed";
      return bail(LBM_ERR_MEM);
    }
    t->allocs.push_back(tp);
    s.tap = tp;
    if ((rc = talloc(t, &s.w, (long long)w.size())) || (rc = talloc(t, &s.den, N))) return bail(rc);
    cudaMemcpyAsync(s.tap, taps.data(), sizeof(int) * taps.size(), cudaMemcpyHostToDevice, t->st);
    cudaMemcpyAsync(s.w, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, t->st);
    cudaStreamSynchronize(t->st);
    k_den<<<grid_for(N), kThreads, 0, t->st>>>(t->g, stage_dev(t, k, 0), s.den);
  }
  if (cudaStreamSynchronize(t->st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    t->err = "set-up kernels failed";
    return bail(LBM_ERR_CUDA);
  }
  *out = t;
  return LBM_OK;
}

int lbm_topopt_destroy(lbm_topopt* t) {
  if (!t) return LBM_OK;
  tfree(t);
  delete t;
  return LBM_OK;
}

const char* lbm_topopt_last_error(const lbm_topopt* t) {
  if (!t) return lbm_last_error(nullptr);
  return t->err.c_str();
}

int lbm_topopt_num_variables(const lbm_topopt* t, int64_t* n) {
  if (!t || !n) return tfail(nullptr, LBM_ERR_ARG, "null argument");
  *n = t->n;
  return LBM_OK;
}

int lbm_topopt_set_variables(lbm_topopt* t, const double* x) {
  if (!t || !x) return tfail(t, LBM_ERR_ARG, "null argument");
  for (long long i = 0; i < t->n; ++i)
    if (!(x[i] >= 0. && x[i] <= 1.)) return tfail(t, LBM_ERR_ARG, "design variable %lld outside [0,1]", i);
  TCUDA(t, cudaMemcpyAsync(t->x, x, sizeof(double) * t->n, cudaMemcpyHostToDevice, t->st));
  TCUDA(t, cudaStreamSynchronize(t->st));
  for (int r = 0; r < t->nreal; ++r) t->have_sens[r] = false;
  return LBM_OK;
}

int lbm_topopt_get_variables(const lbm_topopt* t, double* x) {
  if (!t || !x) return tfail(nullptr, LBM_ERR_ARG, "null argument");
  lbm_topopt* tt = const_cast<lbm_topopt*>(t);
  TCUDA(tt, cudaMemcpyAsync(x, t->x, sizeof(double) * t->n, cudaMemcpyDeviceToHost, t->st));
  TCUDA(tt, cudaStreamSynchronize(t->st));
  return LBM_OK;
}

int lbm_topopt_set_beta(lbm_topopt* t, int stage, double beta) {
  if (!t) return tfail(nullptr, LBM_ERR_ARG, "null handle");
  if (stage < 0 || stage >= t->nstages) return tfail(t, LBM_ERR_ARG, "no stage %d", stage);
  if (!(beta > 0.)) return tfail(t, LBM_ERR_ARG, "beta must be > 0");
  t->cfg.beta[stage] = beta;
  for (int r = 0; r < t->nreal; ++r) t->have_sens[r] = false;
  return LBM_OK;
}

int lbm_topopt_physical(lbm_topopt* t, int r, double* gamma) {
  if (!t || !gamma) return tfail(t, LBM_ERR_ARG, "null argument");
  if (r < 0 || r >= t->nreal) return tfail(t, LBM_ERR_ARG, "no realisation %d", r);
  int rc = forward_chain(t, r);
  if (rc) return rc;
  TCUDA(t, cudaMemcpyAsync(gamma, t->gamma[r], sizeof(double) * t->g.n, cudaMemcpyDeviceToHost, t->st));
  TCUDA(t, cudaStreamSynchronize(t->st));
  return LBM_OK;
}

int lbm_topopt_apply(lbm_topopt* t, int r, lbm_handle* h) {
  if (!t || !h) return tfail(t, LBM_ERR_ARG, "null argument");
  if (r < 0 || r >= t->nreal) return tfail(t, LBM_ERR_ARG, "no realisation %d", r);
  int64_t nc = 0;
  int npop = 0;
  if (lbm_get_sizes(h, &nc, &npop) || nc != t->g.n)
    return tfail(t, LBM_ERR_ARG, "handle has %lld cells, the design chain %lld", (long long)nc, t->g.n);
  int rc = forward_chain(t, r);
  if (rc) return rc;
  TCUDA(t, cudaStreamSynchronize(t->st));
  rc = lbm_set_design_device(h, t->gamma[r]);
  if (rc) return tfail(t, rc, "lbm_set_design_device: %s", lbm_last_error(h));
  return LBM_OK;
}

static int set_sensitivity_common(lbm_topopt* t, int r, double J) {
  int rc = forward_chain(t, r);   // the filtered fields the chain rule is taken at
  if (rc) return rc;
  if (t->nstages == 0) {
    k_gather_box<<<grid_for(t->n), kThreads, 0, t->st>>>(t->g, t->box_d, t->n, t->tmp, t->df[r]);
    if ((rc = check_launch(t))) return rc;
  } else if ((rc = transpose_chain(t, r, t->df[r]))) {
    return rc;
  }
  TCUDA(t, cudaStreamSynchronize(t->st));
  t->J[r] = J;
  t->have_sens[r] = true;
  return LBM_OK;
}

int lbm_topopt_set_sensitivity(lbm_topopt* t, int r, lbm_handle* h, double J) {
  if (!t || !h) return tfail(t, LBM_ERR_ARG, "null argument");
  if (r < 0 || r >= t->nreal) return tfail(t, LBM_ERR_ARG, "no realisation %d", r);
  int64_t nc = 0;
  int npop = 0;
  if (lbm_get_sizes(h, &nc, &npop) || nc != t->g.n)
    return tfail(t, LBM_ERR_ARG, "handle has %lld cells, the design chain %lld", (long long)nc, t->g.n);
  if (!std::isfinite(J)) return tfail(t, LBM_ERR_NONFINITE, "objective is not finite");
  const double* sens = nullptr;
  if (lbm_get_sensitivity_device(h, &sens) || !sens) return tfail(t, LBM_ERR_STATE, "handle has no sensitivity");
  TCUDA(t, cudaDeviceSynchronize());   // the handle's reverse sweep is complete
  TCUDA(t, cudaMemcpyAsync(t->tmp, sens, sizeof(double) * t->g.n, cudaMemcpyDeviceToDevice, t->st));
  return set_sensitivity_common(t, r, J);
}

int lbm_topopt_set_sensitivity_host(lbm_topopt* t, int r, const double* dJdgamma, double J) {
  if (!t || !dJdgamma) return tfail(t, LBM_ERR_ARG, "null argument");
  if (r < 0 || r >= t->nreal) return tfail(t, LBM_ERR_ARG, "no realisation %d", r);
  if (!std::isfinite(J)) return tfail(t, LBM_ERR_NONFINITE, "objective is not finite");
  TCUDA(t, cudaMemcpyAsync(t->tmp, dJdgamma, sizeof(double) * t->g.n, cudaMemcpyHostToDevice, t->st));
  return set_sensitivity_common(t, r, J);
}

int lbm_topopt_get_design_sensitivity(const lbm_topopt* t, int r, double* dJdx) {
  if (!t || !dJdx) return tfail(nullptr, LBM_ERR_ARG, "null argument");
  lbm_topopt* tt = const_cast<lbm_topopt*>(t);
  if (r < 0 || r >= t->nreal) return tfail(tt, LBM_ERR_ARG, "no realisation %d", r);
  if (!t->have_sens[r]) return tfail(tt, LBM_ERR_STATE, "no sensitivity set for realisation %d", r);
  TCUDA(tt, cudaMemcpyAsync(dJdx, t->df[r], sizeof(double) * t->n, cudaMemcpyDeviceToHost, t->st));
  TCUDA(tt, cudaStreamSynchronize(t->st));
  return LBM_OK;
}

int lbm_topopt_update(lbm_topopt* t, double* change, double* constraints) {
  if (!t) return tfail(nullptr, LBM_ERR_ARG, "null handle");
  const lbm_topopt_config& c = t->cfg;
  for (int r = 0; r < t->nreal; ++r)
    if (!t->have_sens[r]) return tfail(t, LBM_ERR_STATE, "no sensitivity set for realisation %d", r);
  const long long n = t->n;
  const int m = t->m;
  int rc;
  double g[kMaxM] = {};
  // constraint values and sensitivities (row j of dg)
  int j = 0;
  if (t->nreal > 1)
    for (int r = 0; r < t->nreal; ++r, ++j) {
      g[j] = t->J[r] + c.magic;
      TCUDA(t, cudaMemcpyAsync(t->dg + (long long)j * n, t->df[r], sizeof(double) * n,
                               cudaMemcpyDeviceToDevice, t->st));
    }
  if (c.volume_type != LBM_VOLUME_NONE) {
    const int vr = c.volume_real;
    if ((rc = forward_chain(t, vr))) return rc;
    // mean of the physical field over the design box
    double* row = t->dg + (long long)j * n;
    k_gather_box<<<grid_for(n), kThreads, 0, t->st>>>(t->g, t->box_d, n, t->gamma[vr], row);
    const int nb = grid_for(n);
    k_sum<<<nb, kThreads, 0, t->st>>>(row, n, t->part);
    if ((rc = check_launch(t))) return rc;
    double sum = 0.;
    if ((rc = reduce_to_host(t, nb, 1, false, &sum))) return rc;
    const double mean = sum / (double)n;
    g[j] = c.volume_type == LBM_VOLUME_FLUID ? -c.volume + mean : (1. - c.volume) - mean;
    // its sensitivity: +-1/n on the full grid, through the filters, onto the box
    k_fill<<<grid_for(t->g.n), kThreads, 0, t->st>>>(
        t->tmp, t->g.n, (c.volume_type == LBM_VOLUME_FLUID ? 1. : -1.) / (double)n);
    if (t->nstages == 0) {
      k_gather_box<<<grid_for(n), kThreads, 0, t->st>>>(t->g, t->box_d, n, t->tmp, row);
    } else if ((rc = transpose_chain(t, vr, row))) {
      return rc;
    }
    ++j;
  }
  const double* df0 = t->nreal > 1 ? t->zero : t->df[0];
  // ---- MMA ----
  t->k += 1;
  MmaDev d{n, m, t->x, t->x1, t->x2, t->L, t->U, t->al, t->be, t->p0, t->q0, t->P, t->Q, df0, t->dg};
  MmaScalars s;
  memset(&s, 0, sizeof(s));
  s.k = t->k;
  s.asyminit = 0.5;
  s.asymdec = 0.7;
  s.asyminc = 1.2;
  s.movlim = c.move_limit;
  const int nb = grid_for(n);
  double b[kMaxM];
  k_mma_gensub<<<nb, kThreads, 0, t->st>>>(d, s, t->part);
  if ((rc = check_launch(t))) return rc;
  if ((rc = reduce_to_host(t, nb, m, false, b))) return rc;
  for (int i = 0; i < m; ++i) b[i] -= g[i];

  double lam[kMaxM], mu[kMaxM], vals[kMaxVals], gr[kMaxM], H[kMaxM * kMaxM], ds[kMaxM], dm[kMaxM];
  for (int i = 0; i < m; ++i) {
    lam[i] = t->c[i] / 2.;
    mu[i] = 1.;
  }
  // x(lam) on the device, y(lam), z(lam) and the dual gradient here
  auto evaluate = [&](bool hess) -> int {
    for (int i = 0; i < m; ++i) {
      if (lam[i] < 0.) lam[i] = 0.;
      s.lam[i] = lam[i];
    }
    s.hess = hess ? 1 : 0;
    k_mma_dual<<<nb, kThreads, 0, t->st>>>(d, s, t->part);
    int r2 = check_launch(t);
    if (r2) return r2;
    const int nv = hess ? m + m * (m + 1) / 2 : m;
    if ((r2 = reduce_to_host(t, nb, nv, false, vals))) return r2;
    double la = 0.;
    for (int i = 0; i < m; ++i) la += lam[i] * t->a[i];
    const double z = std::max(0., 10. * (la - 1.));
    for (int i = 0; i < m; ++i) gr[i] = vals[i] - b[i] - t->a[i] * z - std::max(0., lam[i] - t->c[i]);
    if (hess) {
      int k = m;
      for (int i = 0; i < m; ++i)
        for (int l = i; l < m; ++l) {
          H[i * m + l] = vals[k];
          H[l * m + i] = vals[k];
          ++k;
        }
      for (int i = 0; i < m; ++i)
        if (lam[i] > t->c[i]) H[i * m + i] -= 1.;
      if (la > 1.)
        for (int i = 0; i < m; ++i)
          for (int l = 0; l < m; ++l) H[i * m + l] -= 10. * t->a[i] * t->a[l];
    }
    return 0;
  };
  const double tol = 1.0e-9 * std::sqrt((double)(m + n));
  double eps = 1., err = 1.;
  int iters = 0;
  while (eps > tol) {
    int loop = 0;
    while (err > 0.9 * eps && loop < 100) {
      ++loop;
      ++iters;
      if ((rc = evaluate(true))) return rc;
      double tr = 0.;
      for (int i = 0; i < m; ++i) {
        H[i * m + i] -= mu[i] / lam[i];
        tr += H[i * m + i];
      }
      const double shift = std::min(-1.0e-7, 1.0e-4 * tr / m);
      for (int i = 0; i < m; ++i) {
        H[i * m + i] += shift;
        ds[i] = -gr[i] - eps / lam[i];
      }
      solve_small(H, ds, m);
      for (int i = 0; i < m; ++i) dm[i] = -mu[i] + eps / lam[i] - ds[i] * mu[i] / lam[i];
      double th = 1.005;
      for (int i = 0; i < m; ++i) {
        th = std::max(th, -1.01 * ds[i] / lam[i]);
        th = std::max(th, -1.01 * dm[i] / mu[i]);
      }
      th = 1. / th;
      for (int i = 0; i < m; ++i) {
        lam[i] += th * ds[i];
        mu[i] += th * dm[i];
      }
      if ((rc = evaluate(false))) return rc;
      err = 0.;
      for (int i = 0; i < m; ++i) {
        err = std::max(err, std::fabs(gr[i] + mu[i]));
        err = std::max(err, std::fabs(mu[i] * lam[i] - eps));
      }
    }
    eps *= 0.1;
  }
  t->dual_iterations = iters;
  // x now holds x(lam); the change against the expansion point
  k_max_abs_diff<<<nb, kThreads, 0, t->st>>>(t->x, t->x1, n, t->part);
  if ((rc = check_launch(t))) return rc;
  double ch = 0.;
  if ((rc = reduce_to_host(t, nb, 1, true, &ch))) return rc;
  if (change) *change = ch;
  if (constraints)
    for (int i = 0; i < m; ++i) constraints[i] = g[i];
  for (int r = 0; r < t->nreal; ++r) t->have_sens[r] = false;
  return LBM_OK;
}

}  // extern "C"
