// Host build of the device collision operators and their transposes
// (lbm-topopt_gb300/csrc/lbm_device.cuh) for CPU tests: CUDA qualifiers and
// warp intrinsics are stubbed so the same source compiles with g++, and the
// per-cell functions can be compared with the oracle without a GPU.
// Test infrastructure only.
#include <cmath>
#include <cstdio>
#include <cstring>
#define __device__
#define __host__
#define __forceinline__ inline
#define __global__
#define __launch_bounds__(...)
#include <cuda_fp16.h>
#include <cuda_runtime.h>
struct lbm_dim3_stub { unsigned x = 0, y = 0, z = 0; };
static lbm_dim3_stub threadIdx, blockIdx, blockDim, gridDim;
template <class T> T __shfl_down_sync(unsigned, T v, int) { return v; }
inline int __any_sync(unsigned, int v) { return v; }
inline void __syncthreads() {}
inline void __threadfence() {}
inline unsigned atomicAdd(unsigned* p, unsigned v) { unsigned o = *p; *p += v; return o; }
inline float __ldcs(const float* p) { return *p; }
inline void __stcs(float* p, float v) { *p = v; }
#include "../lbm-topopt_gb300/csrc/lbm_device.cuh"

using namespace lbm;

namespace {
template <class C>
void fill(KParams& p, const lbm_config* c) {
  memset(&p, 0, sizeof(p));
  ModelParams<double>& d = p.md;
  d.omega = c->omega;
  for (int i = 0; i < 8; ++i) d.mrt[i] = c->mrt[i];
  d.pbb_scale = c->interp_scale;
  d.pbb_q = c->interp_q;
  d.diff = c->diffusivity;
  d.ramp_q = c->ramp_q;
  d.ramp_ck = c->ramp_ck;
  d.heat_rate = c->heat_rate;
  d.heat_T = c->heat_T;
  ModelParams<float>& f = p.mf;
  f.omega = (float)d.omega;
  for (int i = 0; i < 8; ++i) f.mrt[i] = (float)d.mrt[i];
  f.pbb_scale = (float)d.pbb_scale;
  f.pbb_q = (float)d.pbb_q;
  f.diff = (float)d.diff;
  f.ramp_q = (float)d.ramp_q;
  f.ramp_ck = (float)d.ramp_ck;
  f.heat_rate = (float)d.heat_rate;
  f.heat_T = (float)d.heat_T;
}

template <int LAT, int COLL, class C>
void collide(const lbm_config* cfg, const double* fin, double g, double* fout) {
  KParams p;
  fill<C>(p, cfg);
  constexpr int Q = Lattice<LAT>::Q;
  C f[Q];
  for (int i = 0; i < Q; ++i) f[i] = (C)fin[i];
  const C gg = (C)g;
  const C imult = C(0.5) * (mp<C>(p).pbb_scale * bp(gg, mp<C>(p).pbb_q));
  C rho, jx, jy, jz, T;
  flow_collide<LAT, COLL>(f, imult, rho, jx, jy, jz, p);
  if constexpr (LAT == LAT_D2Q9_D2Q5) thermal_collide(f + 9, jx, jy, gg, T, p);
  for (int i = 0; i < Q; ++i) fout[i] = (double)f[i];
}

template <int LAT, int COLL, class C>
void reverse(const lbm_config* cfg, const double* fin, double g, const double* lo, double* li,
             double* dgo) {
  KParams p;
  fill<C>(p, cfg);
  constexpr int Q = Lattice<LAT>::Q;
  C f[Q], lam[Q];
  for (int i = 0; i < Q; ++i) {
    f[i] = (C)fin[i];
    lam[i] = (C)lo[i];
  }
  const C gg = (C)g;
  const C imult = C(0.5) * (mp<C>(p).pbb_scale * bp(gg, mp<C>(p).pbb_q));
  const C dimult = C(0.5) * (mp<C>(p).pbb_scale * bp_diff(gg, mp<C>(p).pbb_q));
  C dg = C(0.), uxR = C(0.), uyR = C(0.);
  if constexpr (LAT == LAT_D2Q9_D2Q5) {
    C rho, jx, jy, jz;
    flow_macros<LAT>(f, rho, jx, jy, jz);
    thermal_reverse(f + 9, lam + 9, jx, jy, gg, uxR, uyR, dg, p);
  }
  flow_reverse<LAT, COLL>(f, lam, imult, dimult, dg, p);
  if constexpr (LAT == LAT_D2Q9_D2Q5) {
    for (int i = 0; i < 9; ++i)
      lam[i] += uxR * C(Lattice<LAT>::ex(i)) + uyR * C(Lattice<LAT>::ey(i));
  }
  for (int i = 0; i < Q; ++i) li[i] = (double)lam[i];
  *dgo = (double)dg;
}

template <class C>
int dispatch_collide(const lbm_config* c, const double* fin, double g, double* fout) {
  if (c->lattice == LBM_D2Q9 && c->collision == LBM_BGK) collide<LAT_D2Q9, LBM_BGK, C>(c, fin, g, fout);
  else if (c->lattice == LBM_D2Q9) collide<LAT_D2Q9, LBM_MRT, C>(c, fin, g, fout);
  else if (c->lattice == LBM_D3Q19 && c->collision == LBM_BGK) collide<LAT_D3Q19, LBM_BGK, C>(c, fin, g, fout);
  else if (c->lattice == LBM_D3Q19) collide<LAT_D3Q19, LBM_MRT, C>(c, fin, g, fout);
  else collide<LAT_D2Q9_D2Q5, LBM_BGK, C>(c, fin, g, fout);
  return 0;
}

template <class C>
int dispatch_reverse(const lbm_config* c, const double* fin, double g, const double* lo, double* li,
                     double* dg) {
  if (c->lattice == LBM_D2Q9 && c->collision == LBM_BGK) reverse<LAT_D2Q9, LBM_BGK, C>(c, fin, g, lo, li, dg);
  else if (c->lattice == LBM_D2Q9) reverse<LAT_D2Q9, LBM_MRT, C>(c, fin, g, lo, li, dg);
  else if (c->lattice == LBM_D3Q19 && c->collision == LBM_BGK) reverse<LAT_D3Q19, LBM_BGK, C>(c, fin, g, lo, li, dg);
  else if (c->lattice == LBM_D3Q19) reverse<LAT_D3Q19, LBM_MRT, C>(c, fin, g, lo, li, dg);
  else reverse<LAT_D2Q9_D2Q5, LBM_BGK, C>(c, fin, g, lo, li, dg);
  return 0;
}
}  // namespace

extern "C" {
int dev_collide(const lbm_config* c, int fp32, const double* fin, double g, double* fout) {
  return fp32 ? dispatch_collide<float>(c, fin, g, fout) : dispatch_collide<double>(c, fin, g, fout);
}
int dev_reverse(const lbm_config* c, int fp32, const double* fin, double g, const double* lo,
                double* li, double* dg) {
  return fp32 ? dispatch_reverse<float>(c, fin, g, lo, li, dg)
              : dispatch_reverse<double>(c, fin, g, lo, li, dg);
}
}
