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
inline int __syncthreads_or(int v) { return v; }
inline void __threadfence() {}
inline unsigned atomicAdd(unsigned* p, unsigned v) { unsigned o = *p; *p += v; return o; }
inline double atomicAdd(double* p, double v) { double o = *p; *p += v; return o; }
inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
inline float __ldcs(const float* p) { return *p; }
inline void __stcs(float* p, float v) { *p = v; }
inline float __uint_as_float(unsigned u) { float f; memcpy(&f, &u, 4); return f; }
inline unsigned __float_as_uint(float f) { unsigned u; memcpy(&u, &f, 4); return u; }
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

// f + d from the increment form of the collision (FP32/FP16 storage path)
template <int LAT, int COLL, class C>
void collide_inc(const lbm_config* cfg, const double* fin, double g, double* fout, double* sums) {
  KParams p;
  fill<C>(p, cfg);
  using L = Lattice<LAT>;
  constexpr int Q = L::Q;
  C f[Q], d[Q];
  for (int i = 0; i < Q; ++i) f[i] = (C)fin[i];
  const C gg = (C)g;
  const C imult = C(0.5) * (mp<C>(p).pbb_scale * bp(gg, mp<C>(p).pbb_q));
  C rho, jx, jy, jz;
  flow_collide_inc<LAT, COLL>(
      f, imult, rho, jx, jy, jz, p, [&](auto Q_, C dq) { d[decltype(Q_)::value] = dq; },
      [&](auto QA_, auto QB_, C da, C db) {
        d[decltype(QA_)::value] = da;
        d[decltype(QB_)::value] = db;
      });
  if constexpr (LAT == LAT_D2Q9_D2Q5)
    thermal_collide_inc(f + 9, jx, jy, gg, p, [&](auto I_, C dq) { d[decltype(I_)::value + 9] = dq; });
  for (int i = 0; i < Q; ++i) fout[i] = (double)f[i] + (double)d[i];
  // mass and momentum of the flow increments, and the largest increment
  double m[5] = {0., 0., 0., 0., 0.};
  for (int i = 0; i < L::QF; ++i) {
    m[0] += (double)d[i];
    m[1] += L::ex(i) * (double)d[i];
    m[2] += L::ey(i) * (double)d[i];
    m[3] += L::ez(i) * (double)d[i];
    m[4] = fmax(m[4], fabs((double)d[i]));
  }
  for (int k = 0; k < 5; ++k) sums[k] = m[k];
}

// lo + d from the increment form of the BGK / thermal reverse collision
template <int LAT, class C>
void reverse_inc(const lbm_config* cfg, const double* fin, double g, const double* lo, double* li,
                 double* dgo) {
  KParams p;
  fill<C>(p, cfg);
  using L = Lattice<LAT>;
  constexpr int Q = L::Q;
  C f[Q], lam[Q], d[Q];
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
    thermal_reverse_inc(f + 9, lam + 9, d + 9, jx, jy, gg, uxR, uyR, dg, p);
  }
  bgk_reverse_inc<LAT>(f, lam, d, imult, dimult, dg, p);
  if constexpr (LAT == LAT_D2Q9_D2Q5) {
    for (int i = 0; i < 9; ++i) d[i] += uxR * C(L::ex(i)) + uyR * C(L::ey(i));
  }
  for (int i = 0; i < Q; ++i) li[i] = (double)lam[i] + (double)d[i];
  *dgo = (double)dg;
}

template <class C>
int dispatch_collide_inc(const lbm_config* c, const double* fin, double g, double* fout, double* sums) {
  if (c->lattice == LBM_D2Q9 && c->collision == LBM_BGK) collide_inc<LAT_D2Q9, LBM_BGK, C>(c, fin, g, fout, sums);
  else if (c->lattice == LBM_D2Q9) collide_inc<LAT_D2Q9, LBM_MRT, C>(c, fin, g, fout, sums);
  else if (c->lattice == LBM_D3Q19 && c->collision == LBM_BGK) collide_inc<LAT_D3Q19, LBM_BGK, C>(c, fin, g, fout, sums);
  else if (c->lattice == LBM_D3Q19) collide_inc<LAT_D3Q19, LBM_MRT, C>(c, fin, g, fout, sums);
  else collide_inc<LAT_D2Q9_D2Q5, LBM_BGK, C>(c, fin, g, fout, sums);
  return 0;
}

template <class C>
int dispatch_reverse_inc(const lbm_config* c, const double* fin, double g, const double* lo,
                         double* li, double* dg) {
  if (c->collision != LBM_BGK) return -1;
  if (c->lattice == LBM_D2Q9) reverse_inc<LAT_D2Q9, C>(c, fin, g, lo, li, dg);
  else if (c->lattice == LBM_D3Q19) reverse_inc<LAT_D3Q19, C>(c, fin, g, lo, li, dg);
  else reverse_inc<LAT_D2Q9_D2Q5, C>(c, fin, g, lo, li, dg);
  return 0;
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
int dev_collide_inc(const lbm_config* c, int fp32, const double* fin, double g, double* fout,
                    double* sums) {
  return fp32 ? dispatch_collide_inc<float>(c, fin, g, fout, sums)
              : dispatch_collide_inc<double>(c, fin, g, fout, sums);
}
int dev_reverse_inc(const lbm_config* c, int fp32, const double* fin, double g, const double* lo,
                    double* li, double* dg) {
  return fp32 ? dispatch_reverse_inc<float>(c, fin, g, lo, li, dg)
              : dispatch_reverse_inc<double>(c, fin, g, lo, li, dg);
}
// Round<S>::apply(f, d) for n cells at one time step; out[i] is the stored value
// (as double) of cell i.  half != 0 rounds to FP16.
void dev_round(int half, float f, float d, int n, unsigned step, double* out) {
  const unsigned key = step_key(step, kSaltForward);
  for (int i = 0; i < n; ++i) {
    Dither rnd((unsigned)i, key);
    out[i] = half ? (double)__half2float(Round<__half>::apply(f, d, rnd))
                  : (double)Round<float>::apply(f, d, rnd);
  }
}
// The D3Q19 moment table (15 x 19 rows M, norms N) and the factored pair
// forms computed from it: dev_mrt3d_moments gives rho, jx, jy, jz and the 15
// rows of f; dev_mrt3d_back gives, for relaxed moments r, d0 then E_d and O_d
// for d = 1..9 (19 values).
void dev_mrt3d_table(int* M, int* N) {
  for (int k = 0; k < 15; ++k) {
    N[k] = mrt3d_n(k);
    for (int i = 0; i < 19; ++i) M[k * 19 + i] = mrt3d_m(k, i);
  }
}
void dev_mrt3d_moments(const double* f, double* out) {
  double s[10], a[10], rho, jx, jy, jz;
  for (int d = 1; d <= 9; ++d) {
    s[d] = f[d] + f[d + 9];
    a[d] = f[d] - f[d + 9];
  }
  mrt3d_pair_moments(f, s, a, rho, jx, jy, jz, out + 4);
  out[0] = rho;
  out[1] = jx;
  out[2] = jy;
  out[3] = jz;
}
void dev_mrt3d_back(const double* r, double* out) {
  const Mrt3dEvenBack<double> eb(r);
  out[0] = eb.d0;
  static_for<9>([&](auto D) {
    constexpr int d = decltype(D)::value + 1;
    out[d] = eb.template E<d>();
    out[d + 9] = mrt3d_odd_back<d>(r);
  });
}
// The porosity interpolation BP_q(s) and its derivative in FP32 (fp32 != 0)
// or FP64: out[0] = BP, out[1] = BP'.
void dev_bp(int fp32, double s, double q, double* out) {
  if (fp32) {
    out[0] = (double)bp<float>((float)s, (float)q);
    out[1] = (double)bp_diff<float>((float)s, (float)q);
  } else {
    out[0] = bp<double>(s, q);
    out[1] = bp_diff<double>(s, q);
  }
}
// batch_div(n, d, batch_div_magic(d, nmax)) for the batch layout.
unsigned dev_batch_div(unsigned n, unsigned d, unsigned long long nmax) {
  return batch_div(n, d, batch_div_magic(d, nmax));
}
unsigned dev_batch_div_magic(unsigned long long d, unsigned long long nmax) {
  return batch_div_magic(d, nmax);
}
// Transposed even rows for moment adjoints m: G_0, then G_d for d = 1..9.
void dev_mrt3d_rows_t(const double* m, double* out) {
  const Mrt3dEvenRowsT<double> gt(m);
  out[0] = gt.g0;
  static_for<9>([&](auto D) {
    constexpr int d = decltype(D)::value + 1;
    out[d] = gt.template G<d>();
  });
}
// Round<S>::apply_pair of (f, d) twice per cell for n cells (S = __half when
// half != 0, else float): out[2i] and out[2i+1] are the two stored values of
// cell i.
void dev_round_pair(int half, float f, float d, int n, unsigned step, double* out) {
  const unsigned key = step_key(step, kSaltForward);
  for (int i = 0; i < n; ++i) {
    Dither rnd((unsigned)i, key);
    if (half) {
      __half a, b;
      Round<__half>::apply_pair(f, f, d, d, rnd, a, b);
      out[2 * i] = (double)__half2float(a);
      out[2 * i + 1] = (double)__half2float(b);
    } else {
      float a, b;
      Round<float>::apply_pair(f, f, d, d, rnd, a, b);
      out[2 * i] = (double)a;
      out[2 * i + 1] = (double)b;
    }
  }
}
int dev_collide(const lbm_config* c, int fp32, const double* fin, double g, double* fout) {
  return fp32 ? dispatch_collide<float>(c, fin, g, fout) : dispatch_collide<double>(c, fin, g, fout);
}
int dev_reverse(const lbm_config* c, int fp32, const double* fin, double g, const double* lo,
                double* li, double* dg) {
  return fp32 ? dispatch_reverse<float>(c, fin, g, lo, li, dg)
              : dispatch_reverse<double>(c, fin, g, lo, li, dg);
}
}
