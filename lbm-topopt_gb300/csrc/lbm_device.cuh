// lbm_device.cuh -- device-side building blocks of the GB300 LBM kernels:
// lattices, storage precision traits, collision operators and their
// transposes, boundary conditions and their transposes, objectives.
//
// Populations live in HBM as SoA planes f[q*P + c], c = (z*ny + y)*nx + x
// (x fastest), one plane per direction, P = padded cell count.  FP64 storage
// holds f; FP32/FP16 storage holds the deviation f - w_q of the flow
// populations (temperature populations are stored unshifted), and all
// formulas then run on the deviation with rho replaced by rho - 1, which is
// exact for the incompressible equilibrium feq_i = w_i (rho + ...).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/lbmgpu.h"

namespace lbm {

enum { LAT_D2Q9 = 0, LAT_D3Q19 = 1, LAT_D2Q9_D2Q5 = 2 };

// Compile-time loop: calls f(std::integral_constant<int, I>) for I = 0..N-1,
// so that lattice tables and moment coefficients are constant expressions in
// the body (folded into immediates; register arrays indexed statically).
template <class F, int... Is>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, Is...>) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

// ---------------------------------------------------------------------------
// Lattices (latticeBoltzmann/lattices2d.hh:16-62, lattices3d.hh:141-160).  The
// thermal lattice appends D2Q5 as directions 9..13.

template <int LAT>
struct Lattice;

template <>
struct Lattice<LAT_D2Q9> {
  static constexpr int Q = 9, QF = 9, HALF = 4, DIM = 2, NMAC = 3;
  __host__ __device__ static constexpr int ex(int i) {
    constexpr int v[9] = {0, 1, 0, -1, -1, -1, 0, 1, 1};
    return v[i];
  }
  __host__ __device__ static constexpr int ey(int i) {
    constexpr int v[9] = {0, -1, -1, -1, 0, 1, 1, 1, 0};
    return v[i];
  }
  __host__ __device__ static constexpr int ez(int) { return 0; }
  __host__ __device__ static constexpr int opp(int i) {
    constexpr int v[9] = {0, 5, 6, 7, 8, 1, 2, 3, 4};
    return v[i];
  }
  __host__ __device__ static constexpr double w(int i) {
    constexpr double v[9] = {4. / 9., 1. / 36., 1. / 9., 1. / 36., 1. / 9.,
                             1. / 36., 1. / 9., 1. / 36., 1. / 9.};
    return v[i];
  }
};

template <>
struct Lattice<LAT_D3Q19> {
  static constexpr int Q = 19, QF = 19, HALF = 9, DIM = 3, NMAC = 4;
  __host__ __device__ static constexpr int ex(int i) {
    constexpr int v[19] = {0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1};
    return v[i];
  }
  __host__ __device__ static constexpr int ey(int i) {
    constexpr int v[19] = {0, 0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 1, 0, 1, -1, 0, 0, 1, 1};
    return v[i];
  }
  __host__ __device__ static constexpr int ez(int i) {
    constexpr int v[19] = {0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0};
    return v[i];
  }
  __host__ __device__ static constexpr int opp(int i) {
    constexpr int v[19] = {0, 10, 11, 12, 13, 14, 15, 16, 17, 18, 1, 2, 3, 4, 5, 6, 7, 8, 9};
    return v[i];
  }
  __host__ __device__ static constexpr double w(int i) {
    constexpr double v[19] = {1. / 3.,  1. / 18., 1. / 18., 1. / 18., 1. / 36., 1. / 36., 1. / 36.,
                              1. / 36., 1. / 36., 1. / 36., 1. / 18., 1. / 18., 1. / 18., 1. / 36.,
                              1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};
    return v[i];
  }
};

template <>
struct Lattice<LAT_D2Q9_D2Q5> {
  static constexpr int Q = 14, QF = 9, HALF = 4, DIM = 2, NMAC = 4;
  __host__ __device__ static constexpr int ex(int i) {
    constexpr int v[14] = {0, 1, 0, -1, -1, -1, 0, 1, 1, 0, 0, -1, 0, 1};
    return v[i];
  }
  __host__ __device__ static constexpr int ey(int i) {
    constexpr int v[14] = {0, -1, -1, -1, 0, 1, 1, 1, 0, 0, -1, 0, 1, 0};
    return v[i];
  }
  __host__ __device__ static constexpr int ez(int) { return 0; }
  __host__ __device__ static constexpr int opp(int i) {
    constexpr int v[14] = {0, 5, 6, 7, 8, 1, 2, 3, 4, 9, 12, 13, 10, 11};
    return v[i];
  }
  __host__ __device__ static constexpr double w(int i) {
    constexpr double v[14] = {4. / 9., 1. / 36., 1. / 9., 1. / 36., 1. / 9., 1. / 36., 1. / 9.,
                              1. / 36., 1. / 9., 1. / 3., 1. / 6., 1. / 6., 1. / 6., 1. / 6.};
    return v[i];
  }
};

// ---------------------------------------------------------------------------
// Storage precision.

template <class S>
struct Store;

template <>
struct Store<double> {
  using C = double;   // compute type
  static constexpr bool SHIFT = false;
  __device__ static C ld(const double* p) { return *p; }
  __device__ static void st(double* p, C v) { *p = v; }
};

template <>
struct Store<float> {
  using C = float;
  static constexpr bool SHIFT = true;
  // Plain cached accesses: on GB300 the evict-first (.cs) forms of these
  // loads and stores cut a 19-plane streaming copy from 6.5 to 4.0 TB/s.
  __device__ static C ld(const float* p) { return *p; }
  __device__ static void st(float* p, C v) { *p = v; }
};

template <>
struct Store<__half> {
  using C = float;
  static constexpr bool SHIFT = true;
  __device__ static C ld(const __half* p) { return __half2float(*p); }
  __device__ static void st(__half* p, C v) { *p = __float2half_rn(v); }
};

// Design field storage: FP64 next to FP64 populations, FP32 otherwise.
template <class S>
struct GammaT {
  using T = float;
};
template <>
struct GammaT<double> {
  using T = double;
};

// ---------------------------------------------------------------------------
// Launch parameters.

struct DevBC {
  int kind, face, profile;
  int box[6];
  int tang_x;         // 1: box cells ordered along x (south/north faces); 0: along y, then z
  int n_t;            // box cells along the first tangential axis
  int ncomp;          // table entries per cell: 0 (no table), 1 (factor), 2 or 3 (velocity vector)
  double value;       // value * T(t) at this launch's time t
  float value_f;      // the same in FP32
  double vshift;      // value - 1 (pressure on shifted populations)
  float vshift_f;
  double dir[3];      // velocity direction
  float dir_f[3];
  const double* prof;   // factor (or vector) table of this launch's time step over the box; null = 1
  const float* prof_f;
};

template <class C>
__device__ __forceinline__ C bc_value(const DevBC& b);
template <>
__device__ __forceinline__ double bc_value<double>(const DevBC& b) { return b.value; }
template <>
__device__ __forceinline__ float bc_value<float>(const DevBC& b) { return b.value_f; }
template <class C>
__device__ __forceinline__ C bc_vshift(const DevBC& b);
template <>
__device__ __forceinline__ double bc_vshift<double>(const DevBC& b) { return b.vshift; }
template <>
__device__ __forceinline__ float bc_vshift<float>(const DevBC& b) { return b.vshift_f; }
template <class C>
__device__ __forceinline__ const C* bc_table(const DevBC& b);
template <>
__device__ __forceinline__ const double* bc_table<double>(const DevBC& b) { return b.prof; }
template <>
__device__ __forceinline__ const float* bc_table<float>(const DevBC& b) { return b.prof_f; }
template <class C>
__device__ __forceinline__ C bc_dir(const DevBC& b, int a);
template <>
__device__ __forceinline__ double bc_dir<double>(const DevBC& b, int a) { return b.dir[a]; }
template <>
__device__ __forceinline__ float bc_dir<float>(const DevBC& b, int a) { return b.dir_f[a]; }

// Index of cell (x,y,z) among the box cells, in the order of the tables.
__device__ __forceinline__ int bc_index(const DevBC& b, int x, int y, int z) {
  return b.tang_x ? (x - b.box[0]) : ((z - b.box[4]) * b.n_t + (y - b.box[2]));
}

// Scalar value of a pressure or temperature boundary at a cell: value(t),
// times the tabulated factor if there is one.
template <class C>
__device__ __forceinline__ C bc_scalar(const DevBC& b, int x, int y, int z) {
  C v = bc_value<C>(b);
  const C* t = bc_table<C>(b);
  if (t) v *= t[bc_index(b, x, y, z)];
  return v;
}

// Prescribed velocity at a cell: value(t) * profile * dir, or the tabulated
// vector (the reference's Input functor, ZouHe2d.hh:37).
template <class C>
__device__ __forceinline__ void bc_velocity(const DevBC& b, int x, int y, int z, C& ux, C& uy,
                                            C& uz) {
  const C* t = bc_table<C>(b);
  const int i = bc_index(b, x, y, z);
  if (b.ncomp >= 2) {
    ux = t[i * b.ncomp];
    uy = t[i * b.ncomp + 1];
    uz = b.ncomp == 3 ? t[i * b.ncomp + 2] : C(0.);
    return;
  }
  C s = bc_value<C>(b);
  if (t) s *= t[i];
  ux = s * bc_dir<C>(b, 0);
  uy = s * bc_dir<C>(b, 1);
  uz = s * bc_dir<C>(b, 2);
}

// Model constants in one precision.  KParams carries an FP64 and an FP32 copy
// so that FP32 kernels never convert FP64 launch parameters per thread (GB300
// runs FP64 on a narrow pipe).
template <class C>
struct ModelParams {
  C omega;
  C mrt[8];
  C pbb_scale, pbb_q;
  C diff, ramp_q, ramp_ck, heat_rate, heat_T;
  C obj_weight, w_in, w_out;   // w_in = inv_in*obj_weight, w_out = inv_out*obj_weight
  C cv_diss;                   // (9/2) nu omega^2 of the dissipation objective
  C obj_p[2];                  // objective parameters (regenerator efficiency: Ti, w/D)
};

struct KParams {
  int nx, ny, nz;
  long long P;       // plane stride in elements
  unsigned step;     // time step of the input state
  unsigned key_fwd, key_adj;   // rounding-stream keys of the two step kernels at this step
  // model
  double omega;
  double mrt[8];
  double pbb_scale, pbb_q;
  double diff, ramp_q, ramp_ck, heat_rate, heat_T;
  ModelParams<double> md;
  ModelParams<float> mf;
  // boundary conditions of the input state's time step
  int nbc;
  int apply_bc;
  int bc_y;                // some boundary lies on a south or north face
  DevBC bc[LBM_MAX_BC];
  // objective
  int objective;
  int eval_obj;
  int accumulate;          // add each block's sum to partial[block] (no counter, no result)
  double obj_weight, inv_in, inv_out;
  int obj_in[6], obj_out[6];
  double* partial;         // partial sums: per block (one step) or per warp (summed over steps)
  unsigned int* counter;   // last-block-done counter (reset by the last block)
  double* result;          // J of this step (written by the last block)
  // buffers
  const void* fin;
  void* fout;
  const void* gamma;
  const void* lam_in;      // eta_{t+1}
  void* lam_out;           // eta_t
  double* sens;
  int sens_atomic;         // add to dJ/dgamma with an atomic (reverse steps that fit in L2)
};

template <class C>
__device__ __forceinline__ const ModelParams<C>& mp(const KParams& p);
template <>
__device__ __forceinline__ const ModelParams<double>& mp<double>(const KParams& p) {
  return p.md;
}
template <>
__device__ __forceinline__ const ModelParams<float>& mp<float>(const KParams& p) {
  return p.mf;
}

__host__ __device__ inline bool in_box(const int* b, int x, int y, int z) {
  return x >= b[0] && x <= b[1] && y >= b[2] && y <= b[3] && z >= b[4] && z <= b[5];
}

// ---------------------------------------------------------------------------
// Interpolations (core/interpolationFunctions.hh:17-54).

// a / b for the FP32 interpolations: the fast division on the GPU (about 2
// units in the last place for the denominators here, q + s in [q, q + 1]).
__device__ __forceinline__ float interp_div(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

// BPInterpolation (core/interpolationFunctions.hh:18-25).  FP64 evaluates the
// reference's expressions; FP32 the algebraically equal q(1-s)/(q+s) and
// -q(1+q)/(q+s)^2 with the fast division, which are exactly 0 in fluid cells
// (s = 1) whatever the division's rounding: 1 - s(1+q)/(q+s) is 0 there only
// if the quotient rounds to exactly 1.
template <class C>
__device__ __forceinline__ C bp(C s, C q) {
  if constexpr (sizeof(C) == 4)
    return interp_div(q * (C(1.) - s), q + s);
  else
    return C(1.) - s * (C(1.) + q) / (q + s);
}
template <class C>
__device__ __forceinline__ C bp_diff(C s, C q) {
  if constexpr (sizeof(C) == 4) {
    const C r = interp_div(C(1.), q + s);
    return -(q * (C(1.) + q)) * (r * r);
  } else {
    return (-(C(1.) + q) / (q + s) + s * (C(1.) + q) / ((q + s) * (q + s)));
  }
}
template <class C>
__device__ __forceinline__ C ramp(C s, C q, C ck) {
  return (s * (ck * (C(1.) + q) - C(1.)) + C(1.)) / (ck * (C(1.) + q * s));
}
template <class C>
__device__ __forceinline__ C ramp_diff(C s, C q, C ck) {
  return (ck * (C(1.) + q) - C(1.)) / (ck * (C(1.) + q * s)) -
         ((s * (ck * (C(1.) + q) - C(1.)) + C(1.)) * q) / (ck * (C(1.) + q * s) * (C(1.) + q * s));
}

// ---------------------------------------------------------------------------
// Macros (incompressible: u = j).  D2Q9 keeps the grouping of
// IncompressibleMacros2d<D2Q9> (dynamics/isothermalMacros2d.hh:199-208).

template <class C>
__device__ __forceinline__ void macros_d2q9(const C* f, C& rho, C& jx, C& jy) {
  C ux = f[1] + f[7] + f[8];
  C uy = f[5] + f[6] + f[7];
  rho = ux + uy - f[7] + f[0] + f[2] + f[3] + f[4];
  ux -= f[3] + f[4] + f[5];
  uy -= f[1] + f[2] + f[3];
  jx = ux;
  jy = uy;
}

template <int LAT, class C>
__device__ __forceinline__ void flow_macros(const C* f, C& rho, C& jx, C& jy, C& jz) {
  using L = Lattice<LAT>;
  if (L::DIM == 2) {
    macros_d2q9(f, rho, jx, jy);
    jz = C(0.);
  } else {
    rho = C(0.);
    jx = C(0.);
    jy = C(0.);
    jz = C(0.);
    static_for<L::QF>([&](auto I) {
      constexpr int i = decltype(I)::value;
      rho += f[i];
      if constexpr (L::ex(i) == 1) jx += f[i];
      if constexpr (L::ex(i) == -1) jx -= f[i];
      if constexpr (L::ey(i) == 1) jy += f[i];
      if constexpr (L::ey(i) == -1) jy -= f[i];
      if constexpr (L::ez(i) == 1) jz += f[i];
      if constexpr (L::ez(i) == -1) jz -= f[i];
    });
  }
}

// sum_a e_ia j_a with the zero terms left out
template <int LAT, int i, class C>
__device__ __forceinline__ C e_dot(C jx, C jy, C jz) {
  using L = Lattice<LAT>;
  C v = C(0.);
  if constexpr (L::ex(i) == 1) v += jx;
  if constexpr (L::ex(i) == -1) v -= jx;
  if constexpr (L::ey(i) == 1) v += jy;
  if constexpr (L::ey(i) == -1) v -= jy;
  if constexpr (L::ez(i) == 1) v += jz;
  if constexpr (L::ez(i) == -1) v -= jz;
  return v;
}

// ---------------------------------------------------------------------------
// MRT moment bases: rows of the non-conserved moments.
// D2Q9: dynamics/incompressibleMRT2d.hh:50-60.  D3Q19: dynamics/MRT3d.hh:50-90.

__host__ __device__ constexpr int mrt2d_m(int k, int i) {
  constexpr int M[6][9] = {{-4, 2, -1, 2, -1, 2, -1, 2, -1}, {4, 1, -2, 1, -2, 1, -2, 1, -2},
                           {0, 1, 0, -1, 2, -1, 0, 1, -2},   {0, -1, 2, -1, 0, 1, -2, 1, 0},
                           {0, 0, -1, 0, 1, 0, -1, 0, 1},    {0, -1, 0, 1, 0, -1, 0, 1, 0}};
  return M[k][i];
}
__host__ __device__ constexpr int mrt2d_n(int k) {
  constexpr int N[6] = {36, 36, 12, 12, 4, 4};
  return N[k];
}

__host__ __device__ constexpr int mrt3d_m(int k, int i) {
  constexpr int M[15][19] = {
      {-30, -11, -11, -11, 8, 8, 8, 8, 8, 8, -11, -11, -11, 8, 8, 8, 8, 8, 8},
      {12, -4, -4, -4, 1, 1, 1, 1, 1, 1, -4, -4, -4, 1, 1, 1, 1, 1, 1},
      {0, 0, 0, 4, 0, 0, -1, 1, -1, 1, 0, 0, -4, 0, 0, 1, -1, 1, -1},
      {0, 0, 4, 0, -1, 1, 0, 0, -1, -1, 0, -4, 0, 1, -1, 0, 0, 1, 1},
      {0, 4, 0, 0, -1, -1, -1, -1, 0, 0, -4, 0, 0, 1, 1, 1, 1, 0, 0},
      {0, -1, -1, 2, -2, -2, 1, 1, 1, 1, -1, -1, 2, -2, -2, 1, 1, 1, 1},
      {0, 2, 2, -4, -2, -2, 1, 1, 1, 1, 2, 2, -4, -2, -2, 1, 1, 1, 1},
      {0, -1, 1, 0, 0, 0, -1, -1, 1, 1, -1, 1, 0, 0, 0, -1, -1, 1, 1},
      {0, 2, -2, 0, 0, 0, -1, -1, 1, 1, 2, -2, 0, 0, 0, -1, -1, 1, 1},
      {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 0, 0, 0, 1, -1},
      {0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0},
      {0, 0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 0, 0, 0, 1, -1, 0, 0},
      {0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 0, -1, 1, 1, -1},
      {0, 0, 0, 0, -1, 1, 0, 0, 1, 1, 0, 0, 0, 1, -1, 0, 0, -1, -1},
      {0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, -1, -1, 1, 1, 0, 0}};
  return M[k][i];
}
__host__ __device__ constexpr int mrt3d_n(int k) {
  constexpr int N[15] = {2394, 252, 40, 40, 40, 36, 72, 12, 24, 4, 4, 4, 8, 8, 8};
  return N[k];
}

template <int DIM>
struct MRT {
  static constexpr int K = (DIM == 2) ? 6 : 15;
  static constexpr int QF = (DIM == 2) ? 9 : 19;
  __host__ __device__ static constexpr int m(int k, int i) {
    return DIM == 2 ? mrt2d_m(k, i) : mrt3d_m(k, i);
  }
  __host__ __device__ static constexpr int n(int k) { return DIM == 2 ? mrt2d_n(k) : mrt3d_n(k); }
};

// sum_i M[k][i] f_i, left to right over the nonzero entries of the constant
// row (0 + first term is exact, so this is the reference's expression).
template <int DIM, int K, class C>
__device__ __forceinline__ C mrt_moment(const C* f) {
  using M = MRT<DIM>;
  C s = C(0.);
  static_for<M::QF>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int c = M::m(K, i);
    if constexpr (c == 1) {
      s = s + f[i];
    } else if constexpr (c == -1) {
      s = s - f[i];
    } else if constexpr (c != 0) {
      s = s + C(c) * f[i];
    }
  });
  return s;
}

template <int DIM, class C>
__device__ __forceinline__ void mrt_moments(const C* f, C* mo) {
  static_for<MRT<DIM>::K>([&](auto KK) {
    constexpr int k = decltype(KK)::value;
    mo[k] = mrt_moment<DIM, k>(f);
  });
}

// Relaxation r_k = s_k (m_k - meq_k) written as the reference does
// (incompressibleMRT2d.hh:62-67, MRT3d.hh:92-109).  rho is the "rho-like"
// value (rho, or rho - 1 for shifted storage).
template <class C>
__device__ __forceinline__ void mrt2d_relax(C* mo, C rho, C jx, C jy, const KParams& p) {
  const C s1 = mp<C>(p).mrt[0], s2 = mp<C>(p).mrt[1], s46 = mp<C>(p).mrt[2], om = mp<C>(p).omega;
  C uSqr = jx * jx + jy * jy;
  mo[0] = s1 * (mo[0] + C(2.) * rho - C(3.) * uSqr);
  mo[1] = s2 * (mo[1] - rho + C(3.) * uSqr);
  mo[2] = s46 * (mo[2] + jx);
  mo[3] = s46 * (mo[3] + jy);
  mo[4] = om * (mo[4] - jx * jx + jy * jy);
  mo[5] = om * (mo[5] - jx * jy);
}

template <class C>
__device__ __forceinline__ void mrt3d_relax(C* mo, C rho, C jx, C jy, C jz, const KParams& p) {
  const C s1 = mp<C>(p).mrt[0], s2 = mp<C>(p).mrt[1], s4 = mp<C>(p).mrt[2], s10 = mp<C>(p).mrt[3],
          s16 = mp<C>(p).mrt[4], we = mp<C>(p).mrt[5], wej = mp<C>(p).mrt[6], wxx = mp<C>(p).mrt[7],
          om = mp<C>(p).omega;
  C jSqr = jx * jx + jy * jy + jz * jz;
  mo[0] = s1 * (mo[0] + C(11.) * rho - C(19.) * jSqr);
  mo[1] = s2 * (mo[1] - we * rho - wej * jSqr);
  mo[2] = s4 * (mo[2] + C(2. / 3.) * jx);
  mo[3] = s4 * (mo[3] + C(2. / 3.) * jy);
  mo[4] = s4 * (mo[4] + C(2. / 3.) * jz);
  C tempEq = (C(2.) * jx * jx - (jy * jy + jz * jz));
  mo[5] = om * (mo[5] - tempEq);
  mo[6] = s10 * (mo[6] - wxx * tempEq);
  tempEq = (jy * jy - jz * jz);
  mo[7] = om * (mo[7] - tempEq);
  mo[8] = s10 * (mo[8] - wxx * tempEq);
  mo[9] = om * (mo[9] - jx * jy);
  mo[10] = om * (mo[10] - jy * jz);
  mo[11] = om * (mo[11] - jx * jz);
  mo[12] *= s16;
  mo[13] *= s16;
  mo[14] *= s16;
}

// f_out_i = f_i - sum_k (M[k][i]/N_k) r_k, in k order, coefficients folded at
// compile time.
template <int DIM, class C>
__device__ __forceinline__ void mrt_backmap(C* f, const C* mo) {
  using M = MRT<DIM>;
  static_for<M::QF>([&](auto I) {
    constexpr int i = decltype(I)::value;
    C v = f[i];
    static_for<M::K>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      constexpr int c = M::m(k, i);
      if constexpr (c != 0) {
        constexpr double b = -(double)c / (double)M::n(k);
        v = v + C(b) * mo[k];
      }
    });
    f[i] = v;
  });
}

// ---------------------------------------------------------------------------
// D3Q19 MRT + partial bounce-back in population-pair form.  With
// s_d = f_d + f_{d+9} and a_d = f_d - f_{d+9} (d = 1..9, opp(d) = d+9), the
// even moments (e, eps, p, pi; MRT3d.hh:50-90 rows 0,1,5-11) are sums over f_0
// and s_d, the odd ones (q, m; rows 2-4, 12-14) sums over a_d, and the
// back-map f_i - sum_k (M[k][i]/N_k) r_k splits the same way.  Partial
// bounce-back (partialBouncebackCollision.hh:53-65) leaves s_d unchanged and
// scales a_d by (1 - 2 imult).  Same operator as the reference, about half the
// arithmetic.

// Row k is even (f_d and f_opp(d) weighted alike) or odd (opposite weights);
// every row of the D3Q19 basis is one or the other.
__host__ __device__ constexpr bool mrt3d_even(int k) {
  for (int d = 1; d <= 9; ++d)
    if (mrt3d_m(k, d) != mrt3d_m(k, d + 9)) return false;
  return true;
}
__host__ __device__ constexpr bool mrt3d_odd(int k) {
  if (mrt3d_m(k, 0) != 0) return false;
  for (int d = 1; d <= 9; ++d)
    if (mrt3d_m(k, d) != -mrt3d_m(k, d + 9)) return false;
  return true;
}
static_assert(mrt3d_even(0) && mrt3d_even(1) && mrt3d_odd(2) && mrt3d_odd(3) && mrt3d_odd(4) &&
                  mrt3d_even(5) && mrt3d_even(11) && mrt3d_odd(12) && mrt3d_odd(14),
              "D3Q19 moment rows must split into even and odd rows");

// d(meq_k)/d(rho) and d(meq_k)/d(j_a) of MRT3d.hh:92-109 are applied inline below.

// rho, j and the 15 moment rows of the populations (f0, s_d, a_d) in pair form.
template <class C>
__device__ __forceinline__ void mrt3d_pair_rows(C f0, const C* s, const C* a, C& rho, C& jx, C& jy,
                                                C& jz, C* mo) {
  using L = Lattice<LAT_D3Q19>;
  // The rows share sub-sums (pair d: 1-3 the z, y, x axes, 4-5 the yz, 6-7
  // the xz and 8-9 the xy diagonals); the identities are checked row by row
  // against the moment table by tests/device_math_host.cpp.
  static_assert(L::ez(1) == -1 && L::ey(2) == -1 && L::ex(3) == -1 && L::ey(4) == -1 &&
                    L::ez(4) == -1 && L::ey(5) == 1 && L::ex(6) == -1 && L::ex(7) == 1 &&
                    L::ey(8) == -1 && L::ex(9) == 1 && L::ey(9) == -1,
                "pair order of the factored D3Q19 moments");
  // even rows: e, eps, 3pxx, 3pixx, pww, piww, pxy, pyz, pxz
  const C sax = (s[1] + s[2]) + s[3];
  const C dyz = s[4] + s[5], dxz = s[6] + s[7], dxy = s[8] + s[9];
  const C sdg = (dyz + dxz) + dxy;
  rho = (f0 + sax) + sdg;
  mo[0] = C(8.) * sdg - (C(30.) * f0 + C(11.) * sax);
  mo[1] = (C(12.) * f0 + sdg) - C(4.) * sax;
  const C A = C(2.) * s[3] - (s[1] + s[2]), B = (dxz + dxy) - C(2.) * dyz;
  mo[5] = A + B;
  mo[6] = B - C(2.) * A;
  const C A2 = s[2] - s[1], B2 = dxy - dxz;
  mo[7] = A2 + B2;
  mo[8] = B2 - C(2.) * A2;
  mo[9] = s[8] - s[9];
  mo[10] = s[4] - s[5];
  mo[11] = s[6] - s[7];
  // odd rows: j and q (x, y, z), m (x, y, z)
  const C ux = a[9] - a[8], vx = a[7] - a[6], X = ux + vx;
  jx = X - a[3];
  mo[2] = X + C(4.) * a[3];
  mo[12] = ux - vx;
  const C py = a[5] - a[4], qy = a[8] + a[9], Y = py - qy;
  jy = Y - a[2];
  mo[3] = Y + C(4.) * a[2];
  mo[13] = py + qy;
  const C rz = a[4] + a[5], tz = a[6] + a[7], Z = rz + tz;
  jz = -(Z + a[1]);
  mo[4] = C(4.) * a[1] - Z;
  mo[14] = rz - tz;
}

template <class C>
__device__ __forceinline__ void mrt3d_pair_moments(const C* f, C* s, C* a, C& rho, C& jx, C& jy,
                                                   C& jz, C* mo) {
  static_for<9>([&](auto D) {
    constexpr int d = decltype(D)::value + 1;
    s[d] = f[d] + f[d + 9];
    a[d] = f[d] - f[d + 9];
  });
  mrt3d_pair_rows(f[0], s, a, rho, jx, jy, jz, mo);
}

// Even part of the back-map of the relaxed moments r (mo after mrt3d_relax):
// d0 = -sum_k (M[k][0]/N_k) r_k for the rest population and
// E_d = -2 sum_even k (M[k][d]/N_k) r_k for pair d, from nine shared terms.
template <class C>
struct Mrt3dEvenBack {
  C d0, ax12, R, e3, c45, h10, c67, h11, c89, h9;
  __device__ __forceinline__ explicit Mrt3dEvenBack(const C* mo) {
    d0 = C(30. / 2394.) * mo[0] - C(12. / 252.) * mo[1];
    const C cax = C(22. / 2394.) * mo[0] + C(8. / 252.) * mo[1];
    const C cdg = C(-16. / 2394.) * mo[0] - C(2. / 252.) * mo[1];
    const C P = C(1. / 18.) * (mo[5] - mo[6]);
    const C Q = C(1. / 18.) * mo[5] + C(1. / 36.) * mo[6];
    R = C(1. / 6.) * (mo[7] - mo[8]);
    const C T = C(1. / 6.) * mo[7] + C(1. / 12.) * mo[8];
    ax12 = cax + P;
    e3 = cax - C(2.) * P;
    c45 = cdg + C(2.) * Q;
    const C cq = cdg - Q;
    c67 = cq + T;
    c89 = cq - T;
    h9 = C(0.5) * mo[9];
    h10 = C(0.5) * mo[10];
    h11 = C(0.5) * mo[11];
  }
  template <int d>
  __device__ __forceinline__ C E() const {
    if constexpr (d == 1) return ax12 + R;
    if constexpr (d == 2) return ax12 - R;
    if constexpr (d == 3) return e3;
    if constexpr (d == 4) return c45 - h10;
    if constexpr (d == 5) return c45 + h10;
    if constexpr (d == 6) return c67 - h11;
    if constexpr (d == 7) return c67 + h11;
    if constexpr (d == 8) return c89 - h9;
    if constexpr (d == 9) return c89 + h9;
  }
};

// Transpose of the even rows: G_0 = sum_k M[k][0] m_k and, for pair d,
// G_d = sum_even k M[k][d] m_k (the same sub-sums as Mrt3dEvenBack).
template <class C>
struct Mrt3dEvenRowsT {
  C g0, ax12, R, g3, c45, m10, c67, m11, c89, m9;
  __device__ __forceinline__ explicit Mrt3dEvenRowsT(const C* m) {
    g0 = C(12.) * m[1] - C(30.) * m[0];
    const C cax = C(-11.) * m[0] - C(4.) * m[1];
    const C cdg = C(8.) * m[0] + m[1];
    const C P = m[5] - C(2.) * m[6], Q = m[5] + m[6];
    R = m[7] - C(2.) * m[8];
    const C T = m[7] + m[8];
    ax12 = cax - P;
    g3 = cax + C(2.) * P;
    c45 = cdg - C(2.) * Q;
    const C cq = cdg + Q;
    c67 = cq - T;
    c89 = cq + T;
    m9 = m[9];
    m10 = m[10];
    m11 = m[11];
  }
  template <int d>
  __device__ __forceinline__ C G() const {
    if constexpr (d == 1) return ax12 - R;
    if constexpr (d == 2) return ax12 + R;
    if constexpr (d == 3) return g3;
    if constexpr (d == 4) return c45 + m10;
    if constexpr (d == 5) return c45 - m10;
    if constexpr (d == 6) return c67 + m11;
    if constexpr (d == 7) return c67 - m11;
    if constexpr (d == 8) return c89 + m9;
    if constexpr (d == 9) return c89 - m9;
  }
};

// Odd part of the back-map: O_d = -2 sum_odd k (M[k][d]/N_k) r_k.
template <int d, class C>
__device__ __forceinline__ C mrt3d_odd_back(const C* mo) {
  C O = C(0.);
  static_for<15>([&](auto KK) {
    constexpr int k = decltype(KK)::value;
    constexpr int c = mrt3d_m(k, d);
    if constexpr (mrt3d_odd(k) && c != 0) {
      constexpr double b = -2.0 * (double)c / (double)mrt3d_n(k);
      O += C(b) * mo[k];
    }
  });
  return O;
}

// In place: f <- PBB(MRT(f)); returns the macros of the input.
template <class C>
__device__ __forceinline__ void mrt3d_pair_collide(C* f, C imult, C& rho, C& jx, C& jy, C& jz,
                                                   const KParams& p) {
  C s[10], a[10], mo[15];
  mrt3d_pair_moments(f, s, a, rho, jx, jy, jz, mo);
  mrt3d_relax(mo, rho, jx, jy, jz, p);
  // rest population: f_0 - sum_even (M[k][0]/N_k) r_k
  const Mrt3dEvenBack<C> eb(mo);
  f[0] += eb.d0;
  const C keep = C(1.) - C(2.) * imult;
  static_for<9>([&](auto D) {
    constexpr int d = decltype(D)::value + 1;
    const C sp = s[d] + eb.template E<d>();
    const C ap = (a[d] + mrt3d_odd_back<d>(mo)) * keep;
    f[d] = C(0.5) * (sp + ap);
    f[d + 9] = C(0.5) * (sp - ap);
  });
}

// Transpose of mrt3d_pair_collide at input fin: lam (adjoint of the output)
// in, adjoint of the input out; dg += dimult * d(out)/d(imult)^T lam.
template <class C>
__device__ __forceinline__ void mrt3d_pair_reverse(const C* fin, C* lam, C imult, C dimult, C& dg,
                                                   const KParams& p) {
  C s[10], a[10], mo[15];
  C rho, jx, jy, jz;
  mrt3d_pair_moments(fin, s, a, rho, jx, jy, jz, mo);
  mrt3d_relax(mo, rho, jx, jy, jz, p);
  // adjoints of s' and a'' from the output pairs, kept doubled:
  // ls_d = 2 sbar'_d, la_d = 2 abar'_d; imult adjoint from a' = a + O
  const C keep = C(1.) - C(2.) * imult;
  C ls[10], la[10];
  C imultRev = C(0.);
  static_for<9>([&](auto D) {
    constexpr int d = decltype(D)::value + 1;
    const C ap = a[d] + mrt3d_odd_back<d>(mo);  // a' before partial bounce-back
    ls[d] = lam[d] + lam[d + 9];
    const C la2 = lam[d] - lam[d + 9];          // 2 x adjoint of a''
    imultRev -= ap * la2;
    la[d] = keep * la2;
  });
  dg += dimult * imultRev;
  const C f0b = lam[0];
  // adjoint of the relaxed moments: mb_k = rate_k (-1/N_k) (M lam)_k, the
  // rows applied to (f0b, ls, la) in pair form
  C mb[15];
  {
    C r_, x_, y_, z_;
    mrt3d_pair_rows(f0b, ls, la, r_, x_, y_, z_, mb);
  }
  const C* rt = mp<C>(p).mrt;
  const C om = mp<C>(p).omega;
  static_for<15>([&](auto KK) {
    constexpr int k = decltype(KK)::value;
    // rate of moment k (MRT3d.hh:93-109)
    C rate;
    if constexpr (k == 0) rate = rt[0];
    else if constexpr (k == 1) rate = rt[1];
    else if constexpr (k >= 2 && k <= 4) rate = rt[2];
    else if constexpr (k == 6 || k == 8) rate = rt[3];
    else if constexpr (k >= 12) rate = rt[4];
    else rate = om;
    mb[k] = rate * (C(-1.0 / (double)mrt3d_n(k)) * mb[k]);
  });
  // through -meq(rho, j)
  const C we = rt[5], wej = rt[6], wxx = rt[7];
  const C c2 = C(-2. / 3.);
  const C a56 = mb[5] + wxx * mb[6], a78 = mb[7] + wxx * mb[8];
  const C rR = -(mb[0] * C(-11.) + mb[1] * we);
  const C jR0 = -(mb[0] * C(38.) * jx + mb[1] * C(2.) * wej * jx + mb[2] * c2 + a56 * C(4.) * jx +
                  mb[9] * jy + mb[11] * jz);
  const C jR1 = -(mb[0] * C(38.) * jy + mb[1] * C(2.) * wej * jy + mb[3] * c2 - a56 * C(2.) * jy +
                  a78 * C(2.) * jy + mb[9] * jx + mb[10] * jz);
  const C jR2 = -(mb[0] * C(38.) * jz + mb[1] * C(2.) * wej * jz + mb[4] * c2 - a56 * C(2.) * jz -
                  a78 * C(2.) * jz + mb[10] * jy + mb[11] * jx);
  // through m = M(f0, s, a), rho = f0 + sum s, j = sum e a, and the pair split
  const Mrt3dEvenRowsT<C> gt(mb);
  lam[0] = (f0b + rR) + gt.g0;
  using L = Lattice<LAT_D3Q19>;
  static_for<9>([&](auto D) {
    constexpr int d = decltype(D)::value + 1;
    const C sbar = (C(0.5) * ls[d] + rR) + gt.template G<d>();
    C abar = C(0.5) * la[d] + e_dot<LAT_D3Q19, d>(jR0, jR1, jR2);
    static_for<15>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      constexpr int c = mrt3d_m(k, d);
      if constexpr (c != 0 && mrt3d_odd(k)) abar += C(c) * mb[k];
    });
    lam[d] = sbar + abar;
    lam[d + 9] = sbar - abar;
  });
}

// ---------------------------------------------------------------------------
// Forward flow collision in place: f <- PBB(base(f)); returns the macros of
// the input.  IncompressibleBGK2d<D2Q9> (dynamics/incompressibleBGK2d.hh:120-147),
// incompressible BGK on D3Q19 (dynamics/BGK3d.hh), IncompressibleMRT2d/3d,
// PartialBouncebackCollision (dynamics/partialBouncebackCollision.hh:53-65).

template <int LAT, int COLL, class C>
__device__ __forceinline__ void flow_collide(C* f, C imult, C& rho, C& jx, C& jy, C& jz,
                                             const KParams& p) {
  using L = Lattice<LAT>;
  if constexpr (LAT == LAT_D3Q19 && COLL == LBM_MRT) {
    mrt3d_pair_collide(f, imult, rho, jx, jy, jz, p);
    return;
  }
  flow_macros<LAT>(f, rho, jx, jy, jz);
  const C om = mp<C>(p).omega;
  if (COLL == LBM_BGK) {
    if (L::DIM == 2) {
      const C uSqr = jx * jx + jy * jy;
      const C cFeq = rho - C(1.5) * uSqr;
      const C rel = C(1.) - om;
      const C restW = C(4. / 9.), stW = C(1. / 9.), diagW = C(1. / 36.);
      f[0] = rel * f[0] + om * restW * cFeq;
      f[2] = rel * f[2] + om * stW * (cFeq - C(3.) * jy + C(4.5) * jy * jy);
      f[4] = rel * f[4] + om * stW * (cFeq - C(3.) * jx + C(4.5) * jx * jx);
      f[6] = rel * f[6] + om * stW * (cFeq + C(3.) * jy + C(4.5) * jy * jy);
      f[8] = rel * f[8] + om * stW * (cFeq + C(3.) * jx + C(4.5) * jx * jx);
      f[1] = rel * f[1] + om * diagW * (cFeq + C(3.) * (jx - jy) + C(4.5) * (uSqr - C(2.) * jx * jy));
      f[3] = rel * f[3] + om * diagW * (cFeq - C(3.) * (jx + jy) + C(4.5) * (uSqr + C(2.) * jx * jy));
      f[5] = rel * f[5] + om * diagW * (cFeq + C(3.) * (jy - jx) + C(4.5) * (uSqr - C(2.) * jx * jy));
      f[7] = rel * f[7] + om * diagW * (cFeq + C(3.) * (jx + jy) + C(4.5) * (uSqr + C(2.) * jx * jy));
    } else {
      const C uSqr = jx * jx + jy * jy + jz * jz;
      static_for<L::QF>([&](auto I) {
        constexpr int i = decltype(I)::value;
        const C sc = e_dot<LAT, i>(jx, jy, jz);
        C eq = C(L::w(i)) * (rho + C(3.) * sc + C(4.5) * sc * sc - C(1.5) * uSqr);
        f[i] = f[i] * (C(1.) - om) + om * eq;
      });
    }
  } else {
    C mo[MRT<L::DIM>::K];
    mrt_moments<L::DIM>(f, mo);
    if (L::DIM == 2)
      mrt2d_relax(mo, rho, jx, jy, p);
    else
      mrt3d_relax(mo, rho, jx, jy, jz, p);
    mrt_backmap<L::DIM>(f, mo);
  }
#pragma unroll
  for (int d = 1; d <= L::HALF; ++d) {
    C ftemp = f[d];
    f[d] += imult * (f[d + L::HALF] - f[d]);
    f[d + L::HALF] += imult * (ftemp - f[d + L::HALF]);
  }
}

// Transpose of flow_collide: on entry lam = adjoint of the output, on exit
// lam = adjoint of the input; dg += d(out)/d(imult)^T lam * dimult.
// ReversePartialBouncebackCollision (adjointDynamics/reversePartialBounceback.hh:18-41)
// over ReverseIncompressibleBGK2d<D2Q9> (reverseIncompressibleBGK2d.hh:112-169)
// and the transposes of the MRT operators (derived from the forward).
template <int LAT, int COLL, class C>
__device__ __forceinline__ void flow_reverse(const C* fin, C* lam, C imult, C dimult, C& dg,
                                             const KParams& p) {
  using L = Lattice<LAT>;
  if constexpr (LAT == LAT_D3Q19 && COLL == LBM_MRT) {
    mrt3d_pair_reverse(fin, lam, imult, dimult, dg, p);
    return;
  }
  constexpr int QF = L::QF;
  C fo[QF];
#pragma unroll
  for (int i = 0; i < QF; ++i) fo[i] = fin[i];
  C rho, jx, jy, jz;
  {
    // base collision output (without PBB), as the reverse PBB recomputes it
    flow_macros<LAT>(fo, rho, jx, jy, jz);
    const C om = mp<C>(p).omega;
    if (COLL == LBM_BGK) {
      if (L::DIM == 2) {
        const C uSqr = jx * jx + jy * jy;
        const C cFeq = rho - C(1.5) * uSqr;
        const C rel = C(1.) - om;
        const C restW = C(4. / 9.), stW = C(1. / 9.), diagW = C(1. / 36.);
        fo[0] = rel * fo[0] + om * restW * cFeq;
        fo[2] = rel * fo[2] + om * stW * (cFeq - C(3.) * jy + C(4.5) * jy * jy);
        fo[4] = rel * fo[4] + om * stW * (cFeq - C(3.) * jx + C(4.5) * jx * jx);
        fo[6] = rel * fo[6] + om * stW * (cFeq + C(3.) * jy + C(4.5) * jy * jy);
        fo[8] = rel * fo[8] + om * stW * (cFeq + C(3.) * jx + C(4.5) * jx * jx);
        fo[1] = rel * fo[1] + om * diagW * (cFeq + C(3.) * (jx - jy) + C(4.5) * (uSqr - C(2.) * jx * jy));
        fo[3] = rel * fo[3] + om * diagW * (cFeq - C(3.) * (jx + jy) + C(4.5) * (uSqr + C(2.) * jx * jy));
        fo[5] = rel * fo[5] + om * diagW * (cFeq + C(3.) * (jy - jx) + C(4.5) * (uSqr - C(2.) * jx * jy));
        fo[7] = rel * fo[7] + om * diagW * (cFeq + C(3.) * (jx + jy) + C(4.5) * (uSqr + C(2.) * jx * jy));
      } else {
        const C uSqr = jx * jx + jy * jy + jz * jz;
        static_for<QF>([&](auto I) {
          constexpr int i = decltype(I)::value;
          const C sc = e_dot<LAT, i>(jx, jy, jz);
          C eq = C(L::w(i)) * (rho + C(3.) * sc + C(4.5) * sc * sc - C(1.5) * uSqr);
          fo[i] = fo[i] * (C(1.) - om) + om * eq;
        });
      }
    } else {
      C mo[MRT<L::DIM>::K];
      mrt_moments<L::DIM>(fo, mo);
      if (L::DIM == 2)
        mrt2d_relax(mo, rho, jx, jy, p);
      else
        mrt3d_relax(mo, rho, jx, jy, jz, p);
      mrt_backmap<L::DIM>(fo, mo);
    }
  }
  // reverse PBB
  C imultRev = C(0.);
#pragma unroll
  for (int d = 1; d <= L::HALF; ++d) {
    imultRev += (fo[d] - fo[d + L::HALF]) * lam[d + L::HALF];
    imultRev += (fo[d + L::HALF] - fo[d]) * lam[d];
    C t = lam[d + L::HALF];
    lam[d + L::HALF] += imult * (lam[d] - lam[d + L::HALF]);
    lam[d] += imult * (t - lam[d]);
  }
  dg += dimult * imultRev;
  // reverse base collision
  const C om = mp<C>(p).omega;
  if (COLL == LBM_BGK) {
    if (L::DIM == 2) {
      const C rel = C(1.) - om;
      const C restW = C(4. / 9.), stW = C(1. / 9.), diagW = C(1. / 36.);
      C r0 = C(0.), r1 = C(0.), r2 = C(0.);
      C uSqrRev, cFeqRev, temp;
      C li[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) li[i] = rel * lam[i];
      temp = om * diagW * lam[7];
      cFeqRev = temp;
      uSqrRev = temp;
      r1 += temp * (C(9.) * jy + C(3.));
      r2 += C(3.) * temp * (C(3.) * jx + C(1.));
      temp = om * diagW * lam[5];
      cFeqRev += temp;
      uSqrRev += temp;
      r1 -= temp * (C(9.) * jy + C(3.));
      r2 += temp * (C(3.) - C(9.) * jx);
      temp = om * diagW * lam[3];
      cFeqRev += temp;
      uSqrRev += temp;
      r1 += temp * (C(9.) * jy - C(3.));
      r2 += temp * (C(9.) * jx - C(3.));
      temp = om * diagW * lam[1];
      cFeqRev += temp;
      uSqrRev += temp;
      uSqrRev *= C(4.5);
      r1 += temp * (C(3.) - C(9.) * jy);
      r2 -= temp * (C(9.) * jx + C(3.));
      temp = om * stW * lam[8];
      cFeqRev += temp;
      r1 += (C(9.) * jx + C(3.)) * temp;
      temp = om * stW * lam[6];
      cFeqRev += temp;
      r2 = r2 + (C(9.) * jy + C(3.)) * temp;
      temp = om * stW * lam[4];
      cFeqRev += temp;
      r1 = r1 + (C(9.) * jx - C(3.)) * temp;
      temp = om * stW * lam[2];
      cFeqRev += temp + om * restW * lam[0];
      r2 = r2 + (C(9.) * jy - C(3.)) * temp;
      uSqrRev -= C(1.5) * cFeqRev;
      r0 = r0 + cFeqRev;
      r1 = r1 + C(2.) * jx * uSqrRev;
      r2 = r2 + C(2.) * jy * uSqrRev;
      lam[0] = li[0] + r0;
      lam[1] = li[1] + (r0 + r1 - r2);
      lam[2] = li[2] + (r0 - r2);
      lam[3] = li[3] + (r0 - r1 - r2);
      lam[4] = li[4] + (r0 - r1);
      lam[5] = li[5] + (r0 - r1 + r2);
      lam[6] = li[6] + (r0 + r2);
      lam[7] = li[7] + (r0 + r1 + r2);
      lam[8] = li[8] + (r0 + r1);
    } else {
      C rR = C(0.), jR0 = C(0.), jR1 = C(0.), jR2 = C(0.);
      static_for<QF>([&](auto I) {
        constexpr int i = decltype(I)::value;
        const C sc = e_dot<LAT, i>(jx, jy, jz);
        C a = om * C(L::w(i)) * lam[i];
        rR += a;
        C ds = a * (C(3.) + C(9.) * sc);
        // jR_c += ds e_ic - 3 a j_c, the zero components of e_i left out
        const C t3 = C(3.) * a;
        if constexpr (L::ex(i) == 1) jR0 += ds - t3 * jx;
        else if constexpr (L::ex(i) == -1) jR0 += -ds - t3 * jx;
        else jR0 += -(t3 * jx);
        if constexpr (L::ey(i) == 1) jR1 += ds - t3 * jy;
        else if constexpr (L::ey(i) == -1) jR1 += -ds - t3 * jy;
        else jR1 += -(t3 * jy);
        if constexpr (L::ez(i) == 1) jR2 += ds - t3 * jz;
        else if constexpr (L::ez(i) == -1) jR2 += -ds - t3 * jz;
        else jR2 += -(t3 * jz);
      });
      static_for<QF>([&](auto I) {
        constexpr int i = decltype(I)::value;
        lam[i] = (C(1.) - om) * lam[i] + (rR + e_dot<LAT, i>(jR0, jR1, jR2));
      });
    }
  } else {
    using M = MRT<L::DIM>;
    C a[M::K];
    C rate[M::K];
    if (L::DIM == 2) {
      rate[0] = mp<C>(p).mrt[0];
      rate[1] = mp<C>(p).mrt[1];
      rate[2] = mp<C>(p).mrt[2];
      rate[3] = mp<C>(p).mrt[2];
      rate[4] = om;
      rate[5] = om;
    } else {
      rate[0] = mp<C>(p).mrt[0];
      rate[1] = mp<C>(p).mrt[1];
      rate[2] = rate[3] = rate[4] = mp<C>(p).mrt[2];
      rate[5] = om;
      rate[6] = mp<C>(p).mrt[3];
      rate[7] = om;
      rate[8] = mp<C>(p).mrt[3];
      rate[9] = rate[10] = rate[11] = om;
      rate[12] = rate[13] = rate[14] = mp<C>(p).mrt[4];
    }
    static_for<M::K>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      // sum_i (-M[k][i]/N_k) lam_i
      C s = mrt_moment<L::DIM, k>(lam);
      constexpr double inv = -1.0 / (double)M::n(k);
      a[k] = rate[k] * (C(inv) * s);
    });
    C rR, jR0, jR1, jR2;
    if (L::DIM == 2) {
      rR = -(a[0] * C(-2.) + a[1]);
      jR0 = -(a[0] * C(6.) * jx - a[1] * C(6.) * jx - a[2] + a[4] * C(2.) * jx + a[5] * jy);
      jR1 = -(a[0] * C(6.) * jy - a[1] * C(6.) * jy - a[3] - a[4] * C(2.) * jy + a[5] * jx);
      jR2 = C(0.);
    } else {
      const C we = mp<C>(p).mrt[5], wej = mp<C>(p).mrt[6], wxx = mp<C>(p).mrt[7];
      const C c2 = C(-2. / 3.);
      const C a56 = a[5] + wxx * a[6], a78 = a[7] + wxx * a[8];
      rR = -(a[0] * C(-11.) + a[1] * we);
      jR0 = -(a[0] * C(38.) * jx + a[1] * C(2.) * wej * jx + a[2] * c2 + a56 * C(4.) * jx +
              a[9] * jy + a[11] * jz);
      jR1 = -(a[0] * C(38.) * jy + a[1] * C(2.) * wej * jy + a[3] * c2 - a56 * C(2.) * jy +
              a78 * C(2.) * jy + a[9] * jx + a[10] * jz);
      jR2 = -(a[0] * C(38.) * jz + a[1] * C(2.) * wej * jz + a[4] * c2 - a56 * C(2.) * jz -
              a78 * C(2.) * jz + a[10] * jy + a[11] * jx);
    }
    static_for<QF>([&](auto I) {
      constexpr int i = decltype(I)::value;
      C v = lam[i];
      static_for<M::K>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        constexpr int c = M::m(k, i);
        if constexpr (c == 1) {
          v += a[k];
        } else if constexpr (c == -1) {
          v -= a[k];
        } else if constexpr (c != 0) {
          v += C(c) * a[k];
        }
      });
      lam[i] = v + (rR + e_dot<LAT, i>(jR0, jR1, jR2));
    });
  }
}

// ---------------------------------------------------------------------------
// Temperature lattice (D2Q5, directions 9..13): ThermalBGK2d with the obstacle
// rate of ThermalObstacleCollision (dynamics/thermalBGK2d.hh:58-65,
// thermalObstacleCollision.hh:47-53) after the flow collision
// (thermalDualCollision.hh:57-64), plus solid heating (1-g) h (Th - T) w_i.

template <class C>
__device__ __forceinline__ C thermal_omega(C g, const KParams& p) {
  C imult = mp<C>(p).diff * ramp(g, mp<C>(p).ramp_q, mp<C>(p).ramp_ck);
  return C(1.) / (C(3.) * imult + C(0.5));
}

template <class C>
__device__ __forceinline__ void thermal_collide(C* gp, C ux, C uy, C g, C& T, const KParams& p) {
  constexpr double W5[5] = {1. / 3., 1. / 6., 1. / 6., 1. / 6., 1. / 6.};
  constexpr int EX5[5] = {0, 0, -1, 0, 1}, EY5[5] = {0, -1, 0, 1, 0};
  const C om = thermal_omega(g, p);
  T = gp[0] + gp[1] + gp[2] + gp[3] + gp[4];
  const C hs = (C(1.) - g) * mp<C>(p).heat_rate * (mp<C>(p).heat_T - T);
  static_for<5>([&](auto I) {
    constexpr int i = decltype(I)::value;
    C sc = C(EX5[i]) * ux + C(EY5[i]) * uy;
    C eq = C(W5[i]) * T * (C(1.) + C(3.) * sc);
    gp[i] = gp[i] * (C(1.) - om) + om * eq;
    gp[i] += C(W5[i]) * hs;
  });
}

// ---------------------------------------------------------------------------
// Collision in increment form, for FP32 and FP16 storage.
//
// Rounding to nearest is deterministic: in a slowly varying flow a cell rounds
// the same way at every step, which acts like a small constant source of mass
// and momentum, and the stored state drifts away from the exact one linearly
// in time (4e-4 relative after 20000 steps of a 1024x512 channel in FP32).
// Two changes remove the drift:
//  - the collision produces increments d (f_out = f + d) whose mass and
//    momentum change is exactly the operator's (zero, except the partial
//    bounce-back drag) up to the rounding of d itself, which is orders of
//    magnitude below that of f: BGK increments are projected onto zero mass and
//    momentum, MRT increments are back-mapped from the non-conserved moments
//    only, and the partial bounce-back moves equal and opposite amounts;
//  - f + d is rounded to the storage type without bias (stochastic rounding:
//    uniform noise of one unit in the last place is added before rounding to
//    nearest), keyed on (cell, time step, direction), so a recomputed step
//    reproduces its state bit for bit.

__host__ __device__ __forceinline__ unsigned mix32(unsigned v) {
  v ^= v >> 16;
  v *= 0x7feb352du;
  v ^= v >> 15;
  v *= 0x846ca68bu;
  v ^= v >> 16;
  return v;
}

// Per-cell stream of uniform variates: a hash of (cell, step, salt) seeds a
// 32-bit linear congruential sequence; each draw gives one or two variates.
struct Dither {
  unsigned r;
  // key: step_key(step, salt), the same for every cell of a launch
  __device__ __forceinline__ Dither(unsigned cell, unsigned key) : r(mix32(cell ^ key)) {}
  // uniform in [1, 2) * 2^-K, 23 random mantissa bits (the sequence's low
  // bits have short periods, but they weigh below 2^-16 of the variate, and
  // over the cells' seeds every bit is uniform, so the rounding stays unbiased)
  template <int K>
  __device__ __forceinline__ float raw() {
    r = r * 1664525u + 1013904223u;
    constexpr unsigned kExp = (unsigned)(127 - K) << 23;
    return __uint_as_float(kExp | (r & 0x7fffffu));
  }
  // uniform in [-1/2, 1/2) * 2^-K for K = 23 (FP32) or 10 (FP16)
  template <int K>
  __device__ __forceinline__ float next() {
    constexpr float kHalf = 1.5f / (float)(1u << K);
    return raw<K>() - kHalf;
  }
  // Two variates of raw<K>() from one draw: a from bits 0-22, b from bits
  // 9-31.  Each is uniform on its own; they share bits 9-22, which are a's
  // leading bits but only b's trailing ones (below 2^-9 of b), so b's
  // leading nine bits (23-31) are independent of a.
  template <int K>
  __device__ __forceinline__ void raw_pair(float& a, float& b) {
    r = r * 1664525u + 1013904223u;
    constexpr unsigned kExp = (unsigned)(127 - K) << 23;
    a = __uint_as_float(kExp | (r & 0x7fffffu));
    b = __uint_as_float(kExp | (r >> 9));
  }
};

// Salts of the rounding streams of the two step kernels.
constexpr unsigned kSaltForward = 0x85ebca6bu, kSaltAdjoint = 0xc2b2ae35u;

__host__ __device__ __forceinline__ unsigned step_key(unsigned step, unsigned salt) {
  return mix32(step * 0x9E3779B9u + salt);
}

// Largest power of two not above |v| (0 for zero and subnormals).
__device__ __forceinline__ float pow2_floor(float v) {
  return __uint_as_float(__float_as_uint(v) & 0x7f800000u);
}

template <class S>
struct Round;
template <>
struct Round<float> {
  // The noise is scaled to the unit in the last place of f; where f + d
  // leaves f's binade (|d| is mostly far below |f|) the rounding is still
  // unbiased downwards and nearly so upwards.
  __device__ static __forceinline__ float apply(float f, float d, Dither& rnd) {
    return f + fmaf(rnd.next<23>(), pow2_floor(f), d);
  }
  // Two populations at once from one draw (Dither::raw_pair), in packed
  // FP32x2 arithmetic where the GPU has it; the same values either way.
  __device__ static __forceinline__ void apply_pair(float fa, float fb, float da, float db,
                                                    Dither& rnd, float& oa, float& ob) {
    constexpr float kHalf = 1.5f / (float)(1u << 23);
    float ua, ub;
    rnd.raw_pair<23>(ua, ub);
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    const float2 u = __fadd2_rn(make_float2(ua, ub), make_float2(-kHalf, -kHalf));
    const float2 n = __ffma2_rn(u, make_float2(pow2_floor(fa), pow2_floor(fb)), make_float2(da, db));
    const float2 o = __fadd2_rn(make_float2(fa, fb), n);
    oa = o.x;
    ob = o.y;
#else
    oa = fa + fmaf(ua - kHalf, pow2_floor(fa), da);
    ob = fb + fmaf(ub - kHalf, pow2_floor(fb), db);
#endif
  }
};
template <>
struct Round<__half> {
  __device__ static __forceinline__ __half apply(float f, float d, Dither& rnd) {
    const float s = f + d;
    // below 2^-14 the FP16 spacing stays 2^-24 (subnormals)
    const float bin = fmaxf(pow2_floor(s), 6.103515625e-05f);
    return __float2half_rn(fmaf(rnd.next<10>(), bin, s));
  }
  // Two populations from one draw (Dither::raw_pair), in packed FP32x2
  // arithmetic with one packed conversion where the GPU has them; the same
  // values either way.
  __device__ static __forceinline__ void apply_pair(float fa, float fb, float da, float db,
                                                    Dither& rnd, __half& oa, __half& ob) {
    constexpr float kHalf = 1.5f / (float)(1u << 10);
    constexpr float kSub = 6.103515625e-05f;
    float ua, ub;
    rnd.raw_pair<10>(ua, ub);
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    const float2 sv = __fadd2_rn(make_float2(fa, fb), make_float2(da, db));
    const float2 u = __fadd2_rn(make_float2(ua, ub), make_float2(-kHalf, -kHalf));
    const float2 bin = make_float2(fmaxf(pow2_floor(sv.x), kSub), fmaxf(pow2_floor(sv.y), kSub));
    const float2 r = __ffma2_rn(u, bin, sv);
    const __half2 h = __floats2half2_rn(r.x, r.y);
    oa = __low2half(h);
    ob = __high2half(h);
#else
    const float sa = fa + da, sb = fb + db;
    oa = __float2half_rn(fmaf(ua - kHalf, fmaxf(pow2_floor(sa), kSub), sa));
    ob = __float2half_rn(fmaf(ub - kHalf, fmaxf(pow2_floor(sb), kSub), sb));
#endif
  }
};

// (0.5 (e + a), 0.5 (e - a)): the increments of a population pair from its
// even and odd parts
__device__ __forceinline__ void pair_halves(float e, float a, float& p, float& m) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  const float2 v = __fmul2_rn(make_float2(0.5f, 0.5f), __fadd2_rn(make_float2(e, e), make_float2(a, -a)));
  p = v.x;
  m = v.y;
#else
  p = 0.5f * (e + a);
  m = 0.5f * (e - a);
#endif
}
__device__ __forceinline__ void pair_halves(double e, double a, double& p, double& m) {
  p = 0.5 * (e + a);
  m = 0.5 * (e - a);
}


// Increments of mrt3d_pair_collide (same operator: f + d is its output),
// handed to emit(q, d_q) pair by pair so each pair's registers are freed early.
template <class C, class Emit, class Emit2>
__device__ __forceinline__ void mrt3d_pair_collide_inc(const C* f, C imult, C& rho, C& jx, C& jy,
                                                       C& jz, const KParams& p, Emit&& emit,
                                                       Emit2&& emit2) {
  C s[10], a[10], mo[15];
  mrt3d_pair_moments(f, s, a, rho, jx, jy, jz, mo);
  mrt3d_relax(mo, rho, jx, jy, jz, p);
  const Mrt3dEvenBack<C> eb(mo);
  emit(std::integral_constant<int, 0>{}, eb.d0);
  const C twoim = C(2.) * imult;
  static_for<9>([&](auto D) {
    constexpr int d = decltype(D)::value + 1;
    const C E = eb.template E<d>();
    const C O = mrt3d_odd_back<d>(mo);
    // s' = s + E, a'' = (a + O)(1 - 2 imult) = a + O - 2 imult (a + O); a is
    // recomputed from f (same value) so that only f stays live across the loop
    const C da = O - twoim * ((f[d] - f[d + 9]) + O);
    C dp, dm;
    pair_halves(E, da, dp, dm);
    emit2(std::integral_constant<int, d>{}, std::integral_constant<int, d + 9>{}, dp, dm);
  });
}

// Increments of flow_collide (collision + partial bounce-back), handed to
// emit(q, d_q) once per flow population; returns the macros of the input.
template <int LAT, int COLL, class C, class Emit, class Emit2>
__device__ __forceinline__ void flow_collide_inc(const C* f, C imult, C& rho, C& jx, C& jy, C& jz,
                                                 const KParams& p, Emit&& emit, Emit2&& emit2) {
  using L = Lattice<LAT>;
  if constexpr (LAT == LAT_D3Q19 && COLL == LBM_MRT) {
    mrt3d_pair_collide_inc(f, imult, rho, jx, jy, jz, p, emit, emit2);
  } else if constexpr (COLL == LBM_BGK) {
    // BGK increments d_i = omega (feq_i - f_i), projected onto zero mass and
    // momentum (d_i -= w_i (a + 3 e_i.b) with a = sum d, b = sum e d: then
    // they carry none, as sum w = 1, sum w e = 0, sum w e e = I/3), then the
    // partial bounce-back; all on the even and odd parts of each pair
    // (k, k+H), ee = d_k + d_{k+H} and oo = d_k - d_{k+H}.  An even part
    // carries its pair's mass and an odd part its momentum, so the
    // projection subtracts 2 w_k a from ee and 6 w_k e_k.b from oo.
    constexpr int H = L::HALF;
    flow_macros<LAT>(f, rho, jx, jy, jz);
    const C om = mp<C>(p).omega;
    const C cFeq = rho - C(1.5) * (jx * jx + jy * jy + jz * jz);
    C d0 = om * (C(L::w(0)) * cFeq - f[0]);
    auto even = [&](auto K, C sc) -> C {
      constexpr int k = decltype(K)::value;
      return om * (C(2. * L::w(k)) * (cFeq + C(4.5) * sc * sc) - (f[k] + f[k + H]));
    };
    auto odd = [&](auto K, C sc) -> C {
      constexpr int k = decltype(K)::value;
      return om * (C(6. * L::w(k)) * sc - (f[k] - f[k + H]));
    };
    // D2Q9 keeps the parts in registers between the two passes; D3Q19
    // recomputes them (same expressions, same values) to stay within its
    // register budget
    constexpr bool kKeep = H <= 4;
    C ee[kKeep ? H : 1], oo[kKeep ? H : 1];
    C a = d0, bx = C(0.), by = C(0.), bz = C(0.);
    static_for<H>([&](auto D) {
      constexpr int k = decltype(D)::value + 1;
      const auto K = std::integral_constant<int, k>{};
      const C sc = e_dot<LAT, k>(jx, jy, jz);
      const C e = even(K, sc), o = odd(K, sc);
      if constexpr (kKeep) {
        ee[k - 1] = e;
        oo[k - 1] = o;
      }
      a += e;
      if constexpr (L::ex(k) == 1) bx += o;
      if constexpr (L::ex(k) == -1) bx -= o;
      if constexpr (L::ey(k) == 1) by += o;
      if constexpr (L::ey(k) == -1) by -= o;
      if constexpr (L::ez(k) == 1) bz += o;
      if constexpr (L::ez(k) == -1) bz -= o;
    });
    emit(std::integral_constant<int, 0>{}, d0 - C(L::w(0)) * a);
    const C twoim = C(2.) * imult;
    static_for<H>([&](auto D) {
      constexpr int k = decltype(D)::value + 1;
      const auto K = std::integral_constant<int, k>{};
      C e, o;
      if constexpr (kKeep) {
        e = ee[k - 1];
        o = oo[k - 1];
      } else {
        const C sc = e_dot<LAT, k>(jx, jy, jz);
        e = even(K, sc);
        o = odd(K, sc);
      }
      const C E = e - C(2. * L::w(k)) * a;
      const C O = o - C(6. * L::w(k)) * e_dot<LAT, k>(bx, by, bz);
      // partial bounce-back moves imult ((f_{k+H} - f_k) + (d_{k+H} - d_k))
      // from k+H to k: the odd part becomes O - 2 imult ((f_k - f_{k+H}) + O)
      const C A = O - twoim * ((f[k] - f[k + H]) + O);
      C dp, dm;
      pair_halves(E, A, dp, dm);
      emit2(std::integral_constant<int, k>{}, std::integral_constant<int, k + H>{}, dp, dm);
    });
  } else {
    // MRT on the 2D lattices: increments back-mapped from the relaxed
    // non-conserved moments
    C d[L::QF];
    flow_macros<LAT>(f, rho, jx, jy, jz);
    using M = MRT<L::DIM>;
    C mo[M::K];
    mrt_moments<L::DIM>(f, mo);
    if (L::DIM == 2)
      mrt2d_relax(mo, rho, jx, jy, p);
    else
      mrt3d_relax(mo, rho, jx, jy, jz, p);
    static_for<M::QF>([&](auto I) {
      constexpr int i = decltype(I)::value;
      C v = C(0.);
      static_for<M::K>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        constexpr int c = M::m(k, i);
        if constexpr (c != 0) {
          constexpr double b = -(double)c / (double)M::n(k);
          v += C(b) * mo[k];
        }
      });
      d[i] = v;
    });
    emit(std::integral_constant<int, 0>{}, d[0]);
    // partial bounce-back on the collided values f + d, moving equal and
    // opposite amounts within each pair
    static_for<L::HALF>([&](auto D) {
      constexpr int k = decltype(D)::value + 1;
      const C m = imult * ((f[k + L::HALF] - f[k]) + (d[k + L::HALF] - d[k]));
      emit2(std::integral_constant<int, k>{}, std::integral_constant<int, k + L::HALF>{}, d[k] + m,
            d[k + L::HALF] - m);
    });
  }
}

// Increments of thermal_collide, handed to emit(i, d_i) for i = 0..4: the
// collision conserves sum g up to the rounding of the increments; the heating
// source is added after.
template <class C, class Emit>
__device__ __forceinline__ void thermal_collide_inc(const C* gp, C ux, C uy, C g, const KParams& p,
                                                    Emit&& emit) {
  using L = Lattice<LAT_D2Q9_D2Q5>;   // D2Q5 directions are its entries 9..13
  const C om = thermal_omega(g, p);
  const C T = gp[0] + gp[1] + gp[2] + gp[3] + gp[4];
  const C hs = (C(1.) - g) * mp<C>(p).heat_rate * (mp<C>(p).heat_T - T);
  C dg[5];
  C a = C(0.);
  static_for<5>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const C sc = e_dot<LAT_D2Q9_D2Q5, i + 9>(ux, uy, C(0.));
    const C eq = C(L::w(i + 9)) * T * (C(1.) + C(3.) * sc);
    dg[i] = om * (eq - gp[i]);
    a += dg[i];
  });
  static_for<5>([&](auto I) {
    constexpr int i = decltype(I)::value;
    emit(I, dg[i] + C(L::w(i + 9)) * (hs - a));
  });
}

// Transpose of thermal_collide at input (gin, ux, uy); lam[0..4] in/out;
// returns the adjoint of (ux, uy) and adds to dg.
template <class C>
__device__ __forceinline__ void thermal_reverse(const C* gin, C* lam, C ux, C uy, C g, C& uxR,
                                                C& uyR, C& dg, const KParams& p) {
  constexpr double W5[5] = {1. / 3., 1. / 6., 1. / 6., 1. / 6., 1. / 6.};
  constexpr int EX5[5] = {0, 0, -1, 0, 1}, EY5[5] = {0, -1, 0, 1, 0};
  const C T = gin[0] + gin[1] + gin[2] + gin[3] + gin[4];
  const C om = thermal_omega(g, p);
  C TR = C(0.), omR = C(0.), hsR = C(0.);
  uxR = C(0.);
  uyR = C(0.);
  C li[5];
  static_for<5>([&](auto I) {
    constexpr int i = decltype(I)::value;
    C sc = C(EX5[i]) * ux + C(EY5[i]) * uy;
    C eq = C(W5[i]) * T * (C(1.) + C(3.) * sc);
    li[i] = (C(1.) - om) * lam[i];
    omR += (eq - gin[i]) * lam[i];
    C a = om * lam[i] * C(W5[i]);
    TR += a * (C(1.) + C(3.) * sc);
    uxR += a * T * C(3.) * C(EX5[i]);
    uyR += a * T * C(3.) * C(EY5[i]);
    hsR += C(W5[i]) * lam[i];
  });
  TR += -(C(1.) - g) * mp<C>(p).heat_rate * hsR;
  dg += -mp<C>(p).heat_rate * (mp<C>(p).heat_T - T) * hsR;
  const C den = C(3.) * mp<C>(p).diff * ramp(g, mp<C>(p).ramp_q, mp<C>(p).ramp_ck) + C(0.5);
  dg += omR * (C(-1.) / (den * den)) * C(3.) * mp<C>(p).diff * ramp_diff(g, mp<C>(p).ramp_q, mp<C>(p).ramp_ck);
#pragma unroll
  for (int i = 0; i < 5; ++i) lam[i] = li[i] + TR;
}

// Increments d[0..4] of thermal_reverse: lam + d is its output; the same
// adjoint of (ux, uy) and the same dg.  The constant vector is invariant under
// the transposed collision (sum_j dgeq_j/dT = 1), so the increment is projected
// with c = sum_i W_i (1 + 3 e_i . u) d_i before the heating term is added.
template <class C>
__device__ __forceinline__ void thermal_reverse_inc(const C* gin, const C* lam, C* d, C ux, C uy,
                                                    C g, C& uxR, C& uyR, C& dg, const KParams& p) {
  using L = Lattice<LAT_D2Q9_D2Q5>;   // D2Q5 directions are its entries 9..13
  const C T = gin[0] + gin[1] + gin[2] + gin[3] + gin[4];
  const C om = thermal_omega(g, p);
  C cT = C(0.), omR = C(0.), hsR = C(0.);
  uxR = C(0.);
  uyR = C(0.);
  C wt[5];
  static_for<5>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const C sc = e_dot<LAT_D2Q9_D2Q5, i + 9>(ux, uy, C(0.));
    const C w = C(L::w(i + 9));
    const C eq = w * T * (C(1.) + C(3.) * sc);
    wt[i] = w * (C(1.) + C(3.) * sc);
    cT += wt[i] * lam[i];
    omR += (eq - gin[i]) * lam[i];
    const C a = om * lam[i] * w;
    if constexpr (L::ex(i + 9) != 0) uxR += a * T * C(3. * L::ex(i + 9));
    if constexpr (L::ey(i + 9) != 0) uyR += a * T * C(3. * L::ey(i + 9));
    hsR += w * lam[i];
  });
  C c = C(0.);
  static_for<5>([&](auto I) {
    constexpr int i = decltype(I)::value;
    d[i] = om * (cT - lam[i]);
    c += wt[i] * d[i];
  });
  const C heat = -(C(1.) - g) * mp<C>(p).heat_rate * hsR;
  static_for<5>([&](auto I) {
    constexpr int i = decltype(I)::value;
    d[i] = (d[i] - c) + heat;
  });
  dg += -mp<C>(p).heat_rate * (mp<C>(p).heat_T - T) * hsR;
  const C den = C(3.) * mp<C>(p).diff * ramp(g, mp<C>(p).ramp_q, mp<C>(p).ramp_ck) + C(0.5);
  dg += omR * (C(-1.) / (den * den)) * C(3.) * mp<C>(p).diff *
        ramp_diff(g, mp<C>(p).ramp_q, mp<C>(p).ramp_ck);
}


// ---------------------------------------------------------------------------
// Reverse BGK and thermal collisions in increment form (FP32 adjoints).
//
// The transpose of a BGK collision at state f is lam -> mu + omega (E^T mu - mu)
// with mu the reverse partial bounce-back of lam and E the Jacobian of the
// equilibrium, a projection (E^2 = E) whose transpose keeps the constant
// vector and e_a: these directions are invariant, so rounding errors along
// them add up over the reverse sweep exactly as mass and momentum errors do in
// the forward one.  The increments are projected with (I - E^T), which keeps
// the exact increment unchanged and removes those components, and lam + d is
// rounded without bias (Round / Dither).

// (E^T v)_i = c0 + e_i . c with c0 = sum_j w_j v_j and
// c_a = sum_j w_j (3 e_ja + 9 (e_j . u) e_ja - 3 u_a) v_j (incompressible
// equilibrium at velocity u = j).
template <int LAT, class C>
__device__ __forceinline__ void eq_transpose_coeffs(const C* v, C jx, C jy, C jz, C& c0, C& cx,
                                                    C& cy, C& cz) {
  using L = Lattice<LAT>;
  C p1x = C(0.), p1y = C(0.), p1z = C(0.), p2x = C(0.), p2y = C(0.), p2z = C(0.);
  c0 = C(0.);
  static_for<L::QF>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const C wv = C(L::w(i)) * v[i];
    const C sw = e_dot<LAT, i>(jx, jy, jz) * wv;
    c0 += wv;
    if constexpr (L::ex(i) == 1) { p1x += wv; p2x += sw; }
    if constexpr (L::ex(i) == -1) { p1x -= wv; p2x -= sw; }
    if constexpr (L::ey(i) == 1) { p1y += wv; p2y += sw; }
    if constexpr (L::ey(i) == -1) { p1y -= wv; p2y -= sw; }
    if constexpr (L::ez(i) == 1) { p1z += wv; p2z += sw; }
    if constexpr (L::ez(i) == -1) { p1z -= wv; p2z -= sw; }
  });
  cx = C(3.) * (p1x - jx * c0) + C(9.) * p2x;
  cy = C(3.) * (p1y - jy * c0) + C(9.) * p2y;
  cz = C(3.) * (p1z - jz * c0) + C(9.) * p2z;
}

// Increments d of flow_reverse<LAT, BGK> at input fin: lam + d is its output;
// dg += dimult * d(out)/d(imult)^T lam.
//
// Evaluated on the sum and difference of each population pair (k, k+H): E^T v
// has the even part c0 and the odd part e_k.c, and c0, c take the pair sums
// v_k + v_{k+H} (weight w_k, and w_k e_k.u for the u-dependent part of c) and
// differences v_k - v_{k+H} (weight w_k e_k).  The reverse partial bounce-back
// keeps a pair's sum and scales its difference by 1 - 2 imult.
template <int LAT, class C>
__device__ __forceinline__ void bgk_reverse_inc(const C* fin, const C* lam, C* d, C imult,
                                                C dimult, C& dg, const KParams& p) {
  using L = Lattice<LAT>;
  constexpr int H = L::HALF;
  C rho, jx, jy, jz;
  flow_macros<LAT>(fin, rho, jx, jy, jz);
  const C om = mp<C>(p).omega;
  // sensitivity to imult: sum over pairs of (fo_k - fo_opp)(lam_opp - lam_k),
  // fo the collided state before partial bounce-back, whose pair difference
  // is fd + omega (6 w_k e_k.j - fd) with fd = f_k - f_opp
  C imultRev = C(0.);
  static_for<H>([&](auto D) {
    constexpr int k = decltype(D)::value + 1;
    const C fd = fin[k] - fin[k + H];
    const C sc = e_dot<LAT, k>(jx, jy, jz);
    imultRev += (fd + om * (C(6. * L::w(k)) * sc - fd)) * (lam[k + H] - lam[k]);
  });
  dg += dimult * imultRev;
  // c0 and c of E^T v from the rest value v0 and the pair sums vs(k) and
  // differences vd(k)
  auto transpose = [&](C v0, auto&& vs, auto&& vd, C& c0, C& cx, C& cy, C& cz) {
    C p1x = C(0.), p1y = C(0.), p1z = C(0.), p2x = C(0.), p2y = C(0.), p2z = C(0.);
    c0 = C(L::w(0)) * v0;
    static_for<H>([&](auto D) {
      constexpr int k = decltype(D)::value + 1;
      const auto K = std::integral_constant<int, k>{};
      const C ws = C(L::w(k)) * vs(K);
      const C wd = C(L::w(k)) * vd(K);
      const C sw = e_dot<LAT, k>(jx, jy, jz) * ws;
      c0 += ws;
      if constexpr (L::ex(k) == 1) { p1x += wd; p2x += sw; }
      if constexpr (L::ex(k) == -1) { p1x -= wd; p2x -= sw; }
      if constexpr (L::ey(k) == 1) { p1y += wd; p2y += sw; }
      if constexpr (L::ey(k) == -1) { p1y -= wd; p2y -= sw; }
      if constexpr (L::ez(k) == 1) { p1z += wd; p2z += sw; }
      if constexpr (L::ez(k) == -1) { p1z -= wd; p2z -= sw; }
    });
    cx = C(3.) * (p1x - jx * c0) + C(9.) * p2x;
    cy = C(3.) * (p1y - jy * c0) + C(9.) * p2y;
    cz = C(3.) * (p1z - jz * c0) + C(9.) * p2z;
  };
  const C keep = C(1.) - C(2.) * imult;
  auto lam_sum = [&](auto K) -> C {
    constexpr int k = decltype(K)::value;
    return lam[k] + lam[k + H];
  };
  auto mu_diff = [&](auto K) -> C {
    constexpr int k = decltype(K)::value;
    return keep * (lam[k] - lam[k + H]);
  };
  // reverse collision: omega (E^T mu - mu), projected with (I - E^T)
  C c0, cx, cy, cz;
  transpose(lam[0], lam_sum, mu_diff, c0, cx, cy, cz);
  const C d0 = om * (c0 - lam[0]);
  C ds[H], dd[H];
  static_for<H>([&](auto D) {
    constexpr int k = decltype(D)::value + 1;
    const auto K = std::integral_constant<int, k>{};
    ds[k - 1] = om * (C(2.) * c0 - lam_sum(K));
    dd[k - 1] = om * (C(2.) * e_dot<LAT, k>(cx, cy, cz) - mu_diff(K));
  });
  transpose(
      d0, [&](auto K) -> C { return ds[decltype(K)::value - 1]; },
      [&](auto K) -> C { return dd[decltype(K)::value - 1]; }, c0, cx, cy, cz);
  d[0] = d0 - c0;
  static_for<H>([&](auto D) {
    constexpr int k = decltype(D)::value + 1;
    // the reverse partial bounce-back adds imult (lam_opp - lam_k) to k and
    // takes it from opp
    const C es = ds[k - 1] - C(2.) * c0;
    const C od = (dd[k - 1] - C(2.) * e_dot<LAT, k>(cx, cy, cz)) -
                 C(2.) * imult * (lam[k] - lam[k + H]);
    pair_halves(es, od, d[k], d[k + H]);
  });
}

// ---------------------------------------------------------------------------
// Boundary conditions on one cell's post-stream populations at time t.
// Zou-He (boundaryConditions/ZouHe2d.hh:23-391), Hecht (Hecht3d.hh:62-94,175-209),
// thermal Zou-He (thermalZouHe2d.hh:63-81).  D2Q9 numbering: e_1 = (1,-1),
// e_2 = (0,-1), e_3 = (-1,-1), e_4 = (-1,0), e_5 = (-1,1), e_6 = (0,1),
// e_7 = (1,1), e_8 = (1,0); a face's unknowns are the populations entering
// from outside (west 1,7,8; east 3,4,5; north 1,2,3; south 5,6,7).
//
// On shifted storage (f - w) every relation below holds unchanged for the
// deviations, because each one pairs populations of equal weight, except the
// density sums: the known-population sums of the Zou-He density relations have
// weight 1 (w_0 + w_2 + w_6 + 2(w_3 + w_4 + w_5) = 1 on the west face, and
// alike on the others), so the shifted forms use rho0 - 1 (vshift) in place of
// rho0, or add the 1 back where the density itself is needed.

// Prescribed density of a pressure boundary in the storage's convention.
template <bool SHIFT, class C>
__device__ __forceinline__ C bc_rho(const DevBC& b, int x, int y, int z) {
  if (bc_table<C>(b)) return bc_scalar<C>(b, x, y, z) - (SHIFT ? C(1.) : C(0.));
  return SHIFT ? bc_vshift<C>(b) : bc_value<C>(b);
}

template <int LAT, bool SHIFT, class C>
__device__ __forceinline__ void apply_bcs(C* f, int x, int y, int z, const KParams& p) {
  using L = Lattice<LAT>;
  for (int k = 0; k < p.nbc; ++k) {
    const DevBC& b = p.bc[k];
    if (!in_box(b.box, x, y, z)) continue;
    if (b.kind == LBM_BC_VELOCITY || b.kind == LBM_BC_VELOCITY_STANDARD) {
      C ux, uy, uz;
      bc_velocity<C>(b, x, y, z, ux, uy, uz);
      if (L::DIM == 2) {
        if (b.kind == LBM_BC_VELOCITY_STANDARD) {
          // StandardZouHeVelocityWest2d (ZouHe2d.hh:146-163): the standard
          // equilibrium's density from the known populations
          C rho = (f[0] + f[2] + f[6] + C(2.) * (f[3] + f[4] + f[5]));
          if (SHIFT) rho += C(1.);
          rho = rho / (C(1.) - ux);
          f[1] = f[5] + C(0.5) * (f[6] - f[2]) + C(1. / 6.) * rho * ux - C(0.5) * rho * uy;
          f[7] = f[3] + C(0.5) * (f[2] - f[6]) + C(1. / 6.) * rho * ux + C(0.5) * rho * uy;
          f[8] = f[4] + C(2. / 3.) * rho * ux;
        } else if (b.face == LBM_FACE_WEST) {
          f[1] = C(0.5) * (f[6] - f[2]) + f[5] + C(1. / 6.) * ux - C(0.5) * uy;
          f[7] = C(0.5) * (f[2] - f[6]) + f[3] + C(1. / 6.) * ux + C(0.5) * uy;
          f[8] = f[4] + C(2. / 3.) * ux;
        } else if (b.face == LBM_FACE_EAST) {
          f[3] = f[7] + C(0.5) * (f[6] - f[2]) - C(1. / 6.) * ux - C(0.5) * uy;
          f[4] = f[8] - C(2. / 3.) * ux;
          f[5] = f[1] + C(0.5) * (f[2] - f[6]) - C(1. / 6.) * ux + C(0.5) * uy;
        } else if (b.face == LBM_FACE_NORTH) {
          // IncompressibleZouHeVelocityNorth2d (ZouHe2d.hh:66-81)
          f[1] = C(0.5) * (f[4] - f[8]) + f[5] - C(1. / 6.) * uy + C(0.5) * ux;
          f[2] = f[6] - C(2. / 3.) * uy;
          f[3] = C(0.5) * (f[8] - f[4]) + f[7] - C(1. / 6.) * uy - C(0.5) * ux;
        } else {
          // south: the north operator mirrored in y (1<->7, 2<->6, 3<->5, uy -> -uy)
          f[7] = C(0.5) * (f[4] - f[8]) + f[3] + C(1. / 6.) * uy + C(0.5) * ux;
          f[6] = f[2] + C(2. / 3.) * uy;
          f[5] = C(0.5) * (f[8] - f[4]) + f[1] + C(1. / 6.) * uy - C(0.5) * ux;
        }
      } else {
        C Nyx = C(0.5) * (f[5] + f[11] + f[13] - (f[2] + f[4] + f[14])) - C(1. / 3.) * uy;
        C Nzx = C(0.5) * (f[10] + f[13] + f[14] - (f[1] + f[4] + f[5])) - C(1. / 3.) * uz;
        f[7] = f[16] + C(1. / 6.) * (ux - uz) + Nzx;
        f[9] = f[18] + C(1. / 6.) * (ux - uy) + Nyx;
        f[12] = f[3] + C(1. / 3.) * ux;
        f[15] = f[6] + C(1. / 6.) * (ux + uz) - Nzx;
        f[17] = f[8] + C(1. / 6.) * (ux + uy) - Nyx;
      }
    } else if (b.kind == LBM_BC_PRESSURE || b.kind == LBM_BC_PRESSURE_STANDARD) {
      const C rho0 = bc_rho<SHIFT, C>(b, x, y, z);
      if (L::DIM == 2) {
        if (b.kind == LBM_BC_PRESSURE_STANDARD && !SHIFT) {
          // StandardZouHePressureEast/West2d (ZouHe2d.hh:332-349, 366-383).  The
          // map equals the incompressible one (rho0*ux0 = S - rho0); shifted
          // storage evaluates it in that form below.
          if (b.face == LBM_FACE_EAST) {
            C ux0 = C(-1.) + (f[0] + f[2] + f[6] + C(2.) * (f[1] + f[7] + f[8])) / rho0;
            f[4] = f[8] - C(2. / 3.) * rho0 * ux0;
            f[3] = f[7] - C(1. / 6.) * rho0 * ux0 + C(0.5) * (f[6] - f[2]);
            f[5] = f[1] - C(1. / 6.) * rho0 * ux0 + C(0.5) * (f[2] - f[6]);
          } else {
            C ux0 = C(1.) - (f[0] + f[2] + f[6] + C(2.) * (f[3] + f[4] + f[5])) / rho0;
            f[1] = f[5] + C(1. / 6.) * rho0 * ux0 + C(0.5) * (f[6] - f[2]);
            f[7] = f[3] + C(1. / 6.) * rho0 * ux0 + C(0.5) * (f[2] - f[6]);
            f[8] = f[4] + C(2. / 3.) * rho0 * ux0;
          }
        } else if (b.face == LBM_FACE_EAST) {
          C ux0 = -rho0 + (f[0] + f[2] + f[6] + C(2.) * (f[1] + f[7] + f[8]));
          f[4] = f[8] - C(2. / 3.) * ux0;
          f[3] = f[7] - C(1. / 6.) * ux0 + C(0.5) * (f[6] - f[2]);
          f[5] = f[1] - C(1. / 6.) * ux0 + C(0.5) * (f[2] - f[6]);
        } else if (b.face == LBM_FACE_WEST) {
          C ux0 = rho0 - (f[0] + f[2] + f[6] + C(2.) * (f[3] + f[4] + f[5]));
          f[8] = f[4] + C(2. / 3.) * ux0;
          f[7] = f[3] + C(1. / 6.) * ux0 + C(0.5) * (f[2] - f[6]);
          f[1] = f[5] + C(1. / 6.) * ux0 + C(0.5) * (f[6] - f[2]);
        } else if (b.face == LBM_FACE_NORTH) {
          // the east operator rotated by +90 degrees (x -> y)
          C uy0 = -rho0 + (f[0] + f[8] + f[4] + C(2.) * (f[7] + f[5] + f[6]));
          f[2] = f[6] - C(2. / 3.) * uy0;
          f[1] = f[5] - C(1. / 6.) * uy0 + C(0.5) * (f[4] - f[8]);
          f[3] = f[7] - C(1. / 6.) * uy0 + C(0.5) * (f[8] - f[4]);
        } else {
          // south: the west operator rotated by +90 degrees
          C uy0 = rho0 - (f[0] + f[8] + f[4] + C(2.) * (f[1] + f[2] + f[3]));
          f[6] = f[2] + C(2. / 3.) * uy0;
          f[5] = f[1] + C(1. / 6.) * uy0 + C(0.5) * (f[8] - f[4]);
          f[7] = f[3] + C(1. / 6.) * uy0 + C(0.5) * (f[4] - f[8]);
        }
      } else {
        C ux = f[0] + f[1] + f[2] + f[4] + f[5] + f[10] + f[11] + f[13] + f[14] +
               C(2.) * (f[7] + f[9] + f[12] + f[15] + f[17]) - rho0;
        C Nyx = C(0.5) * (f[5] + f[11] + f[13] - (f[2] + f[4] + f[14]));
        C Nzx = C(0.5) * (f[10] + f[13] + f[14] - (f[1] + f[4] + f[5]));
        f[3] = f[12] - C(1. / 3.) * ux;
        f[6] = f[15] - C(1. / 6.) * ux + Nzx;
        f[8] = f[17] - C(1. / 6.) * ux + Nyx;
        f[16] = f[7] - C(1. / 6.) * ux - Nzx;
        f[18] = f[9] - C(1. / 6.) * ux - Nyx;
      }
    } else if (b.kind == LBM_BC_TEMPERATURE && LAT == LAT_D2Q9_D2Q5) {
      C* g = f + 9;
      g[4] = bc_scalar<C>(b, x, y, z) - g[0] - g[1] - g[2] - g[3];
    }
  }
}

// Transposes, applied in reverse order of the forward boundary loops
// (adjointBoundaryConditions/adjointZouHe2d.cc:5-112, adjointZouHe2d.hh:53-87,
// adjointHecht3d.cc:7-80, adjointThermalZouHe2d.hh:56-71); the south velocity
// and north/south pressure transposes follow from their forward operators.
template <int LAT, class C>
__device__ __forceinline__ void adjoint_bcs(C* a, int x, int y, int z, const KParams& p) {
  using L = Lattice<LAT>;
  for (int k = p.nbc - 1; k >= 0; --k) {
    const DevBC& b = p.bc[k];
    if (!in_box(b.box, x, y, z)) continue;
    if (L::DIM == 3) {
      if (b.kind == LBM_BC_VELOCITY && b.face == LBM_FACE_WEST) {
        a[1] += C(0.5) * (a[15] - a[7]);
        a[2] += C(0.5) * (a[17] - a[9]);
        a[3] += a[12];
        a[4] += C(0.5) * (a[15] + a[17] - (a[7] + a[9]));
        a[5] += C(0.5) * (a[9] + a[15] - (a[7] + a[17]));
        a[6] += a[15];
        a[8] += a[17];
        a[10] += C(0.5) * (a[7] - a[15]);
        a[11] += C(0.5) * (a[9] - a[17]);
        a[13] += C(0.5) * (a[7] + a[9] - (a[15] + a[17]));
        a[14] += C(0.5) * (a[7] + a[17] - (a[9] + a[15]));
        a[16] += a[7];
        a[18] += a[9];
        a[7] = a[9] = a[12] = a[15] = a[17] = C(0.);
      } else if (b.kind == LBM_BC_PRESSURE && b.face == LBM_FACE_EAST) {
        C adjUx = -C(1. / 3.) * a[3] - C(1. / 6.) * (a[6] + a[8] + a[16] + a[18]);
        a[0] += adjUx;
        a[1] += adjUx + C(0.5) * (a[16] - a[6]);
        a[2] += adjUx + C(0.5) * (a[18] - a[8]);
        a[4] += adjUx + C(0.5) * (a[16] + a[18] - (a[6] + a[8]));
        a[5] += adjUx + C(0.5) * (a[8] + a[16] - (a[6] + a[18]));
        a[7] += C(2.) * adjUx + a[16];
        a[9] += C(2.) * adjUx + a[18];
        a[10] += adjUx + C(0.5) * (a[6] - a[16]);
        a[11] += adjUx + C(0.5) * (a[8] - a[18]);
        a[12] += C(2.) * adjUx + a[3];
        a[13] += adjUx + C(0.5) * (a[6] + a[8] - (a[16] + a[18]));
        a[14] += adjUx + C(0.5) * (a[6] + a[18] - (a[8] + a[16]));
        a[15] += C(2.) * adjUx + a[6];
        a[17] += C(2.) * adjUx + a[8];
        a[3] = a[6] = a[8] = a[16] = a[18] = C(0.);
      }
      continue;
    }
    const bool pres = b.kind == LBM_BC_PRESSURE || b.kind == LBM_BC_PRESSURE_STANDARD;
    if (b.kind == LBM_BC_VELOCITY_STANDARD) {
      // AdjointStandardZouHeVelocityWest2d (adjointZouHe2d.hh:62-80)
      C ux, uy, uz;
      bc_velocity<C>(b, x, y, z, ux, uy, uz);
      C adjRho = (C(1. / 6) * (ux / (C(1.) - ux)) - C(0.5) * (uy / (C(1.) - ux))) * a[1] +
                 (C(1. / 6) * (ux / (C(1.) - ux)) + C(0.5) * (uy / (C(1.) - ux))) * a[7] +
                 C(2. / 3.) * (ux / (C(1.) - ux)) * a[8];
      a[0] += adjRho;
      a[2] += C(0.5) * (a[7] - a[1]) + adjRho;
      a[3] += a[7] + C(2.) * adjRho;
      a[4] += a[8] + C(2.) * adjRho;
      a[5] += a[1] + C(2.) * adjRho;
      a[6] += C(0.5) * (a[1] - a[7]) + adjRho;
      a[1] = a[7] = a[8] = C(0.);
    } else if (b.kind == LBM_BC_VELOCITY && b.face == LBM_FACE_WEST) {
      a[2] += C(0.5) * (a[7] - a[1]);
      a[3] += a[7];
      a[4] += a[8];
      a[5] += a[1];
      a[6] += C(0.5) * (a[1] - a[7]);
      a[1] = a[7] = a[8] = C(0.);
    } else if (b.kind == LBM_BC_VELOCITY && b.face == LBM_FACE_EAST) {
      a[1] += a[5];
      a[2] += C(0.5) * (a[5] - a[3]);
      a[6] += C(0.5) * (a[3] - a[5]);
      a[7] += a[3];
      a[8] += a[4];
      a[3] = a[4] = a[5] = C(0.);
    } else if (b.kind == LBM_BC_VELOCITY && b.face == LBM_FACE_NORTH) {
      a[4] += C(0.5) * (a[1] - a[3]);
      a[5] += a[1];
      a[6] += a[2];
      a[7] += a[3];
      a[8] += C(0.5) * (a[3] - a[1]);
      a[1] = a[2] = a[3] = C(0.);
    } else if (b.kind == LBM_BC_VELOCITY && b.face == LBM_FACE_SOUTH) {
      a[4] += C(0.5) * (a[7] - a[5]);
      a[3] += a[7];
      a[2] += a[6];
      a[1] += a[5];
      a[8] += C(0.5) * (a[5] - a[7]);
      a[5] = a[6] = a[7] = C(0.);
    } else if (pres && b.face == LBM_FACE_EAST) {
      C adjU = -C(1. / 6.) * a[3] - C(2. / 3.) * a[4] - C(1. / 6.) * a[5];
      a[0] += adjU;
      a[1] += C(2.) * adjU + a[5];
      a[2] += adjU + C(0.5) * (a[5] - a[3]);
      a[6] += adjU + C(0.5) * (a[3] - a[5]);
      a[7] += C(2.) * adjU + a[3];
      a[8] += C(2.) * adjU + a[4];
      a[3] = a[4] = a[5] = C(0.);
    } else if (pres && b.face == LBM_FACE_WEST) {
      C adjU = C(1. / 6.) * a[1] + C(1. / 6.) * a[7] + C(2. / 3.) * a[8];
      a[0] -= adjU;
      a[2] -= adjU - C(0.5) * (a[7] - a[1]);
      a[3] -= C(2.) * adjU - a[7];
      a[4] -= C(2.) * adjU - a[8];
      a[5] -= C(2.) * adjU - a[1];
      a[6] -= adjU - C(0.5) * (a[1] - a[7]);
      a[1] = a[7] = a[8] = C(0.);
    } else if (pres && b.face == LBM_FACE_NORTH) {
      C adjU = -C(1. / 6.) * a[1] - C(2. / 3.) * a[2] - C(1. / 6.) * a[3];
      a[0] += adjU;
      a[7] += C(2.) * adjU + a[3];
      a[8] += adjU + C(0.5) * (a[3] - a[1]);
      a[4] += adjU + C(0.5) * (a[1] - a[3]);
      a[5] += C(2.) * adjU + a[1];
      a[6] += C(2.) * adjU + a[2];
      a[1] = a[2] = a[3] = C(0.);
    } else if (pres && b.face == LBM_FACE_SOUTH) {
      C adjU = C(1. / 6.) * a[7] + C(1. / 6.) * a[5] + C(2. / 3.) * a[6];
      a[0] -= adjU;
      a[8] -= adjU - C(0.5) * (a[5] - a[7]);
      a[1] -= C(2.) * adjU - a[5];
      a[2] -= C(2.) * adjU - a[6];
      a[3] -= C(2.) * adjU - a[7];
      a[4] -= adjU - C(0.5) * (a[7] - a[5]);
      a[5] = a[6] = a[7] = C(0.);
    } else if (b.kind == LBM_BC_TEMPERATURE && b.face == LBM_FACE_WEST && LAT == LAT_D2Q9_D2Q5) {
      C* g = a + 9;
      g[0] -= g[4];
      g[1] -= g[4];
      g[2] -= g[4];
      g[3] -= g[4];
      g[4] = C(0.);
    }
  }
}

// ---------------------------------------------------------------------------
// Deterministic block + grid reduction of one value per thread: warps sum in
// the compute precision, per-warp partials are added in FP64, each block
// writes its FP64 partial, and the last block to finish sums the partials in
// a fixed order and writes *result.

template <class C>
__device__ __forceinline__ C warp_sum(C v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// bid / nblk: this block's index and the block count of its lattice.
template <class C>
__device__ __forceinline__ void grid_reduce_v(C v, const KParams& p, unsigned bid, unsigned nblk) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const int nthr = blockDim.x * blockDim.y;
  if (p.accumulate) {
    // Sum over time steps: every warp adds its own sum to its own slot
    // (block * warps per block + warp) once per launch, so neither a counter,
    // a fence nor a barrier is needed and the additions come in a fixed
    // order; warps whose cells contribute nothing (e.g. away from the
    // pressure-drop strips) skip the shuffle tree.  The add's result is
    // unused, so the warp does not wait for the slot's old value.
    if (__any_sync(0xffffffffu, v != C(0.))) {
      v = warp_sum(v);
      if ((tid & 31) == 0)
        atomicAdd(&p.partial[(size_t)bid * (size_t)(nthr >> 5) + (size_t)(tid >> 5)], (double)v);
    }
    return;
  }
  __syncthreads();   // the shared slots may still be read from a previous call
  // warps whose cells contribute nothing (e.g. away from the pressure-drop
  // strips) skip the shuffle tree
  if (__any_sync(0xffffffffu, v != C(0.))) v = warp_sum(v);
  if ((tid & 31) == 0) sh[tid >> 5] = (double)v;
  __syncthreads();
  if (tid == 0) {
    double s = 0.;
    for (int w = 0; w < (nthr + 31) / 32; ++w) s += sh[w];
    p.partial[bid] = s;
    __threadfence();
    unsigned prev = atomicAdd(p.counter, 1u);
    last = (prev == nblk - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc = 0.;
  for (unsigned i = tid; i < nblk; i += nthr) acc += ((volatile double*)p.partial)[i];
  acc = warp_sum(acc);
  __syncthreads();
  if ((tid & 31) == 0) sh[tid >> 5] = acc;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.;
    for (int w = 0; w < (nthr + 31) / 32; ++w) tot += sh[w];
    *p.result = tot;
    *p.counter = 0u;
  }
}

template <class C>
__device__ __forceinline__ void grid_reduce(C v, const KParams& p) {
  const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
  const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  grid_reduce_v(v, p, bid, nblk);
}

// ---------------------------------------------------------------------------
// Launch parameters of a batch of lattices advanced by one launch.

constexpr int kMaxBatch = LBM_MAX_BATCH;

// Rows of cells (blockDim.y apart) each thread of a batched step kernel
// advances: the lattice lookup and the parameter loads of a virtual block are
// shared by them.  A virtual block covers blockDim.x x (blockDim.y * rows)
// cells; the objective kernel keeps one row.
constexpr int kBatchRowsForward = 2, kBatchRowsReverse = 1;

struct BatchParams {
  int n;                        // lattices in the batch
  int start[kMaxBatch + 1];     // first virtual block of each lattice; start[n..kMaxBatch] = total
  int gx[kMaxBatch], gy[kMaxBatch];   // blocks along x and y of each lattice (z: one per plane)
  // ceil(2^32 / gx) and ceil(2^32 / gy) for batch_div, or 0 where the
  // multiply-high form does not apply (a divisor of 1, or a product n * d
  // that can reach 2^32)
  unsigned gxm[kMaxBatch], gym[kMaxBatch];
  KParams p[kMaxBatch];
};

// n / d by a multiply-high with m = ceil(2^32 / d): with 2^32 + e = m d
// (0 <= e < d) and n = q d + r, n m / 2^32 = q + r / d + n e / (d 2^32), whose
// floor is q whenever n e < 2^32, so whenever n d < 2^32.  m = 0 falls back
// to the division.
__device__ __forceinline__ unsigned batch_div(unsigned n, unsigned d, unsigned m) {
  return m ? __umulhi(n, m) : n / d;
}

// The m of batch_div: ceil(2^32 / d) when every numerator n < nmax gives
// n * d < 2^32 and d > 1, else 0.
__host__ __device__ inline unsigned batch_div_magic(unsigned long long d, unsigned long long nmax) {
  if (d < 2 || nmax * d >= (1ull << 32)) return 0u;
  return (unsigned)(((1ull << 32) + d - 1) / d);
}

}  // namespace lbm

// The objectives, one functor each (LBMacroFunctional), used by the step kernels.
#include "lbm_objectives.cuh"
