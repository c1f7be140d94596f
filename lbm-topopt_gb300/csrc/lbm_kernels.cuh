// lbm_kernels.cuh -- the GB300 kernels, templated on lattice, collision
// operator and storage precision.  Included by one .cu file per lattice, which
// instantiates them and fills an Ops table (lbm_ops.h).
//
// Forward step (one launch per time step t -> t+1), push form:
//   load f~_t(x) (aligned SoA), apply BC_t if t >= 1 (local to the cell),
//   objective F(f_t) partial, collide (+PBB, + temperature), push each
//   direction to x+e_q or bounce it back into (x, opp q)  ->  f~_{t+1}.
//   The stored state f~ is post-stream, pre-boundary; every reader applies
//   BC_t on load, which reproduces the reference's f_t exactly
//   (LBSolver::stream then boundaryComputations, LBSolver.cc:184-206).
// Reverse step at t, pull form (the transpose of the push):
//   lam_t^post(x,d) = eta_{t+1}(x+e_d, d) or eta_{t+1}(x, opp d) at walls,
//   reverse collision at f_t(x) (FP64 sensitivity accumulation), objective
//   source, boundary transposes  ->  eta_t(x) (aligned store).
#pragma once

#include "lbm_device.cuh"
#include "lbm_ops.h"

namespace lbm {

template <class S>
struct AdjT {
  using T = S;
};
template <>
struct AdjT<__half> {
  using T = float;   // FP16 population storage keeps FP32 adjoints
};

template <int LAT>
__device__ __forceinline__ long long nb_offset(int q, int nx, int ny) {
  using L = Lattice<LAT>;
  return (long long)L::ex(q) + (long long)L::ey(q) * nx + (long long)L::ez(q) * nx * ny;
}

template <int LAT>
__device__ __forceinline__ bool nb_inside(int q, int x, int y, int z, const KParams& p) {
  using L = Lattice<LAT>;
  const int sx = x + L::ex(q), sy = y + L::ey(q), sz = z + L::ez(q);
  return sx >= 0 && sy >= 0 && sz >= 0 && sx < p.nx && sy < p.ny && sz < p.nz;
}

template <int LAT, class S>
__device__ __forceinline__ void load_state(typename Store<S>::C* f, const S* fin, long long c,
                                           long long P) {
  using L = Lattice<LAT>;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) f[q] = Store<S>::ld(fin + q * P + c);
}

// f~ -> f (unshifted FP64 value of population q)
template <int LAT, class S>
__device__ __forceinline__ double to_abs(int q, typename Store<S>::C v) {
  using L = Lattice<LAT>;
  return (Store<S>::SHIFT && q < L::QF) ? (double)v + L::w(q) : (double)v;
}

template <int LAT, class S>
__device__ __forceinline__ typename Store<S>::C from_abs(int q, double v) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  return (Store<S>::SHIFT && q < L::QF) ? C(v - L::w(q)) : C(v);
}

// ---------------------------------------------------------------------------

template <int LAT, int COLL, class S>
__global__ void __launch_bounds__(256) k_forward(KParams p) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  using G = typename GammaT<S>::T;
  constexpr bool SHIFT = Store<S>::SHIFT;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double objv = 0.;
  if (x < p.nx && y < p.ny) {
    const long long c = ((long long)z * p.ny + y) * p.nx + x;
    const S* __restrict__ fin = (const S*)p.fin;
    S* __restrict__ fout = (S*)p.fout;
    C f[L::Q];
    load_state<LAT, S>(f, fin, c, p.P);
    if (p.apply_bc) apply_bcs<LAT, SHIFT>(f, x, y, z, p);
    const C g = C(((const G*)p.gamma)[c]);
    if (p.eval_obj) objv = objective_cell<LAT, SHIFT>(f, g, x, y, z, p);
    const C imult = C(0.5) * (C(p.pbb_scale) * bp(g, C(p.pbb_q)));
    C rho, jx, jy, jz;
    flow_collide<LAT, COLL>(f, imult, rho, jx, jy, jz, p);
    if (LAT == LAT_D2Q9_D2Q5) {
      C T;
      thermal_collide(f + 9, jx, jy, g, T, p);
    }
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      if (nb_inside<LAT>(q, x, y, z, p))
        Store<S>::st(fout + q * p.P + c + nb_offset<LAT>(q, p.nx, p.ny), f[q]);
      else
        Store<S>::st(fout + L::opp(q) * p.P + c, f[q]);
    }
  }
  if (p.eval_obj) grid_reduce(objv, p);
}

template <int LAT, int COLL, class S>
__global__ void __launch_bounds__(256) k_adjoint(KParams p) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  using G = typename GammaT<S>::T;
  using A = typename AdjT<S>::T;
  constexpr bool SHIFT = Store<S>::SHIFT;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const long long c = ((long long)z * p.ny + y) * p.nx + x;
  const A* __restrict__ lin = (const A*)p.lam_in;
  A* __restrict__ lout = (A*)p.lam_out;
  C lam[L::Q];
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    if (nb_inside<LAT>(q, x, y, z, p))
      lam[q] = C(lin[q * p.P + c + nb_offset<LAT>(q, p.nx, p.ny)]);
    else
      lam[q] = C(lin[L::opp(q) * p.P + c]);
  }
  C f[L::Q];
  load_state<LAT, S>(f, (const S*)p.fin, c, p.P);
  if (p.apply_bc) apply_bcs<LAT, SHIFT>(f, x, y, z, p);
  const C g = C(((const G*)p.gamma)[c]);
  const C imult = C(0.5) * (C(p.pbb_scale) * bp(g, C(p.pbb_q)));
  const C dimult = C(0.5) * (C(p.pbb_scale) * bp_diff(g, C(p.pbb_q)));
  C dg = C(0.);
  C uxR = C(0.), uyR = C(0.);
  if (LAT == LAT_D2Q9_D2Q5) {
    C rho, jx, jy, jz;
    flow_macros<LAT>(f, rho, jx, jy, jz);
    thermal_reverse(f + 9, lam + 9, jx, jy, g, uxR, uyR, dg, p);
  }
  flow_reverse<LAT, COLL>(f, lam, imult, dimult, dg, p);
  if (LAT == LAT_D2Q9_D2Q5) {
#pragma unroll
    for (int i = 0; i < 9; ++i) lam[i] += uxR * C(L::ex(i)) + uyR * C(L::ey(i));
  }
  if (p.eval_obj) objective_source<LAT, SHIFT>(f, g, lam, dg, x, y, z, p);
  if (p.apply_bc) adjoint_bcs<LAT>(lam, x, y, z, p);
#pragma unroll
  for (int q = 0; q < L::Q; ++q) lout[q * p.P + c] = A(lam[q]);
  p.sens[c] += (double)dg;
}

// Objective of the state f_t alone (the last step of a forward sweep).
template <int LAT, class S>
__global__ void __launch_bounds__(256) k_objective(KParams p) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  using G = typename GammaT<S>::T;
  constexpr bool SHIFT = Store<S>::SHIFT;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double v = 0.;
  if (x < p.nx && y < p.ny) {
    const long long c = ((long long)z * p.ny + y) * p.nx + x;
    C f[L::Q];
    load_state<LAT, S>(f, (const S*)p.fin, c, p.P);
    if (p.apply_bc) apply_bcs<LAT, SHIFT>(f, x, y, z, p);
    v = objective_cell<LAT, SHIFT>(f, C(((const G*)p.gamma)[c]), x, y, z, p);
  }
  grid_reduce(v, p);
}

// f~_0 = feq(macros) (IsoEquilibriumInitializationLoop2d, isothermalLBLoops2d.hh:264-285;
// ThermalFeq2d for the temperature lattice).
template <int LAT, class S>
__global__ void __launch_bounds__(256) k_init(KParams p, const double* __restrict__ mac) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const long long c = ((long long)z * p.ny + y) * p.nx + x;
  double rho = 1., u[3] = {0., 0., 0.}, T = 0.;
  if (mac) {
    const double* m = mac + c * L::NMAC;
    rho = m[0];
    u[0] = m[1];
    u[1] = m[2];
    if (L::DIM == 3) u[2] = m[3];
    if (LAT == LAT_D2Q9_D2Q5) T = m[3];
  }
  S* fo = (S*)p.fout;
  const double uSqr = (L::DIM == 3) ? u[0] * u[0] + u[1] * u[1] + u[2] * u[2]
                                    : u[0] * u[0] + u[1] * u[1];
  const double rl = Store<S>::SHIFT ? rho - 1. : rho;
#pragma unroll
  for (int i = 0; i < L::QF; ++i) {
    double sc = (L::DIM == 3) ? L::ex(i) * u[0] + L::ey(i) * u[1] + L::ez(i) * u[2]
                              : L::ex(i) * u[0] + L::ey(i) * u[1];
    double eq = L::w(i) * (rl + 3. * sc + 4.5 * sc * sc - 1.5 * uSqr);
    Store<S>::st(fo + i * p.P + c, C(eq));
  }
  if (LAT == LAT_D2Q9_D2Q5) {
#pragma unroll
    for (int i = 9; i < 14; ++i) {
      double sc = L::ex(i) * u[0] + L::ey(i) * u[1];
      Store<S>::st(fo + i * p.P + c, C(L::w(i) * T * (1. + 3. * sc)));
    }
  }
}

// f_t (with BC_t) -> host-order FP64 AoS
template <int LAT, class S>
__global__ void __launch_bounds__(256) k_export(KParams p, double* __restrict__ aos) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const long long c = ((long long)z * p.ny + y) * p.nx + x;
  C f[L::Q];
  load_state<LAT, S>(f, (const S*)p.fin, c, p.P);
  if (p.apply_bc) apply_bcs<LAT, Store<S>::SHIFT>(f, x, y, z, p);
#pragma unroll
  for (int q = 0; q < L::Q; ++q) aos[c * L::Q + q] = to_abs<LAT, S>(q, f[q]);
}

template <int LAT, class S>
__global__ void __launch_bounds__(256) k_import(KParams p, const double* __restrict__ aos) {
  using L = Lattice<LAT>;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const long long c = ((long long)z * p.ny + y) * p.nx + x;
  S* fo = (S*)p.fout;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) Store<S>::st(fo + q * p.P + c, from_abs<LAT, S>(q, aos[c * L::Q + q]));
}

// Macros of f_t: rho, jx, jy (, jz | T)
template <int LAT, class S>
__global__ void __launch_bounds__(256) k_macros(KParams p, double* __restrict__ mac) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const long long c = ((long long)z * p.ny + y) * p.nx + x;
  C f[L::Q];
  load_state<LAT, S>(f, (const S*)p.fin, c, p.P);
  if (p.apply_bc) apply_bcs<LAT, Store<S>::SHIFT>(f, x, y, z, p);
  C rho, jx, jy, jz;
  flow_macros<LAT>(f, rho, jx, jy, jz);
  double* m = mac + c * L::NMAC;
  m[0] = Store<S>::SHIFT ? 1. + (double)rho : (double)rho;
  m[1] = jx;
  m[2] = jy;
  if (L::DIM == 3) m[3] = jz;
  if (LAT == LAT_D2Q9_D2Q5) m[3] = (double)(f[9] + f[10] + f[11] + f[12] + f[13]);
}

// Adjoint of the post-collision state below the last reverse step: S^T eta.
template <int LAT, class S>
__global__ void __launch_bounds__(256) k_export_adjoint(KParams p, double* __restrict__ aos) {
  using L = Lattice<LAT>;
  using A = typename AdjT<S>::T;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const long long c = ((long long)z * p.ny + y) * p.nx + x;
  const A* lin = (const A*)p.lam_in;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    double v;
    if (nb_inside<LAT>(q, x, y, z, p))
      v = (double)lin[q * p.P + c + nb_offset<LAT>(q, p.nx, p.ny)];
    else
      v = (double)lin[L::opp(q) * p.P + c];
    aos[c * L::Q + q] = v;
  }
}

template <class G>
__global__ void k_gamma(const double* __restrict__ src, G* __restrict__ dst, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = G(src[i]);
}

// ---------------------------------------------------------------------------

template <int LAT, int COLL, class S>
struct OpsImpl {
  static void launch(int kind, dim3 grid, dim3 block, cudaStream_t st, const KParams& p,
                     double* aux) {
    switch (kind) {
      case K_FORWARD:
        k_forward<LAT, COLL, S><<<grid, block, 0, st>>>(p);
        break;
      case K_ADJOINT:
        k_adjoint<LAT, COLL, S><<<grid, block, 0, st>>>(p);
        break;
      case K_OBJECTIVE:
        k_objective<LAT, S><<<grid, block, 0, st>>>(p);
        break;
      case K_INIT:
        k_init<LAT, S><<<grid, block, 0, st>>>(p, aux);
        break;
      case K_EXPORT:
        k_export<LAT, S><<<grid, block, 0, st>>>(p, aux);
        break;
      case K_IMPORT:
        k_import<LAT, S><<<grid, block, 0, st>>>(p, aux);
        break;
      case K_MACROS:
        k_macros<LAT, S><<<grid, block, 0, st>>>(p, aux);
        break;
      case K_EXPORT_ADJ:
        k_export_adjoint<LAT, S><<<grid, block, 0, st>>>(p, aux);
        break;
      case K_GAMMA: {
        long long n = (long long)p.nx * p.ny * p.nz;
        k_gamma<typename GammaT<S>::T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
            aux, (typename GammaT<S>::T*)p.gamma, n);
        break;
      }
      default:
        break;
    }
  }
};

}  // namespace lbm
