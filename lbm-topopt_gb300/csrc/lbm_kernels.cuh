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

// Resident 256-thread blocks per SM requested from the compiler (register
// cap).  The FP32/FP16 step kernels are HBM-bound and need the warps to keep
// enough loads in flight: 5 blocks (48 registers) measured fastest for the
// D3Q19 MRT forward step and 4 (64 registers) for its adjoint; the D2Q9
// forward step fits 6 (42 registers, no spills: 4096x2048 step 0.1079 ->
// 0.1025 ms, the 8-channel batch's 0.0342 -> 0.0324 ms; 7 spills and is
// slower); the D3Q19 BGK adjoint in increment form needs more registers than
// 64 and gets 3 blocks (85); the FP64 kernels are FP64-throughput-bound on
// GB300 and keep all their registers.
template <int LAT, int COLL, class S>
struct Occupancy {
  static constexpr int fwd = (LAT == LAT_D2Q9) ? 6 : 5;
  static constexpr int adj = (LAT == LAT_D3Q19 && COLL == LBM_BGK) ? 3 : 4;
  // the register-lean reverse variant: one more resident block per SM (the
  // tuner picks it where the extra warps beat the spills, e.g. the D2Q9 BGK
  // adjoint on lattices larger than L2); the batched D2Q9 one takes two more
  // (6 blocks: the 8-channel batch's reverse step 0.0558 -> 0.0536 ms, while
  // the 4096x2048 single-lattice step went 0.2000 -> 0.2145 ms with it)
  static constexpr int adj_lean = adj + 1;
  static constexpr int adj_lean_batch = (LAT == LAT_D2Q9) ? adj + 2 : adj + 1;
  static constexpr bool has_lean = true;
};
template <int LAT, int COLL>
struct Occupancy<LAT, COLL, double> {
  static constexpr int fwd = 1, adj = 1, adj_lean = 1, adj_lean_batch = 1;
  static constexpr bool has_lean = false;
};

template <class S>
struct AdjT {
  using T = S;
};
template <>
struct AdjT<__half> {
  using T = float;   // FP16 population storage keeps FP32 adjoints
};

// Offset of the neighbour x + e_q in the SoA index (compile-time q).  All
// offsets are 32-bit: the host guarantees Q * P < 2^31.
template <int LAT, int q>
__device__ __forceinline__ int nb_offset(int sx, int sxy) {
  using L = Lattice<LAT>;
  return L::ex(q) + L::ey(q) * sx + L::ez(q) * sxy;
}

template <int LAT, int q>
__device__ __forceinline__ bool nb_inside(int x, int y, int z, const KParams& p) {
  using L = Lattice<LAT>;
  const int sx = x + L::ex(q), sy = y + L::ey(q), sz = z + L::ez(q);
  return sx >= 0 && sy >= 0 && sz >= 0 && sx < p.nx && sy < p.ny && sz < p.nz;
}

// Cells at least one cell away from every domain face: all neighbours exist.
template <int LAT>
__device__ __forceinline__ bool interior(int x, int y, int z, const KParams& p) {
  using L = Lattice<LAT>;
  bool in = x > 0 && x < p.nx - 1 && y > 0 && y < p.ny - 1;
  if (L::DIM == 3) in = in && z > 0 && z < p.nz - 1;
  return in;
}

// Whether every cell of the calling warp lies inside the lattice and one
// cell away from every face; all 32 lanes must call it together (the step
// kernels do so before any divergence).  With it (WARP below) the push and
// the pull take the per-direction tests for the whole warp when one of its
// cells needs them: the interior cells of a warp holding an x = 0 or
// x = nx-1 cell would otherwise wait through both paths.  The same stores
// either way.  The single-lattice 3D steps use it (256x128x128 duct, a
// quarter of the warps hold a face cell: forward 0.1068 -> 0.1036 ms in
// FP32, 0.0959 -> 0.0908 ms in FP16, reverse 0.1563 -> 0.1554 ms and 0.1487
// -> 0.1471 ms); on the 2D lattices and in the batched steps, where few warps
// hold a face cell, the vote cost more than it saved (batched forward step
// 0.0342 -> 0.0352 ms, 4096x2048 D2Q9 reverse step 0.2178 -> 0.2197 ms), so
// they test each lane where it pushes or pulls.
template <int LAT>
__device__ __forceinline__ bool warp_interior(int x, int y, int z, const KParams& p) {
  return __all_sync(0xffffffffu, x < p.nx && y < p.ny && interior<LAT>(x, y, z, p));
}

// The interior decision of the push and the pull: the warp's (WARP) or the
// cell's own.
template <int LAT, bool WARP>
__device__ __forceinline__ bool take_interior(bool warp_in, int x, int y, int z, const KParams& p) {
  if constexpr (WARP)
    return warp_in;
  else
    return interior<LAT>(x, y, z, p);
}

// Step kernels that decide the interior path per warp: the single-lattice 3D ones.
template <int LAT>
constexpr bool kWarpInterior = Lattice<LAT>::DIM == 3;

// Boundary conditions live on the x = 0 and x = nx-1 faces and, in 2D, on
// the y = 0 and y = ny-1 faces (checked when the handle is created; p.bc_y
// says whether any does), so other cells skip the boundary loop.
template <int LAT>
__device__ __forceinline__ bool on_bc_face(int x, int y, const KParams& p) {
  if (Lattice<LAT>::DIM == 3) return p.apply_bc && (x == 0 || x == p.nx - 1);
  return p.apply_bc && (x == 0 || x == p.nx - 1 || (p.bc_y && (y == 0 || y == p.ny - 1)));
}

template <int LAT, class S>
__device__ __forceinline__ void load_state(typename Store<S>::C* f, const S* __restrict__ fin,
                                           int c, int P) {
  using L = Lattice<LAT>;
  static_for<L::Q>([&](auto Q_) {
    constexpr int q = decltype(Q_)::value;
    f[q] = Store<S>::ld(fin + (q * P + c));
  });
}

// f~ -> f (unshifted FP64 value of population q)
template <int LAT, class S, int q>
__device__ __forceinline__ double to_abs(typename Store<S>::C v) {
  using L = Lattice<LAT>;
  if constexpr (Store<S>::SHIFT && q < L::QF) {
    return (double)v + L::w(q);
  } else {
    return (double)v;
  }
}

template <int LAT, class S, int q>
__device__ __forceinline__ typename Store<S>::C from_abs(double v) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  if constexpr (Store<S>::SHIFT && q < L::QF) {
    return C(v - L::w(q));
  } else {
    return C(v);
  }
}

// Push f[q] of cell c to its neighbour (or bounce it back into opp(q) of c).
// Interior cells take one branch with no per-direction tests.
// Values are either in the compute type (converted on store) or already in
// the storage type.
template <class S, class V>
__device__ __forceinline__ void put(S* ptr, V v) {
  if constexpr (std::is_same<S, V>::value)
    *ptr = v;
  else
    Store<S>::st(ptr, v);
}

template <int LAT, class S, class V>
__device__ __forceinline__ void push_all(const V* f, S* __restrict__ fout, int c, int x, int y,
                                         int z, bool in, const KParams& p) {
  using L = Lattice<LAT>;
  const int P = (int)p.P, sx = p.nx, sxy = p.nx * p.ny;
  if (in) {
    static_for<L::Q>([&](auto Q_) {
      constexpr int q = decltype(Q_)::value;
      put(fout + (q * P + c + nb_offset<LAT, q>(sx, sxy)), f[q]);
    });
  } else {
    static_for<L::Q>([&](auto Q_) {
      constexpr int q = decltype(Q_)::value;
      if (nb_inside<LAT, q>(x, y, z, p))
        put(fout + (q * P + c + nb_offset<LAT, q>(sx, sxy)), f[q]);
      else
        put(fout + (L::opp(q) * P + c), f[q]);
    });
  }
}

// Pull lam^post(x, q) = eta(x + e_q, q), or eta(x, opp q) at walls.
template <int LAT, class A, class C>
__device__ __forceinline__ void pull_all(C* lam, const A* __restrict__ lin, int c, int x, int y,
                                         int z, bool in, const KParams& p) {
  using L = Lattice<LAT>;
  const int P = (int)p.P, sx = p.nx, sxy = p.nx * p.ny;
  if (in) {
    static_for<L::Q>([&](auto Q_) {
      constexpr int q = decltype(Q_)::value;
      lam[q] = C(lin[q * P + c + nb_offset<LAT, q>(sx, sxy)]);
    });
  } else {
    static_for<L::Q>([&](auto Q_) {
      constexpr int q = decltype(Q_)::value;
      if (nb_inside<LAT, q>(x, y, z, p))
        lam[q] = C(lin[q * P + c + nb_offset<LAT, q>(sx, sxy)]);
      else
        lam[q] = C(lin[L::opp(q) * P + c]);
    });
  }
}

// ---------------------------------------------------------------------------

// Per-cell bodies, shared by the single-lattice kernels and the batched ones.

// Forward step of cell (x,y,z) = index c from its loaded state f~_t (in f,
// overwritten) and design value g; returns its objective contribution F(f_t).
// in: the warp's cells are all interior (warp_interior), read with WARP.
template <int LAT, int COLL, class S, bool WARP>
__device__ __forceinline__ typename Store<S>::C forward_cell_from(const KParams& p, int x, int y,
                                                                  int z, int c,
                                                                  typename Store<S>::C* f,
                                                                  typename Store<S>::C g, bool in) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  constexpr bool SHIFT = Store<S>::SHIFT;
  C objv = C(0.);
  {
    S* __restrict__ fout = (S*)p.fout;
    if (on_bc_face<LAT>(x, y, p)) apply_bcs<LAT, SHIFT>(f, x, y, z, p);
    if (p.eval_obj) objv = objective_cell<LAT, SHIFT>(f, g, x, y, z, p);
    const C imult = C(0.5) * (mp<C>(p).pbb_scale * bp(g, mp<C>(p).pbb_q));
    C rho, jx, jy, jz;
    if constexpr (SHIFT) {
      // FP32/FP16 storage: increments, rounded to the storage type without bias
      Dither rnd((unsigned)c, p.key_fwd);
      S o[L::Q];
      flow_collide_inc<LAT, COLL>(
          f, imult, rho, jx, jy, jz, p,
          [&](auto Q_, C dq) {
            constexpr int q = decltype(Q_)::value;
            o[q] = Round<S>::apply(f[q], dq, rnd);
          },
          [&](auto QA_, auto QB_, C da, C db) {
            constexpr int qa = decltype(QA_)::value, qb = decltype(QB_)::value;
            Round<S>::apply_pair(f[qa], f[qb], da, db, rnd, o[qa], o[qb]);
          });
      if constexpr (LAT == LAT_D2Q9_D2Q5)
        thermal_collide_inc(f + 9, jx, jy, g, p, [&](auto I_, C dq) {
          constexpr int q = decltype(I_)::value + 9;
          o[q] = Round<S>::apply(f[q], dq, rnd);
        });
      push_all<LAT, S>(o, fout, c, x, y, z, take_interior<LAT, WARP>(in, x, y, z, p), p);
    } else {
      flow_collide<LAT, COLL>(f, imult, rho, jx, jy, jz, p);
      if (LAT == LAT_D2Q9_D2Q5) {
        C T;
        thermal_collide(f + 9, jx, jy, g, T, p);
      }
      push_all<LAT, S>(f, fout, c, x, y, z, take_interior<LAT, WARP>(in, x, y, z, p), p);
    }
  }
  return objv;
}

// Forward step of cell (x,y,z); returns its objective contribution F(f_t).
// in: warp_interior of the calling warp, read with WARP.
template <int LAT, int COLL, class S, bool WARP>
__device__ __forceinline__ typename Store<S>::C forward_cell(const KParams& p, int x, int y, int z,
                                                             bool in) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  using G = typename GammaT<S>::T;
  C objv = C(0.);
  if (x < p.nx && y < p.ny) {
    const int c = (z * p.ny + y) * p.nx + x;
    C f[L::Q];
    load_state<LAT, S>(f, (const S*)p.fin, c, (int)p.P);
    objv = forward_cell_from<LAT, COLL, S, WARP>(p, x, y, z, c, f, C(((const G*)p.gamma)[c]), in);
  }
  return objv;
}

// dJ/dgamma(c) += dg, one addition per cell and launch either way: the same
// sum.  An atomic add whose result is unused lets the warp go on without
// waiting for the old FP64 value; a read-modify-write keeps the addition on
// the SM.  D3Q19 always takes the atomic (reverse step 0.1605 to 0.1558 ms on
// the 256x128x128 duct).  The 2D lattices take it where the reverse step's
// working set fits in L2 (p.sens_atomic, set by the host): on the 1024x512
// channel it made the step 5% faster, while on a 4096x2048 lattice, streaming
// from DRAM, it made it 2.5% slower.
template <int LAT>
__device__ __forceinline__ void add_sensitivity(double* sens, int c, double dg, int atomic) {
  if (LAT == LAT_D3Q19 || atomic)
    atomicAdd(sens + c, dg);
  else
    sens[c] += dg;
}

// Reverse step of cell (x,y,z); in: warp_interior of the calling warp, read
// with WARP.
template <int LAT, int COLL, class S, bool WARP>
__device__ __forceinline__ void adjoint_cell(const KParams& p, int x, int y, int z, bool in) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  using G = typename GammaT<S>::T;
  using A = typename AdjT<S>::T;
  constexpr bool SHIFT = Store<S>::SHIFT;
  if (x >= p.nx || y >= p.ny) return;
  const int c = (z * p.ny + y) * p.nx + x;
  const A* __restrict__ lin = (const A*)p.lam_in;
  A* __restrict__ lout = (A*)p.lam_out;
  C lam[L::Q];
  pull_all<LAT, A, C>(lam, lin, c, x, y, z, take_interior<LAT, WARP>(in, x, y, z, p), p);
  C f[L::Q];
  load_state<LAT, S>(f, (const S*)p.fin, c, (int)p.P);
  if (on_bc_face<LAT>(x, y, p)) apply_bcs<LAT, SHIFT>(f, x, y, z, p);
  const C g = C(((const G*)p.gamma)[c]);
  const C imult = C(0.5) * (mp<C>(p).pbb_scale * bp(g, mp<C>(p).pbb_q));
  const C dimult = C(0.5) * (mp<C>(p).pbb_scale * bp_diff(g, mp<C>(p).pbb_q));
  C dg = C(0.);
  C uxR = C(0.), uyR = C(0.);
  if constexpr (SHIFT && COLL == LBM_BGK) {
    // FP32 adjoints: increments, rounded without bias away from the boundary faces
    C d[L::Q];
    if constexpr (LAT == LAT_D2Q9_D2Q5) {
      C rho, jx, jy, jz;
      flow_macros<LAT>(f, rho, jx, jy, jz);
      thermal_reverse_inc(f + 9, lam + 9, d + 9, jx, jy, g, uxR, uyR, dg, p);
    }
    bgk_reverse_inc<LAT>(f, lam, d, imult, dimult, dg, p);
    if constexpr (LAT == LAT_D2Q9_D2Q5) {
      static_for<9>([&](auto I) {
        constexpr int i = decltype(I)::value;
        d[i] += e_dot<LAT, i>(uxR, uyR, C(0.));
      });
    }
    if (p.eval_obj) objective_source<LAT, SHIFT>(f, g, d, dg, x, y, z, p);
    if (on_bc_face<LAT>(x, y, p)) {
      static_for<L::Q>([&](auto Q_) {
        constexpr int q = decltype(Q_)::value;
        lam[q] += d[q];
      });
      adjoint_bcs<LAT>(lam, x, y, z, p);
      static_for<L::Q>([&](auto Q_) {
        constexpr int q = decltype(Q_)::value;
        lout[q * (int)p.P + c] = A(lam[q]);
      });
    } else {
      // flow pairs (k, k + HALF) share one draw and packed arithmetic; the
      // rest population and the temperature lattice round one by one
      Dither rnd((unsigned)c, p.key_adj);
      const int P = (int)p.P;
      lout[c] = Round<A>::apply(lam[0], d[0], rnd);
      static_for<L::HALF>([&](auto D_) {
        constexpr int k = decltype(D_)::value + 1, o = k + L::HALF;
        A a, b;
        Round<A>::apply_pair(lam[k], lam[o], d[k], d[o], rnd, a, b);
        lout[k * P + c] = a;
        lout[o * P + c] = b;
      });
      static_for<L::Q - L::QF>([&](auto T_) {
        constexpr int q = decltype(T_)::value + L::QF;
        lout[q * P + c] = Round<A>::apply(lam[q], d[q], rnd);
      });
    }
    add_sensitivity<LAT>(p.sens, c, (double)dg, p.sens_atomic);
    return;
  }
  if (LAT == LAT_D2Q9_D2Q5) {
    C rho, jx, jy, jz;
    flow_macros<LAT>(f, rho, jx, jy, jz);
    thermal_reverse(f + 9, lam + 9, jx, jy, g, uxR, uyR, dg, p);
  }
  flow_reverse<LAT, COLL>(f, lam, imult, dimult, dg, p);
  if constexpr (LAT == LAT_D2Q9_D2Q5) {
    static_for<9>([&](auto I) {
      constexpr int i = decltype(I)::value;
      lam[i] += e_dot<LAT, i>(uxR, uyR, C(0.));
    });
  }
  if (p.eval_obj) objective_source<LAT, SHIFT>(f, g, lam, dg, x, y, z, p);
  if (on_bc_face<LAT>(x, y, p)) adjoint_bcs<LAT>(lam, x, y, z, p);
  static_for<L::Q>([&](auto Q_) {
    constexpr int q = decltype(Q_)::value;
    lout[q * (int)p.P + c] = A(lam[q]);
  });
  add_sensitivity<LAT>(p.sens, c, (double)dg, p.sens_atomic);
}

// Objective of the state f_t at cell (x,y,z) alone.
template <int LAT, class S>
__device__ __forceinline__ typename Store<S>::C objective_only_cell(const KParams& p, int x, int y,
                                                                   int z) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  using G = typename GammaT<S>::T;
  constexpr bool SHIFT = Store<S>::SHIFT;
  C v = C(0.);
  if (x < p.nx && y < p.ny) {
    const int c = (z * p.ny + y) * p.nx + x;
    C f[L::Q];
    load_state<LAT, S>(f, (const S*)p.fin, c, (int)p.P);
    if (on_bc_face<LAT>(x, y, p)) apply_bcs<LAT, SHIFT>(f, x, y, z, p);
    v = objective_cell<LAT, SHIFT>(f, C(((const G*)p.gamma)[c]), x, y, z, p);
  }
  return v;
}

// Start of every time-step kernel.  The step kernels are launched with
// programmatic stream serialisation (launch_overlapped): their CTAs may be
// scheduled while the previous kernel in the stream drains its last wave.
// Each CTA lets the next launch proceed, then waits until the previous grid
// has completed and its writes are visible, before it touches memory.
__device__ __forceinline__ void step_prologue() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <int LAT, int COLL, class S>
__global__ void __launch_bounds__(256, Occupancy<LAT, COLL, S>::fwd) k_forward(KParams p) {
  step_prologue();
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  constexpr bool W = kWarpInterior<LAT>;
  const bool in = W ? warp_interior<LAT>(x, y, blockIdx.z, p) : false;
  const auto objv = forward_cell<LAT, COLL, S, W>(p, x, y, blockIdx.z, in);
  if (p.eval_obj) grid_reduce(objv, p);
}

template <int LAT, int COLL, class S, bool LEAN = false>
__global__ void __launch_bounds__(256, LEAN ? Occupancy<LAT, COLL, S>::adj_lean
                                            : Occupancy<LAT, COLL, S>::adj) k_adjoint(KParams p) {
  step_prologue();
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  constexpr bool W = kWarpInterior<LAT>;
  const bool in = W ? warp_interior<LAT>(x, y, blockIdx.z, p) : false;
  adjoint_cell<LAT, COLL, S, W>(p, x, y, blockIdx.z, in);
}

// Objective of the state f_t alone (the last step of a forward sweep).
template <int LAT, class S>
__global__ void __launch_bounds__(256) k_objective(KParams p) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  grid_reduce(objective_only_cell<LAT, S>(p, x, y, blockIdx.z), p);
}

// ---------------------------------------------------------------------------
// Batched kernels: one launch advances every lattice of a batch (uneven sizes,
// each with its own boundaries, design and objective).  The virtual blocks of
// all lattices are concatenated and the grid strides over them (the step
// kernels are launched with one block per virtual block, the objective kernel
// with the resident blocks), so small and large lattices share the SMs.
// Per-lattice parameters are read in place from the launch's parameter space.

// Lattice of virtual block vb: the number of lattice starts at or below it
// past the first.  The slots past the batch start at the total, and every
// start is read at a fixed offset of the parameter space, with no loop.
__device__ __forceinline__ int batch_lattice_of(const BatchParams& bp, int vb) {
  int i = 0;
  static_for<kMaxBatch - 1>([&](auto K) { i += vb >= bp.start[decltype(K)::value + 1] ? 1 : 0; });
  return i;
}

template <int LAT, int COLL, class S>
__global__ void __launch_bounds__(256, Occupancy<LAT, COLL, S>::fwd)
    k_forward_batch(const __grid_constant__ BatchParams bp) {
  step_prologue();
  for (int vb = blockIdx.x; vb < bp.start[kMaxBatch]; vb += gridDim.x) {
    const int i = batch_lattice_of(bp, vb);
    const KParams& p = bp.p[i];
    const int lb = vb - bp.start[i];
    const int r = (int)batch_div((unsigned)lb, (unsigned)bp.gx[i], bp.gxm[i]);
    const int bz = (int)batch_div((unsigned)r, (unsigned)bp.gy[i], bp.gym[i]);
    const int x = (lb - r * bp.gx[i]) * blockDim.x + threadIdx.x;
    const int y = (r - bz * bp.gy[i]) * (blockDim.y * kBatchRowsForward) + threadIdx.y;
    // the rows' contributions summed in FP64, as the partial sums they join
    // are: FP64 sums of FP32 values of similar size are exact, so the block
    // shape does not change them (and only where the objective is evaluated:
    // GB300's FP64 pipe is narrow)
    double objv = 0.;
#pragma unroll 1
    for (int k = 0; k < kBatchRowsForward; ++k) {
      const auto v = forward_cell<LAT, COLL, S, false>(p, x, y + k * (int)blockDim.y, bz, false);
      if (p.eval_obj) objv += (double)v;
    }
    if (p.eval_obj) grid_reduce_v(objv, p, lb, bp.start[i + 1] - bp.start[i]);
  }
}

template <int LAT, int COLL, class S, bool LEAN = false>
__global__ void __launch_bounds__(256, LEAN ? Occupancy<LAT, COLL, S>::adj_lean_batch
                                            : Occupancy<LAT, COLL, S>::adj)
    k_adjoint_batch(const __grid_constant__ BatchParams bp) {
  step_prologue();
  for (int vb = blockIdx.x; vb < bp.start[kMaxBatch]; vb += gridDim.x) {
    const int i = batch_lattice_of(bp, vb);
    const KParams& p = bp.p[i];
    const int lb = vb - bp.start[i];
    const int r = (int)batch_div((unsigned)lb, (unsigned)bp.gx[i], bp.gxm[i]);
    const int bz = (int)batch_div((unsigned)r, (unsigned)bp.gy[i], bp.gym[i]);
    const int x = (lb - r * bp.gx[i]) * blockDim.x + threadIdx.x;
    const int y = (r - bz * bp.gy[i]) * (blockDim.y * kBatchRowsReverse) + threadIdx.y;
#pragma unroll 1
    for (int k = 0; k < kBatchRowsReverse; ++k)
      adjoint_cell<LAT, COLL, S, false>(p, x, y + k * (int)blockDim.y, bz, false);
  }
}

template <int LAT, class S>
__global__ void __launch_bounds__(256) k_objective_batch(const __grid_constant__ BatchParams bp) {
  for (int vb = blockIdx.x; vb < bp.start[kMaxBatch]; vb += gridDim.x) {
    const int i = batch_lattice_of(bp, vb);
    const KParams& p = bp.p[i];
    const int lb = vb - bp.start[i];
    const int r = (int)batch_div((unsigned)lb, (unsigned)bp.gx[i], bp.gxm[i]);
    const int bz = (int)batch_div((unsigned)r, (unsigned)bp.gy[i], bp.gym[i]);
    const int x = (lb - r * bp.gx[i]) * blockDim.x + threadIdx.x;
    const int y = (r - bz * bp.gy[i]) * blockDim.y + threadIdx.y;
    const auto v = objective_only_cell<LAT, S>(p, x, y, bz);
    if (p.eval_obj) grid_reduce_v(v, p, lb, bp.start[i + 1] - bp.start[i]);
  }
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
  const int c = (z * p.ny + y) * p.nx + x;
  // in the compute type: FP64 for FP64 storage, FP32 otherwise (the FP64 pipe
  // made this FP32-state initialisation take 1.2 ms on the 4.2M-cell duct)
  C rl = Store<S>::SHIFT ? C(0.) : C(1.), u[3] = {C(0.), C(0.), C(0.)}, T = C(0.);
  if (mac) {
    const double* m = mac + (long long)c * L::NMAC;
    rl = Store<S>::SHIFT ? C(m[0] - 1.) : C(m[0]);
    u[0] = C(m[1]);
    u[1] = C(m[2]);
    if (L::DIM == 3) u[2] = C(m[3]);
    if (LAT == LAT_D2Q9_D2Q5) T = C(m[3]);
  }
  S* fo = (S*)p.fout;
  const C uSqr = (L::DIM == 3) ? u[0] * u[0] + u[1] * u[1] + u[2] * u[2] : u[0] * u[0] + u[1] * u[1];
  static_for<L::QF>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const C sc = e_dot<LAT, i>(u[0], u[1], u[2]);
    const C eq = C(L::w(i)) * (rl + C(3.) * sc + C(4.5) * sc * sc - C(1.5) * uSqr);
    Store<S>::st(fo + i * p.P + c, eq);
  });
  if constexpr (LAT == LAT_D2Q9_D2Q5) {
    static_for<5>([&](auto I) {
      constexpr int i = 9 + decltype(I)::value;
      const C sc = e_dot<LAT, i>(u[0], u[1], C(0.));
      Store<S>::st(fo + i * p.P + c, C(L::w(i)) * T * (C(1.) + C(3.) * sc));
    });
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
  const int c = (z * p.ny + y) * p.nx + x;
  C f[L::Q];
  load_state<LAT, S>(f, (const S*)p.fin, c, (int)p.P);
  if (on_bc_face<LAT>(x, y, p)) apply_bcs<LAT, Store<S>::SHIFT>(f, x, y, z, p);
  static_for<L::Q>([&](auto Q_) {
    constexpr int q = decltype(Q_)::value;
    aos[(long long)c * L::Q + q] = to_abs<LAT, S, q>(f[q]);
  });
}

template <int LAT, class S>
__global__ void __launch_bounds__(256) k_import(KParams p, const double* __restrict__ aos) {
  using L = Lattice<LAT>;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const int c = (z * p.ny + y) * p.nx + x;
  S* fo = (S*)p.fout;
  static_for<L::Q>([&](auto Q_) {
    constexpr int q = decltype(Q_)::value;
    Store<S>::st(fo + q * p.P + c, from_abs<LAT, S, q>(aos[(long long)c * L::Q + q]));
  });
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
  const int c = (z * p.ny + y) * p.nx + x;
  C f[L::Q];
  load_state<LAT, S>(f, (const S*)p.fin, c, (int)p.P);
  if (on_bc_face<LAT>(x, y, p)) apply_bcs<LAT, Store<S>::SHIFT>(f, x, y, z, p);
  C rho, jx, jy, jz;
  flow_macros<LAT>(f, rho, jx, jy, jz);
  double* m = mac + (long long)c * L::NMAC;
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
  const int c = (z * p.ny + y) * p.nx + x;
  const A* lin = (const A*)p.lam_in;
  double lam[L::Q];
  pull_all<LAT, A, double>(lam, lin, c, x, y, z, false, p);
  static_for<L::Q>([&](auto Q_) {
    constexpr int q = decltype(Q_)::value;
    aos[(long long)c * L::Q + q] = lam[q];
  });
}

// *bits = bit pattern of max |f_t - f_{t-1}| over every population of every
// cell, each state with its own step's boundary conditions applied on load
// (the reference compares post-boundary states, regenerator2d.cc:160-170).
// Non-negative doubles order like their bit patterns, so an integer atomicMax
// finds the maximum in any order; a NaN (pattern above every number) wins.
template <int LAT, class S>
__global__ void __launch_bounds__(256) k_max_change_bc(const KParams pc, const KParams pp,
                                                      unsigned long long* bits) {
  using L = Lattice<LAT>;
  using C = typename Store<S>::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double m = 0.;
  if (x < pc.nx && y < pc.ny) {
    const int c = (z * pc.ny + y) * pc.nx + x;
    C f[L::Q], g[L::Q];
    load_state<LAT, S>(f, (const S*)pc.fin, c, (int)pc.P);
    load_state<LAT, S>(g, (const S*)pp.fin, c, (int)pp.P);
    if (on_bc_face<LAT>(x, y, pc)) apply_bcs<LAT, Store<S>::SHIFT>(f, x, y, z, pc);
    if (on_bc_face<LAT>(x, y, pp)) apply_bcs<LAT, Store<S>::SHIFT>(g, x, y, z, pp);
    static_for<L::Q>([&](auto Q_) {
      constexpr int q = decltype(Q_)::value;
      const double d = fabs((double)f[q] - (double)g[q]);
      m = (d > m || d != d) ? d : m;
    });
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_down_sync(0xffffffffu, m, o);
    m = (v > m || v != v) ? v : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(bits, (unsigned long long)__double_as_longlong(m));
}

template <class G>
__global__ void k_gamma(const double* __restrict__ src, G* __restrict__ dst, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = G(src[i]);
}

// ---------------------------------------------------------------------------

// Launch of a kernel that begins with step_prologue, with programmatic stream
// serialisation allowed.
template <class K, class P>
void launch_overlapped(K kern, dim3 grid, dim3 block, cudaStream_t st, const P& arg) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, arg);
}

template <int LAT, int COLL, class S>
struct OpsImpl {
  static void launch_batch(int kind, dim3 grid, dim3 block, cudaStream_t st, const BatchParams& bp) {
    switch (kind) {
      case K_FORWARD:
        launch_overlapped(k_forward_batch<LAT, COLL, S>, grid, block, st, bp);
        break;
      case K_ADJOINT:
        launch_overlapped(k_adjoint_batch<LAT, COLL, S>, grid, block, st, bp);
        break;
      case K_ADJOINT_LEAN:
        launch_overlapped(k_adjoint_batch<LAT, COLL, S, Occupancy<LAT, COLL, S>::has_lean>, grid,
                          block, st, bp);
        break;
      case K_OBJECTIVE:
        k_objective_batch<LAT, S><<<grid, block, 0, st>>>(bp);
        break;
      default:
        break;
    }
  }
  static const void* kernel_address(int kind) {
    switch (kind) {
      case K_FORWARD:
        return (const void*)k_forward_batch<LAT, COLL, S>;
      case K_ADJOINT:
        return (const void*)k_adjoint_batch<LAT, COLL, S>;
      case K_ADJOINT_LEAN:
        return (const void*)k_adjoint_batch<LAT, COLL, S, Occupancy<LAT, COLL, S>::has_lean>;
      case K_OBJECTIVE:
        return (const void*)k_objective_batch<LAT, S>;
      default:
        return nullptr;
    }
  }
  static void max_change(dim3 grid, dim3 block, cudaStream_t st, const KParams& cur,
                         const KParams& prev, unsigned long long* bits) {
    k_max_change_bc<LAT, S><<<grid, block, 0, st>>>(cur, prev, bits);
  }
  static void launch(int kind, dim3 grid, dim3 block, cudaStream_t st, const KParams& p,
                     double* aux) {
    switch (kind) {
      case K_FORWARD:
        launch_overlapped(k_forward<LAT, COLL, S>, grid, block, st, p);
        break;
      case K_ADJOINT:
        launch_overlapped(k_adjoint<LAT, COLL, S>, grid, block, st, p);
        break;
      case K_ADJOINT_LEAN:
        launch_overlapped(k_adjoint<LAT, COLL, S, Occupancy<LAT, COLL, S>::has_lean>, grid, block,
                          st, p);
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
