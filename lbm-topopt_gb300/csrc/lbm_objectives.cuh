// lbm_objectives.cuh -- the objectives, one functor each: the GB300 form of
// the reference's LBMacroFunctional (functionals/LBMacroFunctional.hh:6-14).
//
// A functor has
//   id                        its LBM_OBJ_* code
//   uses                      which boxes of lbm_config it reads (kUsesIn / kUsesOut)
//   thermal                   whether it needs the temperature lattice
//   evaluate<LAT,SHIFT>(...)  weight * F of one cell            (evaluate)
//   source<LAT,SHIFT>(...)    lam += weight * dF/df,            (adjointCollideSource)
//                             dg  += weight * dF/dgamma          (adjointSensitivitySource)
// and is listed once in ObjectiveList below.  The step kernels call the one
// the launch names through a compile-time unrolled dispatch over the list, so
// an objective is fused into the forward and reverse steps like the built-in
// ones: adding one takes a functor, an LBM_OBJ_* code and a list entry.
//
// The weight w (timeConst of the reference) and the box normalisations reach
// the kernels precomputed in ModelParams: obj_weight = w, w_in = w/|in|,
// w_out = w/|out| in the compute precision.  On shifted storage (f - w_i) the
// populations' rest part is already removed: objectives linear in rho see
// rho - 1 and must cancel the constant themselves (the pressure drop does,
// weight*1 - weight*1 over its two means).
#pragma once

#include "lbm_device.cuh"

namespace lbm {

constexpr unsigned kUsesIn = 1u, kUsesOut = 2u;

// component a of e_i
template <class L>
__host__ __device__ constexpr int lat_e(int i, int a) {
  return a == 0 ? L::ex(i) : a == 1 ? L::ey(i) : L::ez(i);
}

// e_i^T P e_i for a symmetric 3x3 P, the zero terms left out (the rest in the
// order a, b = 0..DIM-1)
template <int LAT, int i, class C>
__device__ __forceinline__ C e_quad(const C (&P)[3][3]) {
  using L = Lattice<LAT>;
  C v = C(0.);
  static_for<L::DIM>([&](auto A) {
    constexpr int a = decltype(A)::value;
    static_for<L::DIM>([&](auto B) {
      constexpr int b = decltype(B)::value;
      constexpr int eab = lat_e<L>(i, a) * lat_e<L>(i, b);
      if constexpr (eab == 1) v += P[a][b];
      if constexpr (eab == -1) v -= P[a][b];
    });
  });
  return v;
}

// P_ab = sum_i e_ia e_ib f_i over the flow lattice
template <int LAT, class C>
__device__ __forceinline__ void second_moment(const C* f, C (&P)[3][3]) {
  using L = Lattice<LAT>;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) P[a][b] = C(0.);
  static_for<L::QF>([&](auto I) {
    constexpr int i = decltype(I)::value;
    static_for<L::DIM>([&](auto A) {
      constexpr int a = decltype(A)::value;
      static_for<L::DIM>([&](auto B) {
        constexpr int b = decltype(B)::value;
        constexpr int eab = lat_e<L>(i, a) * lat_e<L>(i, b);
        if constexpr (eab == 1) P[a][b] += f[i];
        if constexpr (eab == -1) P[a][b] -= f[i];
      });
    });
  });
}

// lam_d -= v * e_dx over the flow populations: the source of -v * u_x with
// u = j (incompressible)
template <int LAT, class C>
__device__ __forceinline__ void minus_ex_source(C* lam, C v) {
  using L = Lattice<LAT>;
  static_for<L::QF>([&](auto D) {
    constexpr int d = decltype(D)::value;
    if constexpr (L::ex(d) == 1) lam[d] -= v;
    if constexpr (L::ex(d) == -1) lam[d] += v;
  });
}

// PressureDrop2d (functionals/pressureDrop2d.hh:30-68): w (mean rho over the
// inflow box - mean rho over the outflow box); 3D the same over faces.
struct ObjPressureDrop {
  static constexpr int id = LBM_OBJ_PRESSURE_DROP;
  static constexpr unsigned uses = kUsesIn | kUsesOut;
  static constexpr bool thermal = false;
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ C evaluate(const C* f, C, int x, int y, int z,
                                               const KParams& p) {
    bool i1 = in_box(p.obj_in, x, y, z), i2 = in_box(p.obj_out, x, y, z);
    if (!i1 && !i2) return C(0.);
    C rho, jx, jy, jz;
    flow_macros<LAT>(f, rho, jx, jy, jz);
    C v = C(0.);
    if (i1) v += mp<C>(p).w_in * rho;
    if (i2) v -= mp<C>(p).w_out * rho;
    return v;
  }
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ void source(const C*, C, C* lam, C&, int x, int y, int z,
                                                const KParams& p) {
    using L = Lattice<LAT>;
    if (in_box(p.obj_in, x, y, z)) {
      const C v = mp<C>(p).w_in;
#pragma unroll
      for (int d = 0; d < L::QF; ++d) lam[d] += v;
    }
    if (in_box(p.obj_out, x, y, z)) {
      const C v = mp<C>(p).w_out;
#pragma unroll
      for (int d = 0; d < L::QF; ++d) lam[d] -= v;
    }
  }
};

// OutflowEast2d (functionals/outflow2d.hh:15-54): -w (mean u_x over the
// outflow box).
struct ObjOutflow {
  static constexpr int id = LBM_OBJ_OUTFLOW;
  static constexpr unsigned uses = kUsesOut;
  static constexpr bool thermal = false;
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ C evaluate(const C* f, C, int x, int y, int z,
                                               const KParams& p) {
    if (!in_box(p.obj_out, x, y, z)) return C(0.);
    C rho, jx, jy, jz;
    flow_macros<LAT>(f, rho, jx, jy, jz);
    return -mp<C>(p).w_out * jx;
  }
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ void source(const C*, C, C* lam, C&, int x, int y, int z,
                                                const KParams& p) {
    if (in_box(p.obj_out, x, y, z)) minus_ex_source<LAT>(lam, mp<C>(p).w_out);
  }
};

// ThroughFlow2d (functionals/throughFlow2d.hh:17-83), the objective of the
// robust pump (applications/RobustPump2d/robustPump2d.cc:165-166):
// -w (mean u_x over the inflow box + mean u_x over the outflow box).
struct ObjThroughFlow {
  static constexpr int id = LBM_OBJ_THROUGH_FLOW;
  static constexpr unsigned uses = kUsesIn | kUsesOut;
  static constexpr bool thermal = false;
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ C evaluate(const C* f, C, int x, int y, int z,
                                               const KParams& p) {
    bool i1 = in_box(p.obj_in, x, y, z), i2 = in_box(p.obj_out, x, y, z);
    if (!i1 && !i2) return C(0.);
    C rho, jx, jy, jz;
    flow_macros<LAT>(f, rho, jx, jy, jz);
    C v = C(0.);
    if (i1) v -= mp<C>(p).w_in * jx;
    if (i2) v -= mp<C>(p).w_out * jx;
    return v;
  }
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ void source(const C*, C, C* lam, C&, int x, int y, int z,
                                                const KParams& p) {
    if (in_box(p.obj_in, x, y, z)) minus_ex_source<LAT>(lam, mp<C>(p).w_in);
    if (in_box(p.obj_out, x, y, z)) minus_ex_source<LAT>(lam, mp<C>(p).w_out);
  }
};

// ThermalOutflowEast2d (functionals/temperatureFlow2d.hh:18-52): -w sum u_x T
// over the outflow box.
struct ObjHeatFlux {
  static constexpr int id = LBM_OBJ_HEAT_FLUX;
  static constexpr unsigned uses = kUsesOut;
  static constexpr bool thermal = true;
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ C evaluate(const C* f, C, int x, int y, int z,
                                               const KParams& p) {
    if constexpr (LAT != LAT_D2Q9_D2Q5) {
      return C(0.);
    } else {
      if (!in_box(p.obj_out, x, y, z)) return C(0.);
      C rho, jx, jy, jz;
      flow_macros<LAT>(f, rho, jx, jy, jz);
      C T = f[9] + f[10] + f[11] + f[12] + f[13];
      return -mp<C>(p).obj_weight * jx * T;
    }
  }
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ void source(const C* f, C, C* lam, C&, int x, int y, int z,
                                                const KParams& p) {
    if constexpr (LAT == LAT_D2Q9_D2Q5) {
      using L = Lattice<LAT>;
      if (in_box(p.obj_out, x, y, z)) {
        C rho, jx, jy, jz;
        flow_macros<LAT>(f, rho, jx, jy, jz);
        C T = f[9] + f[10] + f[11] + f[12] + f[13];
        const C tc = mp<C>(p).obj_weight;
        static_for<9>([&](auto D) {
          constexpr int d = decltype(D)::value;
          lam[d] -= tc * C(L::ex(d)) * T;
        });
#pragma unroll
        for (int d = 9; d < 14; ++d) lam[d] -= tc * jx;
      }
    }
  }
};

// Dissipated power (no reference counterpart), over the whole lattice:
// D = 2 alpha |j|^2 + (9/2) nu omega^2 sum_ab Pneq_ab^2 with
// Pneq = sum_i e_i e_i f_i - rho/3 I - j j, alpha = 0.5 interp_scale BP_q(gamma),
// nu = (1/omega - 1/2)/3 (cv_diss = (9/2) nu omega^2, set by the host).
struct ObjDissipation {
  static constexpr int id = LBM_OBJ_DISSIPATION;
  static constexpr unsigned uses = 0;
  static constexpr bool thermal = false;
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ C evaluate(const C* f, C g, int, int, int,
                                               const KParams& p) {
    using L = Lattice<LAT>;
    C rho, j[3];
    flow_macros<LAT>(f, rho, j[0], j[1], j[2]);
    C P[3][3];
    second_moment<LAT>(f, P);
    C s2 = C(0.);
#pragma unroll
    for (int a = 0; a < L::DIM; ++a) {
#pragma unroll
      for (int b = 0; b < L::DIM; ++b) {
        C v = P[a][b] - j[a] * j[b];
        if (a == b) v -= rho / C(3.);
        s2 += v * v;
      }
    }
    const C cv = mp<C>(p).cv_diss;
    const C alpha = C(0.5) * (mp<C>(p).pbb_scale * bp(g, mp<C>(p).pbb_q));
    C jj = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    return mp<C>(p).obj_weight * (C(2.) * alpha * jj + cv * s2);
  }
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ void source(const C* f, C g, C* lam, C& dg, int, int, int,
                                                const KParams& p) {
    using L = Lattice<LAT>;
    C rho, j[3];
    flow_macros<LAT>(f, rho, j[0], j[1], j[2]);
    C P[3][3];
    second_moment<LAT>(f, P);
    C tr = C(0.);
#pragma unroll
    for (int a = 0; a < L::DIM; ++a) {
#pragma unroll
      for (int b = 0; b < L::DIM; ++b) P[a][b] -= j[a] * j[b];
      P[a][a] -= rho / C(3.);
      tr += P[a][a];
    }
    // P j once; per population only the lattice vector's nonzero components
    // (products with a zero component are not folded away in IEEE arithmetic)
    C pj[3] = {C(0.), C(0.), C(0.)};
#pragma unroll
    for (int a = 0; a < L::DIM; ++a)
#pragma unroll
      for (int b = 0; b < L::DIM; ++b) pj[a] += P[a][b] * j[b];
    const C cv = mp<C>(p).cv_diss;
    const C alpha = C(0.5) * (mp<C>(p).pbb_scale * bp(g, mp<C>(p).pbb_q));
    const C tc = mp<C>(p).obj_weight;
    const C a4 = C(4.) * alpha, c2 = cv * C(2.), tr3 = tr / C(3.);
    static_for<L::QF>([&](auto I) {
      constexpr int i = decltype(I)::value;
      const C ej = e_dot<LAT, i>(j[0], j[1], j[2]);
      const C pej = e_dot<LAT, i>(pj[0], pj[1], pj[2]);   // e . P j
      const C pe = e_quad<LAT, i>(P);                     // e . P e
      lam[i] += tc * (a4 * ej + c2 * ((pe - tr3) - C(2.) * pej));
    });
    C jj = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    dg += tc * (C(2.) * (C(0.5) * (mp<C>(p).pbb_scale * bp_diff(g, mp<C>(p).pbb_q))) * jj);
  }
};

// DomainTemperature2d (functionals/domainTemperature2d.hh:13-40): w (mean T
// over the box).
struct ObjDomainTemperature {
  static constexpr int id = LBM_OBJ_DOMAIN_TEMPERATURE;
  static constexpr unsigned uses = kUsesOut;
  static constexpr bool thermal = true;
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ C evaluate(const C* f, C, int x, int y, int z,
                                               const KParams& p) {
    if constexpr (LAT != LAT_D2Q9_D2Q5) {
      return C(0.);
    } else {
      if (!in_box(p.obj_out, x, y, z)) return C(0.);
      return mp<C>(p).w_out * (f[9] + f[10] + f[11] + f[12] + f[13]);
    }
  }
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ void source(const C*, C, C* lam, C&, int x, int y, int z,
                                                const KParams& p) {
    if constexpr (LAT == LAT_D2Q9_D2Q5) {
      if (in_box(p.obj_out, x, y, z)) {
        const C v = mp<C>(p).w_out;
#pragma unroll
        for (int d = 9; d < 14; ++d) lam[d] += v;
      }
    }
  }
};

// RegeneratorEfficiency2d (functionals/regeneratorEfficiency2d.hh:16-88):
// J_t = w sum (1-gamma)(T - Ti) / D over the box, D = sum (1-gamma)(Tb - Ti)
// (design-dependent, computed by the host when the design is set; obj_p[1] =
// w/D).  The per-cell parts are here; the derivative of 1/D (dD/dgamma_c =
// -(Tb - Ti) in the box) gives every box cell the same term J (Tb - Ti)/D,
// which the host adds once per reverse sweep (or per reverse step) from J.
// The reference's adjoint sources use timeConst where the evaluate uses
// none and vice versa (adjointCollideSource divides by timeConst * D,
// adjointSensitivitySource leaves timeConst off the -(T - Ti) D term); they
// equal these derivatives only for timeConst = 1.
struct ObjRegeneratorEfficiency {
  static constexpr int id = LBM_OBJ_REGENERATOR_EFFICIENCY;
  static constexpr unsigned uses = kUsesOut;
  static constexpr bool thermal = true;
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ C evaluate(const C* f, C g, int x, int y, int z,
                                               const KParams& p) {
    if constexpr (LAT != LAT_D2Q9_D2Q5) {
      return C(0.);
    } else {
      if (!in_box(p.obj_out, x, y, z)) return C(0.);
      const C T = f[9] + f[10] + f[11] + f[12] + f[13];
      return mp<C>(p).obj_p[1] * ((C(1.) - g) * (T - mp<C>(p).obj_p[0]));
    }
  }
  template <int LAT, bool SHIFT, class C>
  static __device__ __forceinline__ void source(const C* f, C g, C* lam, C& dg, int x, int y,
                                                int z, const KParams& p) {
    if constexpr (LAT == LAT_D2Q9_D2Q5) {
      if (in_box(p.obj_out, x, y, z)) {
        const C wd = mp<C>(p).obj_p[1];
        const C v = wd * (C(1.) - g);
#pragma unroll
        for (int d = 9; d < 14; ++d) lam[d] += v;
        const C T = f[9] + f[10] + f[11] + f[12] + f[13];
        dg -= wd * (T - mp<C>(p).obj_p[0]);
      }
    }
  }
};

template <class... Os>
struct ObjList {};

// Every objective the kernels know.  Append a functor here to add one.
using ObjectiveList = ObjList<ObjPressureDrop, ObjDissipation, ObjHeatFlux, ObjOutflow,
                              ObjThroughFlow, ObjDomainTemperature, ObjRegeneratorEfficiency>;

// Host-side facts about an objective (validation, box normalisation).
struct ObjectiveInfo {
  int id;
  unsigned uses;
  bool thermal;
};

template <class... Os>
constexpr int objective_count(ObjList<Os...>) {
  return (int)sizeof...(Os);
}

template <class... Os>
__host__ __device__ constexpr ObjectiveInfo objective_info_at(ObjList<Os...>, int k) {
  constexpr ObjectiveInfo all[] = {ObjectiveInfo{Os::id, Os::uses, Os::thermal}...};
  return all[k];
}

// The `||` fold stops at the objective that matches: the ones after it cost
// no comparison (a `,` fold would test every entry at every cell).
template <int LAT, bool SHIFT, class C, class... Os>
__device__ __forceinline__ C objective_dispatch(ObjList<Os...>, const C* f, C g, int x, int y,
                                                int z, const KParams& p) {
  C v = C(0.);
  (void)((p.objective == Os::id &&
          (v = Os::template evaluate<LAT, SHIFT>(f, g, x, y, z, p), true)) ||
         ...);
  return v;
}

template <int LAT, bool SHIFT, class C, class... Os>
__device__ __forceinline__ void source_dispatch(ObjList<Os...>, const C* f, C g, C* lam, C& dg,
                                                int x, int y, int z, const KParams& p) {
  (void)((p.objective == Os::id &&
          (Os::template source<LAT, SHIFT>(f, g, lam, dg, x, y, z, p), true)) ||
         ...);
}

// Weighted objective of one cell, in the compute precision.
template <int LAT, bool SHIFT, class C>
__device__ __forceinline__ C objective_cell(const C* f, C g, int x, int y, int z,
                                            const KParams& p) {
  return objective_dispatch<LAT, SHIFT>(ObjectiveList{}, f, g, x, y, z, p);
}

// lam += weight * dF/df ; dg += weight * dF/dgamma
template <int LAT, bool SHIFT, class C>
__device__ __forceinline__ void objective_source(const C* f, C g, C* lam, C& dg, int x, int y,
                                                 int z, const KParams& p) {
  source_dispatch<LAT, SHIFT>(ObjectiveList{}, f, g, lam, dg, x, y, z, p);
}

}  // namespace lbm
