/*
 * ref_harness.cpp -- drives the reference's own operator and loop classes,
 * compiled in place from the reference sources against oracle/ref_shim, with
 * the same entry points as the C restatement (lbm_oracle.h, prefix ref_
 * instead of orc_).  TEST INFRASTRUCTURE ONLY: it exists to pin the
 * restatement to the reference and to generate golden vectors; it is built
 * into oracle/_ref/ only where the reference tree is present.
 *
 * Reference code used unmodified: lattices2d/3d, interpolationFunctions,
 * IncompressibleBGK2d<D2Q9>, IncompressibleMRT2d<D2Q9>, IncompressibleMRT3d<D3Q19>,
 * PartialBouncebackCollision + ReversePartialBouncebackCollision,
 * ReverseIncompressibleBGK2d/MRT2d/MRT3d, ObstIsoCollisionLoop2d, IsoStreamLoop2d,
 * IsoEquilibriumInitializationLoop2d, SourceAdjointObstIsoCollisionLoop2d,
 * AdjointIsoStreamingLoop2d, the incompressible Zou-He boundary loops and their
 * adjoints, WangCheckpointing + DynamicCheckpointing; for the thermal double
 * distribution, ThermalDualCollision over PartialBouncebackCollision<BGK2d> and
 * ThermalObstacleCollision<ThermalBGK2d<D2Q5>, RampInterpolation> with its
 * getSourceAdjoint() operator (ReverseThermalDualCollision /
 * ReverseThermalObstacleCollision / ReverseThermalBGK2d),
 * SourceAdjointObstThermalCollisionLoop2d, ThermalFeq2d and
 * AdjointThermalZouHeWest2d<D2Q9,D2Q5>.
 * Written out here because the reference does not compile them at HEAD: the 3D pull
 * stream and its transpose (a generalisation of isothermalLBLoops2d.hh:65-86 and
 * adjointIsothermalLBLoops2d.hh:139-163), the Hecht boundaries (Hecht3d.hh overrides a
 * two-argument execute) and their adjoints (adjointHecht3d.hh:35 does not parse), and
 * the functionals' evaluate/adjointCollideSource (they need the PETSc DMDA solver); for
 * the thermal lattice also the pull stream with mid-way bounce-back (the reference's
 * thermal stream loops, dynamics/thermalStreamingLoop2d.hh:27-63, leave off-domain
 * directions to explicit bounce-back boundaries), the forward ThermalZouHeWest2d
 * (thermalZouHe2d.hh:68-80 overrides a two-argument execute) and
 * ThermalOutflowEast2d (functionals/temperatureFlow2d.hh:18-54).
 */
#include "petsc.h"

#include "latticeBoltzmann/lattices2d.hh"
#include "latticeBoltzmann/lattices3d.hh"
#include "core/interpolationFunctions.hh"
#include "dynamics/incompressibleBGK2d.hh"
#include "dynamics/incompressibleMRT2d.hh"
#include "dynamics/partialBouncebackCollision.hh"
#include "dynamics/thermalBGK2d.hh"
#include "dynamics/thermalObstacleCollision.hh"
#include "dynamics/thermalDualCollision.hh"
#include "dynamics/isothermalLBLoops2d.hh"
#include "adjointDynamics/adjointThermalLBLoops2d.hh"
#include "adjointBoundaryConditions/adjointThermalZouHe2d.hh"
#include "adjointDynamics/adjointIsothermalLBLoops2d.hh"
#include "boundaryConditions/ZouHe2d.hh"
#include "dynamics/equilibriumDistributions3d.hh"
#include "dynamics/MRT3d.hh"
#include "adjointDynamics/reverseMRT3d.hh"
#include "topOpt/dynamicCheckpointing.hh"
#include "topOpt/staticCheckpointing.hh"
#include "topOpt/MMA.hh"

#include "../include/lbmgpu.h"

#include <cstdint>
#include <memory>
#include <vector>

namespace {

/* alpha(gamma) scaling of the reference's BP interpolation: PBB multiplies
 * interp(gamma) by 0.5 (partialBouncebackCollision.hh:58). */
struct ScaledBP {
  BPInterpolation<> bp;
  double scale;
  ScaledBP() : bp(), scale(1.) {}
  ScaledBP(double q, double s) : bp(q), scale(s) {}
  double operator()(double s) const { return scale * bp(s); }
  double diff(double s) const { return scale * bp.diff(s); }
  /* declared so PartialBouncebackCollision's CoDiPack signature parses; never called */
  ScaledBP getCodiAdjoint() const { return *this; }
};

struct Cfg3Constants {
  static constexpr PetscScalar s1 = 1.2, s2 = 1.2, s4 = 1.2, s10 = 1.2, s16 = 1.2;
  static constexpr PetscScalar we = 3., wej = -5.5, wxx = -0.5;
};

/* IncompressibleMRT3d lacks the LatticeType/getSourceAdjoint members that
 * PartialBouncebackCollision requires; this adapter adds them. */
template <class C>
struct MRT3dAdapter : public IncompressibleMRT3d<D3Q19, double, C> {
  using Base = IncompressibleMRT3d<D3Q19, double, C>;
  using LatticeType = D3Q19;
  static constexpr PetscInt numAdditionalFields = 0;
  double om;
  MRT3dAdapter() : Base(1.), om(1.) {}
  explicit MRT3dAdapter(double o) : Base(o), om(o) {}
  MRT3dAdapter getCodiAdjoint() const { return *this; }
  ReverseIncompressibleMRT3d<D3Q19, double, C> getSourceAdjoint() const {
    return ReverseIncompressibleMRT3d<D3Q19, double, C>(om);
  }
};

double time_factor(const lbm_bc& b, int t) {
  if (b.time_law == LBM_TIME_SINE) return b.amp == 0. ? 0. : b.amp * sin(2. * M_PI * (double)t / b.period);
  if (b.amp == 0.) return 1.;
  return 1. + b.amp * sin(2. * M_PI * (double)t / b.period);
}

/* parabola across the lattice along the face (s = y on west/east faces, x on
 * south/north faces), times the same in z in 3D */
double profile(const lbm_config& c, const lbm_bc& b, int x, int y, int z) {
  if (b.profile != LBM_PROFILE_PARABOLIC) return 1.;
  const bool yface = b.face == LBM_FACE_SOUTH || b.face == LBM_FACE_NORTH;
  const int n = yface ? c.nx : c.ny, s = yface ? x : y;
  double mid = (double)(n - 1) / 2.;
  double p = (mid * mid - (s - mid) * (s - mid)) / (mid * mid);
  if (c.lattice == LBM_D3Q19) {
    double mz = (double)(c.nz - 1) / 2.;
    p *= (mz * mz - (z - mz) * (z - mz)) / (mz * mz);
  }
  return p;
}

/* Tabulated inputs per boundary slot (the library's lbm_set_bc_profile): nt
 * rows of npos cells of ncomp values, cells along the face. */
struct Table {
  std::vector<double> v;
  int nt = 0, ncomp = 0;
  long long npos = 0;
};
Table g_tables[LBM_MAX_BC];

const double* table_entry(const lbm_bc& b, int k, int t, int i, int j) {
  if (b.profile != LBM_PROFILE_TABLE) return nullptr;
  const Table& tb = g_tables[k];
  if (tb.v.empty()) throw 4;
  const bool yface = b.face == LBM_FACE_SOUTH || b.face == LBM_FACE_NORTH;
  const long long pos = yface ? i - b.box[0] : j - b.box[2];
  return tb.v.data() + ((long long)(t % tb.nt) * tb.npos + pos) * tb.ncomp;
}

/* The Input functors the reference's Zou-He loops call (ZouHe2d.hh:37):
 * velocity value * T(t) * profile * dir (or a tabulated vector), density
 * value * T(t) (times a tabulated factor). */
struct VelFunc {
  lbm_config c;
  lbm_bc b;
  int k;
  void operator()(PetscInt t, PetscInt i, PetscInt j, PetscScalar& ux, PetscScalar& uy) const {
    const double* e = table_entry(b, k, (int)t, (int)i, (int)j);
    if (e && g_tables[k].ncomp >= 2) {
      ux = e[0];
      uy = e[1];
      return;
    }
    double v = b.value * time_factor(b, t);
    v *= e ? e[0] : profile(c, b, i, j, 0);
    const bool nodir = b.dir[0] == 0. && b.dir[1] == 0. && b.dir[2] == 0.;
    ux = v * (nodir ? 1. : b.dir[0]);
    uy = v * (nodir ? 0. : b.dir[1]);
  }
};

struct PresFunc {
  lbm_config c;
  lbm_bc b;
  int k;
  void operator()(PetscInt t, PetscInt i, PetscInt j, PetscScalar& rho) const {
    rho = b.value * time_factor(b, t);
    const double* e = table_entry(b, k, (int)t, (int)i, (int)j);
    if (e) rho *= e[0];
  }
};

/* The reference's boundary loop for b (and its adjoint loop, null where the
 * reference has none: the standard pressure boundaries, LBBoundaryLoop.cc:11-18);
 * throws for boundaries the reference does not have. */
void make_zouhe(const lbm_config& c, int k, LBBoundaryLoop** l, AdjointLBBoundaryLoop** al) {
  const lbm_bc& b = c.bc[k];
  Box2d bb(b.box[0], b.box[1], b.box[2], b.box[3]);
  *l = nullptr;
  *al = nullptr;
  if (b.kind == LBM_BC_VELOCITY) {
    VelFunc vf{c, b, k};
    if (b.face == LBM_FACE_WEST) *l = new IncompressibleZouHeVelocityWest2d<D2Q9, VelFunc>(bb, vf);
    if (b.face == LBM_FACE_EAST) *l = new IncompressibleZouHeVelocityEast2d<D2Q9, VelFunc>(bb, vf);
    if (b.face == LBM_FACE_NORTH) *l = new IncompressibleZouHeVelocityNorth2d<D2Q9, VelFunc>(bb, vf);
  } else if (b.kind == LBM_BC_VELOCITY_STANDARD) {
    VelFunc vf{c, b, k};
    if (b.face == LBM_FACE_WEST) *l = new StandardZouHeVelocityWest2d<D2Q9, VelFunc>(bb, vf);
  } else if (b.kind == LBM_BC_PRESSURE) {
    PresFunc pf{c, b, k};
    if (b.face == LBM_FACE_EAST) *l = new IncompressibleZouHePressureEast2d<D2Q9, PresFunc>(bb, pf);
    if (b.face == LBM_FACE_WEST) *l = new IncompressibleZouHePressureWest2d<D2Q9, PresFunc>(bb, pf);
  } else if (b.kind == LBM_BC_PRESSURE_STANDARD) {
    PresFunc pf{c, b, k};
    if (b.face == LBM_FACE_EAST) *l = new StandardZouHePressureEast2d<D2Q9, PresFunc>(bb, pf);
    if (b.face == LBM_FACE_WEST) *l = new StandardZouHePressureWest2d<D2Q9, PresFunc>(bb, pf);
  }
  if (!*l) throw 1;
  if ((*l)->getAdjointBoundaryLoop(al)) *al = nullptr;
}

/* T*** / T**** views over contiguous AoS storage, as DMDAVecGetArrayDOF gives. */
struct View2 {
  std::vector<double*> rows;
  std::vector<double**> cols;
  double*** p;
  View2(double* data, int nx, int ny, int dof) : rows((size_t)nx * ny), cols(ny) {
    for (int j = 0; j < ny; ++j) {
      for (int i = 0; i < nx; ++i) rows[(size_t)j * nx + i] = data + ((size_t)j * nx + i) * dof;
      cols[j] = &rows[(size_t)j * nx];
    }
    p = cols.data();
  }
};

struct Sens2 {
  std::vector<double*> cols;
  double** p;
  Sens2(double* data, int nx, int ny) : cols(ny) {
    for (int j = 0; j < ny; ++j) cols[j] = data + (size_t)j * nx;
    p = cols.data();
  }
};

double box_inv(const int* b) {
  return (double)(1. / ((b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1)));
}

/* ------------------------------------------------------------------ */
/* 2D D2Q9 with the reference's loop classes */

template <class Base>
struct Sim2d {
  using Op = PartialBouncebackCollision<Base, ScaledBP>;
  lbm_config c;
  int nx, ny, Q = 9, NMAC = 3;
  Op op;
  Box2d box;
  std::vector<std::unique_ptr<LBBoundaryLoop>> bcs;
  std::vector<std::unique_ptr<AdjointLBBoundaryLoop>> abcs;

  Sim2d(const lbm_config& cfg, Base base)
      : c(cfg), nx(cfg.nx), ny(cfg.ny), op(base, ScaledBP(cfg.interp_q, cfg.interp_scale)),
        box(0, cfg.nx - 1, 0, cfg.ny - 1) {
    for (int k = 0; k < c.nbc; ++k) {
      LBBoundaryLoop* l;
      AdjointLBBoundaryLoop* al;
      make_zouhe(c, k, &l, &al);
      bcs.emplace_back(l);
      abcs.emplace_back(al);
    }
  }

  void init(const double* macros, std::vector<double>& f) {
    std::vector<double> mac((size_t)nx * ny * 3);
    for (size_t k = 0; k < (size_t)nx * ny; ++k) {
      mac[3 * k] = macros ? macros[3 * k] : 1.;
      mac[3 * k + 1] = macros ? macros[3 * k + 1] : 0.;
      mac[3 * k + 2] = macros ? macros[3 * k + 2] : 0.;
    }
    View2 vf(f.data(), nx, ny, Q), vm(mac.data(), nx, ny, 3);
    IsoEquilibriumInitializationLoop2d<IncompressibleFeq2d<D2Q9>> loop(box);
    loop.execute(vf.p, vm.p, nullptr);
  }

  /* collide() of LBSolver::collide (LBSolver.cc:163-182) */
  void collide(std::vector<double>& f, std::vector<double>& mac, std::vector<double>& gamma) {
    View2 vf(f.data(), nx, ny, Q), vm(mac.data(), nx, ny, 3), vg(gamma.data(), nx, ny, 1);
    ObstIsoCollisionLoop2d<Op> loop(box, op);
    loop.execute(vf.p, vm.p, vg.p);
  }

  /* stream() of LBSolver::stream (LBSolver.cc:184-206), one rank: the local copy is
   * the whole array. */
  void stream(std::vector<double>& f, int t) {
    std::vector<double> fl = f;
    View2 vf(f.data(), nx, ny, Q), vl(fl.data(), nx, ny, Q);
    IsoStreamLoop2d<D2Q9> loop(box, box);
    loop.execute(vf.p, vl.p, nullptr);
    for (auto& b : bcs) b->execute(t, vf.p, vf.p);
  }

  double functional(const std::vector<double>& mac) {
    double tc = c.obj_weight, ps = 0.;
    if (c.objective == LBM_OBJ_THROUGH_FLOW) {
      /* ThroughFlow2d::evaluate (functionals/throughFlow2d.hh:17-40), one rank */
      double invIn = box_inv(c.obj_in), invOut = box_inv(c.obj_out), iif = 0., of = 0.;
      for (int j = c.obj_in[2]; j <= c.obj_in[3]; ++j)
        for (int i = c.obj_in[0]; i <= c.obj_in[1]; ++i)
          iif -= tc * invIn * mac[((size_t)j * nx + i) * 3 + 1];
      for (int j = c.obj_out[2]; j <= c.obj_out[3]; ++j)
        for (int i = c.obj_out[0]; i <= c.obj_out[1]; ++i)
          of -= tc * invOut * mac[((size_t)j * nx + i) * 3 + 1];
      return iif + of;
    }
    if (c.objective == LBM_OBJ_OUTFLOW) {
      double inv = box_inv(c.obj_out), of = 0.;
      for (int j = c.obj_out[2]; j <= c.obj_out[3]; ++j)
        for (int i = c.obj_out[0]; i <= c.obj_out[1]; ++i)
          of -= tc * inv * mac[((size_t)j * nx + i) * 3 + 1];
      return of;
    }
    if (c.objective != LBM_OBJ_PRESSURE_DROP) return 0.;
    double invIn = box_inv(c.obj_in), invOut = box_inv(c.obj_out);
    for (int j = c.obj_in[2]; j <= c.obj_in[3]; ++j)
      for (int i = c.obj_in[0]; i <= c.obj_in[1]; ++i)
        ps += tc * invIn * mac[((size_t)j * nx + i) * 3];
    for (int j = c.obj_out[2]; j <= c.obj_out[3]; ++j)
      for (int i = c.obj_out[0]; i <= c.obj_out[1]; ++i)
        ps -= tc * invOut * mac[((size_t)j * nx + i) * 3];
    return ps;
  }

  void source(std::vector<double>& adj) {
    if (c.objective == LBM_OBJ_THROUGH_FLOW) {
      /* ThroughFlow2d::adjointCollideSource, incompressible macros (throughFlow2d.hh:41-59) */
      double tc = c.obj_weight, invIn = box_inv(c.obj_in), invOut = box_inv(c.obj_out);
      for (int j = c.obj_in[2]; j <= c.obj_in[3]; ++j)
        for (int i = c.obj_in[0]; i <= c.obj_in[1]; ++i)
          for (int d = 0; d < 9; ++d) adj[((size_t)j * nx + i) * 9 + d] -= invIn * tc * D2Q9::ex[d];
      for (int j = c.obj_out[2]; j <= c.obj_out[3]; ++j)
        for (int i = c.obj_out[0]; i <= c.obj_out[1]; ++i)
          for (int d = 0; d < 9; ++d) adj[((size_t)j * nx + i) * 9 + d] -= invOut * tc * D2Q9::ex[d];
      return;
    }
    if (c.objective == LBM_OBJ_OUTFLOW) {
      double tc = c.obj_weight, inv = box_inv(c.obj_out);
      for (int j = c.obj_out[2]; j <= c.obj_out[3]; ++j)
        for (int i = c.obj_out[0]; i <= c.obj_out[1]; ++i)
          for (int d = 0; d < 9; ++d) adj[((size_t)j * nx + i) * 9 + d] -= inv * tc * D2Q9::ex[d];
      return;
    }
    if (c.objective != LBM_OBJ_PRESSURE_DROP) return;
    double tc = c.obj_weight, invIn = box_inv(c.obj_in), invOut = box_inv(c.obj_out);
    for (int j = c.obj_in[2]; j <= c.obj_in[3]; ++j)
      for (int i = c.obj_in[0]; i <= c.obj_in[1]; ++i)
        for (int d = 0; d < 9; ++d) adj[((size_t)j * nx + i) * 9 + d] += invIn * tc;
    for (int j = c.obj_out[2]; j <= c.obj_out[3]; ++j)
      for (int i = c.obj_out[0]; i <= c.obj_out[1]; ++i)
        for (int d = 0; d < 9; ++d) adj[((size_t)j * nx + i) * 9 + d] -= invOut * tc;
  }

  /* Reverse step: AdjointLBSolver::adjointCollide, computeCollideSource, adjointStream
   * (adjointLBSolver.cc:28-102). */
  void adjoint_step(std::vector<double>& adj, std::vector<double>& f, std::vector<double>& gamma,
                    std::vector<double>& sens, int t) {
    auto rop = op.getSourceAdjoint();
    View2 va(adj.data(), nx, ny, Q), vf(f.data(), nx, ny, Q), vg(gamma.data(), nx, ny, 1);
    Sens2 vs(sens.data(), nx, ny);
    SourceAdjointObstIsoCollisionLoop2d<Op, decltype(rop)> aloop(box, rop);
    aloop.execute(va.p, vf.p, vg.p, vs.p);
    source(adj);
    for (auto& b : abcs) {
      if (!b) throw 2;   /* a boundary without an adjoint in the reference */
      b->execute(t, va.p, vf.p);
    }
    std::vector<double> al = adj;
    View2 vl(al.data(), nx, ny, Q);
    AdjointIsoStreamingLoop2d<Op> sloop(box, box);
    sloop.execute(va.p, vl.p, nullptr, nullptr);
  }
};

/* ------------------------------------------------------------------ */
/* 3D D3Q19 MRT + PBB with the reference's per-cell operators */

template <class C>
struct Sim3d {
  using Op = PartialBouncebackCollision<MRT3dAdapter<C>, ScaledBP>;
  lbm_config c;
  int nx, ny, nz, Q = 19, NMAC = 4;
  Op op;
  Sim3d(const lbm_config& cfg)
      : c(cfg), nx(cfg.nx), ny(cfg.ny), nz(cfg.nz),
        op(MRT3dAdapter<C>(cfg.omega), ScaledBP(cfg.interp_q, cfg.interp_scale)) {}
  size_t idx(int x, int y, int z) const { return ((size_t)z * ny + y) * nx + x; }

  void init(const double* macros, std::vector<double>& f) {
    for (size_t k = 0; k < (size_t)nx * ny * nz; ++k) {
      double rho = macros ? macros[4 * k] : 1., ux = macros ? macros[4 * k + 1] : 0.,
             uy = macros ? macros[4 * k + 2] : 0., uz = macros ? macros[4 * k + 3] : 0.;
      double uSqr = ux * ux + uy * uy + uz * uz;
      IncompressibleFeq3d<D3Q19>::setAllEquilibria(&f[k * Q], rho, ux, uy, uz, uSqr);
    }
  }
  void collide(std::vector<double>& f, std::vector<double>& mac, std::vector<double>& gamma) {
    for (size_t k = 0; k < (size_t)nx * ny * nz; ++k) op(&f[k * Q], &f[k * Q], &mac[4 * k], &gamma[k]);
  }
  void stream(std::vector<double>& f, int t) {
    std::vector<double> fl = f;
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x)
          for (int d = 1; d < 19; ++d) {
            int sx = x - D3Q19::ex[d], sy = y - D3Q19::ey[d], sz = z - D3Q19::ez[d];
            if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz)
              f[idx(x, y, z) * Q + d] = fl[idx(sx, sy, sz) * Q + d];
            else
              f[idx(x, y, z) * Q + d] = fl[idx(x, y, z) * Q + D3Q19::opp[d]];
          }
    for (int k = 0; k < c.nbc; ++k) {
      const lbm_bc& b = c.bc[k];
      for (int z = b.box[4]; z <= b.box[5]; ++z)
        for (int y = b.box[2]; y <= b.box[3]; ++y) {
          double* fd = &f[idx(b.box[0], y, z) * Q];
          double v = b.value * time_factor(b, t);
          if (b.profile == LBM_PROFILE_TABLE) throw 4;
          if (b.kind == LBM_BC_VELOCITY) {
            v *= profile(c, b, b.box[0], y, z);
            const bool nodir = b.dir[0] == 0. && b.dir[1] == 0. && b.dir[2] == 0.;
            double ux = v * (nodir ? 1. : b.dir[0]), uy = v * (nodir ? 0. : b.dir[1]),
                   uz = v * (nodir ? 0. : b.dir[2]);
            double Nyx = 0.5 * (fd[5] + fd[11] + fd[13] - (fd[2] + fd[4] + fd[14])) - (1. / 3.) * uy;
            double Nzx = 0.5 * (fd[10] + fd[13] + fd[14] - (fd[1] + fd[4] + fd[5])) - (1. / 3.) * uz;
            fd[7] = fd[16] + (1. / 6.) * (ux - uz) + Nzx;
            fd[9] = fd[18] + (1. / 6.) * (ux - uy) + Nyx;
            fd[12] = fd[3] + (1. / 3.) * ux;
            fd[15] = fd[6] + (1. / 6.) * (ux + uz) - Nzx;
            fd[17] = fd[8] + (1. / 6.) * (ux + uy) - Nyx;
          } else {
            double rho0 = v;
            double ux = fd[0] + fd[1] + fd[2] + fd[4] + fd[5] + fd[10] + fd[11] + fd[13] + fd[14] +
                        2. * (fd[7] + fd[9] + fd[12] + fd[15] + fd[17]) - rho0;
            double Nyx = 0.5 * (fd[5] + fd[11] + fd[13] - (fd[2] + fd[4] + fd[14]));
            double Nzx = 0.5 * (fd[10] + fd[13] + fd[14] - (fd[1] + fd[4] + fd[5]));
            fd[3] = fd[12] - (1. / 3.) * ux;
            fd[6] = fd[15] - (1. / 6.) * ux + Nzx;
            fd[8] = fd[17] - (1. / 6.) * ux + Nyx;
            fd[16] = fd[7] - (1. / 6.) * ux - Nzx;
            fd[18] = fd[9] - (1. / 6.) * ux - Nyx;
          }
        }
    }
  }
  double functional(const std::vector<double>& mac) {
    if (c.objective != LBM_OBJ_PRESSURE_DROP) return 0.;
    double tc = c.obj_weight, ps = 0., invIn = box_inv(c.obj_in), invOut = box_inv(c.obj_out);
    for (int z = c.obj_in[4]; z <= c.obj_in[5]; ++z)
      for (int y = c.obj_in[2]; y <= c.obj_in[3]; ++y)
        for (int x = c.obj_in[0]; x <= c.obj_in[1]; ++x) ps += tc * invIn * mac[idx(x, y, z) * 4];
    for (int z = c.obj_out[4]; z <= c.obj_out[5]; ++z)
      for (int y = c.obj_out[2]; y <= c.obj_out[3]; ++y)
        for (int x = c.obj_out[0]; x <= c.obj_out[1]; ++x) ps -= tc * invOut * mac[idx(x, y, z) * 4];
    return ps;
  }
  void adjoint_step(std::vector<double>& adj, std::vector<double>& f, std::vector<double>& gamma,
                    std::vector<double>& sens, int t) {
    (void)t;
    auto rop = op.getSourceAdjoint();
    for (size_t k = 0; k < (size_t)nx * ny * nz; ++k) {
      double fout[19], rin[19], mac[4], rmac[4] = {0, 0, 0, 0}, robst = 0.;
      for (int d = 0; d < 19; ++d) rin[d] = 0.;
      rop(&f[k * Q], fout, mac, &gamma[k], rin, &adj[k * Q], rmac, &robst);
      for (int d = 0; d < 19; ++d) adj[k * Q + d] = rin[d];
      sens[k] += robst;
    }
    if (c.objective == LBM_OBJ_PRESSURE_DROP) {
      double tc = c.obj_weight, invIn = box_inv(c.obj_in), invOut = box_inv(c.obj_out);
      for (int z = c.obj_in[4]; z <= c.obj_in[5]; ++z)
        for (int y = c.obj_in[2]; y <= c.obj_in[3]; ++y)
          for (int x = c.obj_in[0]; x <= c.obj_in[1]; ++x)
            for (int d = 0; d < 19; ++d) adj[idx(x, y, z) * Q + d] += invIn * tc;
      for (int z = c.obj_out[4]; z <= c.obj_out[5]; ++z)
        for (int y = c.obj_out[2]; y <= c.obj_out[3]; ++y)
          for (int x = c.obj_out[0]; x <= c.obj_out[1]; ++x)
            for (int d = 0; d < 19; ++d) adj[idx(x, y, z) * Q + d] -= invOut * tc;
    }
    for (int k = c.nbc - 1; k >= 0; --k) {
      const lbm_bc& b = c.bc[k];
      for (int z = b.box[4]; z <= b.box[5]; ++z)
        for (int y = b.box[2]; y <= b.box[3]; ++y) {
          double* a = &adj[idx(b.box[0], y, z) * Q];
          if (b.kind == LBM_BC_VELOCITY) {
            a[1] += 0.5 * (a[15] - a[7]);
            a[2] += 0.5 * (a[17] - a[9]);
            a[3] += a[12];
            a[4] += 0.5 * (a[15] + a[17] - (a[7] + a[9]));
            a[5] += 0.5 * (a[9] + a[15] - (a[7] + a[17]));
            a[6] += a[15];
            a[8] += a[17];
            a[10] += 0.5 * (a[7] - a[15]);
            a[11] += 0.5 * (a[9] - a[17]);
            a[13] += 0.5 * (a[7] + a[9] - (a[15] + a[17]));
            a[14] += 0.5 * (a[7] + a[17] - (a[9] + a[15]));
            a[16] += a[7];
            a[18] += a[9];
            a[7] = a[9] = a[12] = a[15] = a[17] = 0.;
          } else {
            double adjUx = -(1. / 3.) * a[3] - (1. / 6.) * (a[6] + a[8] + a[16] + a[18]);
            a[0] += adjUx;
            a[1] += adjUx + 0.5 * (a[16] - a[6]);
            a[2] += adjUx + 0.5 * (a[18] - a[8]);
            a[4] += adjUx + 0.5 * (a[16] + a[18] - (a[6] + a[8]));
            a[5] += adjUx + 0.5 * (a[8] + a[16] - (a[6] + a[18]));
            a[7] += 2. * adjUx + a[16];
            a[9] += 2. * adjUx + a[18];
            a[10] += adjUx + 0.5 * (a[6] - a[16]);
            a[11] += adjUx + 0.5 * (a[8] - a[18]);
            a[12] += 2. * adjUx + a[3];
            a[13] += adjUx + 0.5 * (a[6] + a[8] - (a[16] + a[18]));
            a[14] += adjUx + 0.5 * (a[6] + a[18] - (a[8] + a[16]));
            a[15] += 2. * adjUx + a[6];
            a[17] += 2. * adjUx + a[8];
            a[3] = a[6] = a[8] = a[16] = a[18] = 0.;
          }
        }
    }
    std::vector<double> al = adj;
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x)
          for (int d = 1; d < 19; ++d) {
            int sx = x + D3Q19::ex[d], sy = y + D3Q19::ey[d], sz = z + D3Q19::ez[d];
            if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz)
              adj[idx(x, y, z) * Q + d] = al[idx(sx, sy, sz) * Q + d];
            else
              adj[idx(x, y, z) * Q + d] = al[idx(x, y, z) * Q + D3Q19::opp[d]];
          }
  }
};


/* ------------------------------------------------------------------ */
/* Thermal double distribution: D2Q9 BGK + partial bounce-back flow and D2Q5
 * temperature, 14 DOF per cell (flow first, ThermalDualCollision's layout). */

struct SimThermal {
  using Iso = PartialBouncebackCollision<IncompressibleBGK2d<D2Q9>, ScaledBP>;
  using Th = ThermalObstacleCollision<ThermalBGK2d<D2Q5>, RampInterpolation<>>;
  using Op = ThermalDualCollision<Iso, Th>;
  lbm_config c;
  int nx, ny, Q = 14, NMAC = 4;
  Op op;
  Box2d box;
  std::vector<std::unique_ptr<LBBoundaryLoop>> bcs;
  std::vector<std::unique_ptr<AdjointLBBoundaryLoop>> abcs;

  /* the thermal Zou-He inlets (restated: ThermalZouHeWest2d<.,D2Q5,.>::execute,
   * thermalZouHe2d.hh:68-80) */
  std::vector<lbm_bc> tbcs;

  SimThermal(const lbm_config& cfg)
      : c(cfg), nx(cfg.nx), ny(cfg.ny),
        op(Iso(IncompressibleBGK2d<D2Q9>(cfg.omega), ScaledBP(cfg.interp_q, cfg.interp_scale)),
           Th(ThermalBGK2d<D2Q5>(1., cfg.diffusivity), RampInterpolation<>(cfg.ramp_q, cfg.ramp_ck))),
        box(0, cfg.nx - 1, 0, cfg.ny - 1) {
    /* the reference has no solid heating term: only heat_rate = 0 is its model */
    if (cfg.heat_rate != 0.) throw 3;
    for (int k = 0; k < c.nbc; ++k) {
      const lbm_bc& b = c.bc[k];
      if (b.kind == LBM_BC_TEMPERATURE && b.face == LBM_FACE_WEST) {
        if (b.profile == LBM_PROFILE_TABLE) throw 4;
        tbcs.push_back(b);
        abcs.emplace_back(new AdjointThermalZouHeWest2d<D2Q9, D2Q5>(
            Box2d(b.box[0], b.box[1], b.box[2], b.box[3])));
        continue;
      }
      LBBoundaryLoop* l;
      AdjointLBBoundaryLoop* al;
      make_zouhe(c, k, &l, &al);
      bcs.emplace_back(l);
      abcs.emplace_back(al);
    }
  }
  size_t idx(int x, int y) const { return (size_t)y * nx + x; }

  void init(const double* macros, std::vector<double>& f) {
    for (size_t k = 0; k < (size_t)nx * ny; ++k) {
      double rho = macros ? macros[4 * k] : 1., ux = macros ? macros[4 * k + 1] : 0.,
             uy = macros ? macros[4 * k + 2] : 0., T = macros ? macros[4 * k + 3] : 0.;
      IncompressibleFeq2d<D2Q9>::setAllEquilibria(&f[k * Q], rho, ux, uy, ux * ux + uy * uy);
      ThermalFeq2d<D2Q5>::setAllEquilibria(&f[k * Q + 9], ux, uy, T);
    }
  }
  void collide(std::vector<double>& f, std::vector<double>& mac, std::vector<double>& gamma) {
    for (size_t k = 0; k < (size_t)nx * ny; ++k) op(&f[k * Q], &f[k * Q], &mac[4 * k], &gamma[k]);
  }
  template <class L>
  void stream_lattice(std::vector<double>& f, const std::vector<double>& fl, int off) {
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x)
        for (int d = 1; d < L::numDOF; ++d) {
          int sx = x - L::ex[d], sy = y - L::ey[d];
          if (sx >= 0 && sy >= 0 && sx < nx && sy < ny)
            f[idx(x, y) * Q + off + d] = fl[idx(sx, sy) * Q + off + d];
          else
            f[idx(x, y) * Q + off + d] = fl[idx(x, y) * Q + off + L::opp[d]];
        }
  }
  void stream(std::vector<double>& f, int t) {
    std::vector<double> fl = f;
    stream_lattice<D2Q9>(f, fl, 0);
    stream_lattice<D2Q5>(f, fl, 9);
    View2 vf(f.data(), nx, ny, Q);
    for (auto& b : bcs) b->execute(t, vf.p, vf.p);
    for (const lbm_bc& b : tbcs)
      for (int y = b.box[2]; y <= b.box[3]; ++y) {
        double* g = &f[idx(b.box[0], y) * Q + 9];
        double T = b.value * time_factor(b, t);
        g[4] = T - g[0] - g[1] - g[2] - g[3];
      }
  }
  /* ThermalOutflowEast2d::evaluate (temperatureFlow2d.hh:18-32), summed without MPI */
  double functional(const std::vector<double>& mac) {
    if (c.objective != LBM_OBJ_HEAT_FLUX) return 0.;
    double tc = c.obj_weight, pout = 0.;
    for (int y = c.obj_out[2]; y <= c.obj_out[3]; ++y)
      for (int x = c.obj_out[0]; x <= c.obj_out[1]; ++x)
        pout -= tc * mac[idx(x, y) * 4 + 1] * mac[idx(x, y) * 4 + 3];
    return pout;
  }
  /* ThermalOutflowEast2d::adjointCollideSource (temperatureFlow2d.hh:33-52) */
  void source(std::vector<double>& adj, const std::vector<double>& f) {
    if (c.objective != LBM_OBJ_HEAT_FLUX) return;
    double tc = c.obj_weight;
    for (int y = c.obj_out[2]; y <= c.obj_out[3]; ++y)
      for (int x = c.obj_out[0]; x <= c.obj_out[1]; ++x) {
        const double* fd = &f[idx(x, y) * Q];
        double ux = 0., T;
        IncompressibleMacros2d<D2Q9>::computeUx(fd, ux);
        StandardThermalMacros2d<D2Q5>::compute(fd + 9, T);
        double* a = &adj[idx(x, y) * Q];
        for (int d = 0; d < 9; ++d) a[d] -= tc * D2Q9::ex[d] * T;
        for (int d = 0; d < 5; ++d) a[9 + d] -= tc * ux;
      }
  }
  template <class L>
  void adjoint_stream_lattice(std::vector<double>& adj, const std::vector<double>& al, int off) {
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x)
        for (int d = 1; d < L::numDOF; ++d) {
          int sx = x + L::ex[d], sy = y + L::ey[d];
          if (sx >= 0 && sy >= 0 && sx < nx && sy < ny)
            adj[idx(x, y) * Q + off + d] = al[idx(sx, sy) * Q + off + d];
          else
            adj[idx(x, y) * Q + off + d] = al[idx(x, y) * Q + off + L::opp[d]];
        }
  }
  void adjoint_step(std::vector<double>& adj, std::vector<double>& f, std::vector<double>& gamma,
                    std::vector<double>& sens, int t) {
    auto rop = op.getSourceAdjoint();
    View2 va(adj.data(), nx, ny, Q), vf(f.data(), nx, ny, Q), vg(gamma.data(), nx, ny, 1);
    Sens2 vs(sens.data(), nx, ny);
    SourceAdjointObstThermalCollisionLoop2d<Op, decltype(rop)> aloop(box, rop);
    aloop.execute(va.p, vf.p, vg.p, vs.p);
    source(adj, f);
    for (auto& b : abcs) {
      if (!b) throw 2;
      b->execute(t, va.p, vf.p);
    }
    std::vector<double> al = adj;
    adjoint_stream_lattice<D2Q9>(adj, al, 0);
    adjoint_stream_lattice<D2Q5>(adj, al, 9);
  }
};

/* ------------------------------------------------------------------ */
/* Generic drivers (the reference applications' loop, robustPump2d.cc:234-276) */

template <class S>
int run_forward(S& s, const lbm_config& c, const double* gamma, const double* macros, int n,
                double* f_out, double* J_steps, double* J_sum) {
  size_t ncell = (size_t)c.nx * c.ny * (c.lattice == LBM_D3Q19 ? c.nz : 1);
  std::vector<double> f(ncell * s.Q), mac(ncell * s.NMAC), g(gamma, gamma + ncell);
  s.init(macros, f);
  s.collide(f, mac, g);
  double acc = 0.;
  for (int t = 1; t <= n; ++t) {
    s.stream(f, t);
    if (t == n) std::memcpy(f_out, f.data(), sizeof(double) * f.size());
    s.collide(f, mac, g);
    double v = s.functional(mac);
    if (J_steps) J_steps[t - 1] = v;
    acc += v;
  }
  if (n == 0) std::memcpy(f_out, f.data(), sizeof(double) * f.size());
  if (J_sum) *J_sum = acc;
  return 0;
}

template <class S>
int run_gradient(S& s, const lbm_config& c, const double* gamma, const double* macros, int n,
                 double* J_sum, double* sens_out) {
  size_t ncell = (size_t)c.nx * c.ny * (c.lattice == LBM_D3Q19 ? c.nz : 1);
  std::vector<double> f(ncell * s.Q), mac(ncell * s.NMAC), g(gamma, gamma + ncell);
  std::vector<std::vector<double>> states((size_t)n + 1);
  s.init(macros, f);
  states[0] = f;
  s.collide(f, mac, g);
  double acc = 0.;
  for (int t = 1; t <= n; ++t) {
    s.stream(f, t);
    states[t] = f;
    s.collide(f, mac, g);
    acc += s.functional(mac);
  }
  if (J_sum) *J_sum = acc;
  std::vector<double> adj(ncell * s.Q, 0.), sens(ncell, 0.);
  for (int t = n; t >= 1; --t) s.adjoint_step(adj, states[t], g, sens, t);
  std::memcpy(sens_out, sens.data(), sizeof(double) * ncell);
  return 0;
}

bool is_cfg3_rates(const lbm_config& c) {
  return c.mrt[0] == 1.2 && c.mrt[1] == 1.2 && c.mrt[2] == 1.2 && c.mrt[3] == 1.2 &&
         c.mrt[4] == 1.2 && c.mrt[5] == 3. && c.mrt[6] == -5.5 && c.mrt[7] == -0.5;
}
bool is_default3_rates(const lbm_config& c) {
  return c.mrt[0] == 1.19 && c.mrt[1] == 1.4 && c.mrt[2] == 1.2 && c.mrt[3] == 1.4 &&
         c.mrt[4] == 1.4 && c.mrt[5] == 3. && c.mrt[6] == -5.5 && c.mrt[7] == -0.5;
}
bool is_mrt2d_rates(const lbm_config& c) {
  return c.mrt[0] == 1.4 && c.mrt[1] == 1.4 && c.mrt[2] == 1.2;
}

template <class F>
int dispatch(const lbm_config& c, F&& fn) {
  if (c.lattice == LBM_D2Q9 && c.collision == LBM_BGK) {
    Sim2d<IncompressibleBGK2d<D2Q9>> s(c, IncompressibleBGK2d<D2Q9>(c.omega));
    return fn(s);
  }
  if (c.lattice == LBM_D2Q9 && c.collision == LBM_MRT && is_mrt2d_rates(c)) {
    Sim2d<IncompressibleMRT2d<D2Q9>> s(c, IncompressibleMRT2d<D2Q9>(c.omega));
    return fn(s);
  }
  if (c.lattice == LBM_D3Q19 && c.collision == LBM_MRT && is_cfg3_rates(c)) {
    Sim3d<Cfg3Constants> s(c);
    return fn(s);
  }
  if (c.lattice == LBM_D3Q19 && c.collision == LBM_MRT && is_default3_rates(c)) {
    Sim3d<MRT3d_Compile_constants> s(c);
    return fn(s);
  }
  if (c.lattice == LBM_D2Q9_D2Q5 && c.collision == LBM_BGK) {
    SimThermal s(c);
    return fn(s);
  }
  return -2;
}

/* Checkpoint schedule driven with integer "states" so the reversal can be checked. */
class CountingCheckpointing : public DynamicCheckpointing {
 public:
  CountingCheckpointing(PetscInt k, Vec v) : DynamicCheckpointing(k, v) {}
  double state = 0.;
  long long recomputed = 0;

 protected:
  PetscErrorCode advance(void*) override {
    state += 1.;
    ++recomputed;
    return 0;
  }
  PetscErrorCode setSolverState(PetscInt, Vec v, void*) override {
    state = v->v[0];
    return 0;
  }
  PetscErrorCode copyFromSolverState(Vec v, void*) override {
    v->v[0] = state;
    return 0;
  }
};

/* The reference's static placement, driven the same way. */
class CountingStatic : public StaticCheckpointing {
 public:
  CountingStatic(PetscInt k, PetscInt nt, Vec v) : StaticCheckpointing(k, nt, v) {}
  size_t numSaved() const { return checkpoints.size(); }
  double state = 0.;
  long long recomputed = 0;

 protected:
  PetscErrorCode advance(void*) override {
    state += 1.;
    ++recomputed;
    return 0;
  }
  PetscErrorCode setSolverState(PetscInt, Vec v, void*) override {
    state = v->v[0];
    return 0;
  }
  PetscErrorCode copyFromSolverState(Vec v, void*) override {
    v->v[0] = state;
    return 0;
  }
};

}  // namespace

extern "C" {

/* Table of boundary slot k (see Table); table = NULL clears it. */
int ref_set_bc_profile(int k, int nt, int ncomp, long long npos, const double* table) {
  if (k < 0 || k >= LBM_MAX_BC) return -1;
  Table& tb = g_tables[k];
  tb.v.clear();
  tb.nt = tb.ncomp = 0;
  tb.npos = 0;
  if (!table) return 0;
  tb.v.assign(table, table + (size_t)nt * (size_t)npos * (size_t)ncomp);
  tb.nt = nt;
  tb.ncomp = ncomp;
  tb.npos = npos;
  return 0;
}

int ref_forward(const lbm_config* cfg, const double* gamma, const double* macros, int nsteps,
                double* f_out, double* J_steps, double* J_sum) {
  try {
    return dispatch(*cfg, [&](auto& s) {
      return run_forward(s, *cfg, gamma, macros, nsteps, f_out, J_steps, J_sum);
    });
  } catch (...) {
    return -2;
  }
}

int ref_gradient(const lbm_config* cfg, const double* gamma, const double* macros, int nsteps,
                 double* J_sum, double* sens) {
  try {
    return dispatch(*cfg, [&](auto& s) {
      return run_gradient(s, *cfg, gamma, macros, nsteps, J_sum, sens);
    });
  } catch (...) {
    return -2;
  }
}

int ref_adjoint_step(const lbm_config* cfg, const double* gamma, const double* f_t, int t,
                     double* lam, double* sens) {
  try {
    return dispatch(*cfg, [&](auto& s) {
      size_t ncell = (size_t)cfg->nx * cfg->ny * (cfg->lattice == LBM_D3Q19 ? cfg->nz : 1);
      std::vector<double> adj(lam, lam + ncell * s.Q), f(f_t, f_t + ncell * s.Q),
          g(gamma, gamma + ncell), se(sens, sens + ncell);
      s.adjoint_step(adj, f, g, se, t);
      std::memcpy(lam, adj.data(), sizeof(double) * adj.size());
      std::memcpy(sens, se.data(), sizeof(double) * ncell);
      return 0;
    });
  } catch (...) {
    return -2;
  }
}

int ref_collide_cell(const lbm_config* cfg, const double* fin, double gamma, double* fout,
                     double* mac) {
  try {
    return dispatch(*cfg, [&](auto& s) {
      double g = gamma, m[4] = {0, 0, 0, 0};
      s.op(fin, fout, m, &g);
      if (mac)
        for (int j = 0; j < s.NMAC; ++j) mac[j] = m[j];
      return 0;
    });
  } catch (...) {
    return -2;
  }
}

int ref_reverse_cell(const lbm_config* cfg, const double* fin, double gamma, const double* lam_out,
                     double* lam_in, double* dgamma) {
  try {
    return dispatch(*cfg, [&](auto& s) {
      auto rop = s.op.getSourceAdjoint();
      double fi[19], fout[19], lo[19], mac[4], rmac[4] = {0, 0, 0, 0}, g = gamma, dg = 0.;
      for (int d = 0; d < s.Q; ++d) {
        fi[d] = fin[d];
        lo[d] = lam_out[d];
        lam_in[d] = 0.;
      }
      rop(fi, fout, mac, &g, lam_in, lo, rmac, &dg);
      if (dgamma) *dgamma = dg;
      return 0;
    });
  } catch (...) {
    return -2;
  }
}

int ref_wang_count(int nsteps, int nsnap, long long* recomputed, int* ok) {
  if (nsnap < 2 || nsteps < 1) return -1;
  _p_Vec proto;
  proto.v.assign(1, 0.);
  CountingCheckpointing ck(nsnap, &proto);
  ck.reset(nullptr);
  _p_Vec cur;
  cur.v.assign(1, 0.);
  for (int s = 0; s <= nsteps; ++s) {
    cur.v[0] = s;
    ck.makeCheckpoint(s, &cur, nullptr);
  }
  int good = 1;
  for (int s = nsteps; s >= 1; --s) {
    ck.getForwardSolution(s, &cur, nullptr);
    if (cur.v[0] != (double)s) good = 0;
  }
  *recomputed = ck.recomputed;
  if (ok) *ok = good;
  return 0;
}

/* StaticCheckpointing(nsnap, nsteps + 1): the forward sweep offers states
 * 0..nsteps (as the applications do, e.g. pump2d.cc:146); saved counts the
 * states it kept. */
int ref_static_count(int nsteps, int nsnap, long long* recomputed, int* ok, int* saved) {
  if (nsnap < 2 || nsteps < 1) return -1;
  _p_Vec proto;
  proto.v.assign(1, 0.);
  CountingStatic ck(nsnap, nsteps + 1, &proto);
  _p_Vec cur;
  cur.v.assign(1, 0.);
  for (int s = 0; s <= nsteps; ++s) {
    cur.v[0] = s;
    ck.makeCheckpoint(s, &cur, nullptr);
  }
  if (saved) *saved = (int)ck.numSaved();
  int good = 1;
  for (int s = nsteps; s >= 1; --s) {
    ck.getForwardSolution(s, &cur, nullptr);
    if (cur.v[0] != (double)s) good = 0;
  }
  *recomputed = ck.recomputed;
  if (ok) *ok = good;
  return 0;
}

/* The reference's MMA (topOpt/MMA.hh:111-229) on plain arrays: one object
 * kept across updates so the asymptotes adapt as in an optimisation loop. */
struct ref_mma {
  MMA* mma = nullptr;
  int n = 0, m = 0;
  _p_Vec x, df0;
  std::vector<_p_Vec> dg;
};

void* ref_mma_create(int n, int m, const double* x0, const double* robust_a) {
  ref_mma* r = new ref_mma;
  r->n = n;
  r->m = m;
  r->x.v.assign(x0, x0 + n);
  r->df0.v.assign(n, 0.);
  r->dg.resize(m);
  for (auto& v : r->dg) v.v.assign(n, 0.);
  r->mma = new MMA(n, m, &r->x);
  if (robust_a) {
    std::vector<double> a(robust_a, robust_a + m);
    r->mma->SetRobustConstants(a.data());
  }
  return r;
}

/* x <- MMA update (Update with the outer move limit on [0,1]); *change = max |x_new - x_old| */
int ref_mma_update(void* h, double* x, const double* df0dx, const double* g, const double* dgdx,
                   double movlim, double* change) {
  ref_mma* r = (ref_mma*)h;
  std::memcpy(r->x.v.data(), x, sizeof(double) * r->n);
  std::memcpy(r->df0.v.data(), df0dx, sizeof(double) * r->n);
  std::vector<Vec> dgv(r->m);
  for (int j = 0; j < r->m; ++j) {
    std::memcpy(r->dg[j].v.data(), dgdx + (size_t)j * r->n, sizeof(double) * r->n);
    dgv[j] = &r->dg[j];
  }
  std::vector<double> gv(g, g + r->m);
  int rc = r->mma->Update(&r->x, &r->df0, gv.data(), dgv.data(), movlim);
  double ch = 0.;
  r->mma->DesignChange(&r->x, ch);
  if (change) *change = ch;
  std::memcpy(x, r->x.v.data(), sizeof(double) * r->n);
  return rc;
}

void ref_mma_destroy(void* h) {
  ref_mma* r = (ref_mma*)h;
  delete r->mma;
  delete r;
}

}  // extern "C"
