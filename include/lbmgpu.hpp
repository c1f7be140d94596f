// lbmgpu.hpp -- header-only C++ facade over the C ABI of lbmgpu.h that keeps
// the method names of the reference's solver classes, so a reference-style
// driver (applications/RobustPump2d/robustPump2d.cc:234-276) ports by
// swapping types:
//
//   IsothermalLBSolver2d<Op>          -> lbmgpu::IsothermalLBSolver
//     (latticeBoltzmann/isothermalLBSolver2d.hh:20-110, LBSolver.hh:14-73)
//   AdjointLBSolver                   -> lbmgpu::AdjointLBSolver
//     (adjointLatticeBoltzmann/adjointLBSolver.hh:11-46)
//   LBDynamicCheckpointing            -> lbmgpu::LBDynamicCheckpointing
//     (topOpt/LBCheckpointing.hh:20-29)
//
// Errors come back as the ABI's int status (0 = ok), the role PetscErrorCode
// plays in the reference; lastError() gives the text.
#ifndef LBMGPU_HPP
#define LBMGPU_HPP

#include <cstdint>
#include <string>
#include <vector>

#include "lbmgpu.h"

namespace lbmgpu {

class IsothermalLBSolver {
 public:
  IsothermalLBSolver() = default;
  IsothermalLBSolver(const IsothermalLBSolver&) = delete;
  IsothermalLBSolver& operator=(const IsothermalLBSolver&) = delete;
  ~IsothermalLBSolver() { lbm_destroy(h_); }

  // make(comm, info, op) + addBoundaryCondition(...) of the reference: the
  // whole set-up is one config.
  int make(const lbm_config& cfg) {
    lbm_destroy(h_);
    h_ = nullptr;
    int rc = lbm_create(&cfg, &h_);
    if (rc == LBM_OK) {
      lbm_get_sizes(h_, &ncells_, &npop_);
      cfg_ = cfg;
    }
    return rc;
  }
  // The reference's Input functor of a 2D Zou-He boundary (boundaryConditions/
  // ZouHe2d.hh:37, e.g. InflowVelocity of applications/RobustPump2d/
  // robustPump2d.cc:13-25) for boundary k, whose config has
  // LBM_PROFILE_TABLE: the functor is sampled on the boundary's cells for
  // `period` time steps, reused periodically (t mod period), and handed to
  // lbm_set_bc_profile.  Velocity boundaries take
  //   void operator()(long t, long i, long j, double& ux, double& uy) const;
  template <class Input>
  int setVelocityInput(int k, int period, const Input& in) {
    std::vector<double> tab;
    int npos = sample(k, period, 2, &tab, [&](long t, long i, long j, double* v) {
      in(t, i, j, v[0], v[1]);
    });
    if (npos < 0) return LBM_ERR_ARG;
    return lbm_set_bc_profile(h_, k, period, 2, tab.data());
  }
  // Pressure and temperature boundaries take
  //   void operator()(long t, long i, long j, double& value) const;
  // whose value multiplies the boundary's value * T(t) (a config value of 1
  // with no oscillation takes the functor's value as it is).
  template <class Input>
  int setScalarInput(int k, int period, const Input& in) {
    std::vector<double> tab;
    int npos = sample(k, period, 1, &tab, [&](long t, long i, long j, double* v) {
      in(t, i, j, v[0]);
    });
    if (npos < 0) return LBM_ERR_ARG;
    return lbm_set_bc_profile(h_, k, period, 1, tab.data());
  }
  // LBSolver::setFieldFromDesignVec (LBSolver.cc:333-348)
  int setFieldFromDesignVec(const std::vector<double>& gamma) {
    if ((int64_t)gamma.size() != ncells_) return LBM_ERR_ARG;
    return lbm_set_design(h_, gamma.data());
  }
  // LBSolver::initializeAtEquilibrium (LBSolver.cc:234-249); macros empty = rest
  int initializeAtEquilibrium(const std::vector<double>& macros = {}) {
    return lbm_init_equilibrium(h_, macros.empty() ? nullptr : macros.data());
  }
  // collide() + stream() (LBSolver.cc:163-206) n times, with the objective of
  // every new state summed into *value (computeMacroFunctional, LBSolver.cc:74-91)
  int collideAndStream(int n = 1, double* value = nullptr) {
    return lbm_forward(h_, n, nullptr, value);
  }
  int getCurrentTimestep(int* t) const { return lbm_get_time(h_, t); }
  int getDistributions(std::vector<double>* f) const {
    f->resize((size_t)ncells_ * npop_);
    return lbm_get_populations(h_, f->data());
  }
  // LBSolver::setDistributions + setCurrentTimestep (LBSolver.cc:65-97)
  int setDistributions(const std::vector<double>& f, int t) {
    if ((int64_t)f.size() != ncells_ * npop_) return LBM_ERR_ARG;
    return lbm_set_populations(h_, f.data(), t);
  }
  int getMacros(std::vector<double>* mac, int nmac) const {
    mac->resize((size_t)ncells_ * nmac);
    return lbm_get_macros(h_, mac->data());
  }
  int autotune(int nsteps = 5) { return lbm_autotune(h_, nsteps); }
  std::string lastError() const { return lbm_last_error(h_); }
  lbm_handle* handle() const { return h_; }
  int64_t numCells() const { return ncells_; }
  int numPopulations() const { return npop_; }

 private:
  // values of boundary k's cells (along the face: y on west/east faces, x on
  // south/north faces) for t = 0..period-1; -1 for a bad boundary or period
  template <class F>
  int sample(int k, int period, int ncomp, std::vector<double>* tab, F f) const {
    if (!h_ || k < 0 || k >= cfg_.nbc || period < 1) return -1;
    const lbm_bc& b = cfg_.bc[k];
    const bool yface = b.face == LBM_FACE_SOUTH || b.face == LBM_FACE_NORTH;
    const int s0 = yface ? b.box[0] : b.box[2], s1 = yface ? b.box[1] : b.box[3];
    const int npos = s1 - s0 + 1;
    tab->assign((size_t)period * npos * ncomp, 0.);
    for (int t = 0; t < period; ++t)
      for (int s = s0; s <= s1; ++s) {
        const long i = yface ? s : b.box[0], j = yface ? b.box[2] : s;
        f(t, i, j, tab->data() + ((size_t)t * npos + (s - s0)) * ncomp);
      }
    return npos;
  }

  lbm_handle* h_ = nullptr;
  lbm_config cfg_{};
  int64_t ncells_ = 0;
  int npop_ = 0;
};

// The reverse sweep works on the forward solver's handle: its state is the
// f_t the reverse step differentiates (getForwardSolution places it there).
class AdjointLBSolver {
 public:
  explicit AdjointLBSolver(IsothermalLBSolver& s) : s_(s) {}
  // AdjointLBSolver::resetAdjoints (adjointLBSolver.cc:138-145)
  int resetAdjoints() { return lbm_adjoint_reset(s_.handle()); }
  // adjointCollide + computeCollideSource + computeSensitivitySource +
  // adjointStream (adjointLBSolver.cc:28-122) at the state held by the solver
  int adjointStep() { return lbm_adjoint_step(s_.handle()); }
  // AdjointLBSolver::getSensitivities (adjointLBSolver.cc:153-157)
  int getSensitivities(std::vector<double>* sens) const {
    sens->resize((size_t)s_.numCells());
    return lbm_get_sensitivity(s_.handle(), sens->data());
  }
  int getAdjoints(std::vector<double>* lam) const {
    lam->resize((size_t)s_.numCells() * s_.numPopulations());
    return lbm_get_adjoint(s_.handle(), lam->data());
  }

 private:
  IsothermalLBSolver& s_;
};

// Forward sweep with Wang et al. dynamic checkpointing in device memory, the
// reverse sweep, and dJ/dgamma: the driver loop of robustPump2d.cc:234-276
// with LBDynamicCheckpointing (topOpt/LBCheckpointing.cc:37-65) as one call.
class LBDynamicCheckpointing {
 public:
  LBDynamicCheckpointing(int numCheckpoints, IsothermalLBSolver& s) : k_(numCheckpoints), s_(s) {}
  virtual ~LBDynamicCheckpointing() = default;
  int objectiveAndGradient(int numSteps, double* J, std::vector<double>* sens,
                           lbm_gradient_stats* stats = nullptr) {
    sens->resize((size_t)s_.numCells());
    return lbm_gradient_schedule(s_.handle(), numSteps, k_, schedule(), J, sens->data(), stats);
  }

 protected:
  virtual int schedule() const { return LBM_SCHEDULE_DYNAMIC; }

 private:
  int k_;
  IsothermalLBSolver& s_;
};

// LBStaticCheckpointing(numCheckpoints, numTimesteps, solver)
// (topOpt/LBCheckpointing.cc:4-35): placement planned before the sweep for
// numTimesteps - 1 steps, as applications/pump2d/pump2d.cc:146 constructs it.
class LBStaticCheckpointing : public LBDynamicCheckpointing {
 public:
  LBStaticCheckpointing(int numCheckpoints, int numTimesteps, IsothermalLBSolver& s)
      : LBDynamicCheckpointing(numCheckpoints, s), nt_(numTimesteps) {}
  // the reference plans for numTimesteps - 1 steps; other sweep lengths are refused
  int objectiveAndGradient(int numSteps, double* J, std::vector<double>* sens,
                           lbm_gradient_stats* stats = nullptr) {
    if (numSteps != nt_ - 1) return LBM_ERR_ARG;
    return LBDynamicCheckpointing::objectiveAndGradient(numSteps, J, sens, stats);
  }

 protected:
  int schedule() const override { return LBM_SCHEDULE_STATIC; }

 private:
  int nt_;
};

}  // namespace lbmgpu

#endif  // LBMGPU_HPP
