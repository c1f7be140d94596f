// The robust pump's set-up (applications/RobustPump2d/robustPump2d.cc:52-104)
// driven through the C++ facade (include/lbmgpu.hpp) with a reference-style
// Input functor: MRT + partial bounce-back on an n x n lattice, Zou-He pressure
// segments west and east, a north Zou-He velocity inlet whose velocity is the
// functor below (the same signature and law as the reference's
// InflowVelocity), and the through-flow objective over the two pressure
// segments.  Prints J and dJ/dgamma as text.  Test infrastructure: the pytest
// suite compiles it and checks its output against the oracle.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../include/lbmgpu.hpp"

namespace {

// u_y = -sin(2 pi t / freq) vmax (r^2 - (i - mid)^2) / r^2, u_x = 0
struct InflowVelocity {
  void operator()(long timestep, long idx, long, double& ux, double& uy) const {
    ux = 0.;
    uy = -std::sin(2. * M_PI * timestep / freq) * (vmax * (inletRad * inletRad - (idx - mid) * (idx - mid))) /
         (inletRad * inletRad);
  }
  double vmax;
  double mid;
  double inletRad;
  long freq;
};

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: cpp_pump_driver n nsteps freq design.bin\n");
    return 2;
  }
  const int n = std::atoi(argv[1]), nsteps = std::atoi(argv[2]), freq = std::atoi(argv[3]);
  const int th = n / 3;
  std::vector<double> gamma((size_t)n * n);
  FILE* fp = std::fopen(argv[4], "rb");
  if (!fp || std::fread(gamma.data(), sizeof(double), gamma.size(), fp) != gamma.size()) return 3;
  std::fclose(fp);

  lbm_config cfg;
  lbm_config_default(&cfg);
  cfg.lattice = LBM_D2Q9;
  cfg.collision = LBM_MRT;
  cfg.nx = cfg.ny = n;
  cfg.nz = 1;
  cfg.omega = 1. / 0.8;
  cfg.mrt[0] = 1.4;   // IncompressibleMRT2d's rates (incompressibleMRT2d.hh:88-90)
  cfg.mrt[1] = 1.4;
  cfg.mrt[2] = 1.2;
  cfg.interp_scale = 0.1;
  cfg.interp_q = 0.1;
  cfg.nbc = 3;
  lbm_bc west = {LBM_BC_PRESSURE, LBM_FACE_WEST, LBM_PROFILE_UNIFORM, {0, 0, th + 1, 2 * th, 0, 0}, 1., 0., 1.};
  lbm_bc east = {LBM_BC_PRESSURE, LBM_FACE_EAST, LBM_PROFILE_UNIFORM, {n - 1, n - 1, th + 1, 2 * th, 0, 0}, 1., 0., 1.};
  lbm_bc north = {LBM_BC_VELOCITY, LBM_FACE_NORTH, LBM_PROFILE_TABLE, {th + 1, 2 * th, n - 1, n - 1, 0, 0}, 1., 0., 1.};
  cfg.bc[0] = west;
  cfg.bc[1] = east;
  cfg.bc[2] = north;
  cfg.objective = LBM_OBJ_THROUGH_FLOW;
  for (int i = 0; i < 6; ++i) {
    cfg.obj_in[i] = west.box[i];
    cfg.obj_out[i] = east.box[i];
  }
  cfg.obj_weight = 1. / nsteps;

  lbmgpu::IsothermalLBSolver solver;
  if (solver.make(cfg)) {
    std::fprintf(stderr, "make: %s\n", solver.lastError().c_str());
    return 1;
  }
  InflowVelocity vf;
  vf.vmax = 0.05;
  vf.mid = (double)(n - 1) / 2.;
  vf.inletRad = (double)th / 2.;
  vf.freq = freq;
  if (solver.setVelocityInput(2, freq, vf)) {
    std::fprintf(stderr, "input: %s\n", solver.lastError().c_str());
    return 1;
  }
  if (solver.setFieldFromDesignVec(gamma)) return 1;
  if (solver.initializeAtEquilibrium()) return 1;
  lbmgpu::LBStaticCheckpointing check(10, nsteps + 1, solver);   // robustPump2d.cc:166
  double J = 0.;
  std::vector<double> sens;
  if (check.objectiveAndGradient(nsteps, &J, &sens)) {
    std::fprintf(stderr, "gradient: %s\n", solver.lastError().c_str());
    return 1;
  }
  std::printf("J %.17g\nsens", J);
  for (double s : sens) std::printf(" %.17g", s);
  std::printf("\n");
  return 0;
}
