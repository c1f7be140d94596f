// A reference-style C++ driver on the C++ facade (include/lbmgpu.hpp): the
// loop structure of applications/RobustPump2d/robustPump2d.cc:234-276 with the
// solver, adjoint solver and checkpointing swapped for the GPU classes.
// Reads a D2Q9 channel set-up from argv, prints J, dJ/dgamma and f as text.
// Test infrastructure: the pytest suite compiles it and checks its output
// against the oracle.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../include/lbmgpu.hpp"

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: cpp_driver nx ny nsteps design.bin\n");
    return 2;
  }
  const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nsteps = std::atoi(argv[3]);
  std::vector<double> gamma((size_t)nx * ny);
  FILE* fp = std::fopen(argv[4], "rb");
  if (!fp || std::fread(gamma.data(), sizeof(double), gamma.size(), fp) != gamma.size()) return 3;
  std::fclose(fp);

  lbm_config cfg;
  lbm_config_default(&cfg);
  cfg.lattice = LBM_D2Q9;
  cfg.collision = LBM_BGK;
  cfg.nx = nx;
  cfg.ny = ny;
  cfg.nz = 1;
  cfg.omega = 1. / 0.8;
  cfg.interp_scale = 0.1;   // alpha_max = 0.05
  cfg.interp_q = 0.1;
  cfg.nbc = 2;
  lbm_bc in = {LBM_BC_VELOCITY, LBM_FACE_WEST, LBM_PROFILE_PARABOLIC, {0, 0, 1, ny - 2, 0, 0}, 0.05, 0., 1.};
  lbm_bc out = {LBM_BC_PRESSURE, LBM_FACE_EAST, LBM_PROFILE_UNIFORM, {nx - 1, nx - 1, 1, ny - 2, 0, 0}, 1., 0., 1.};
  cfg.bc[0] = in;
  cfg.bc[1] = out;
  cfg.objective = LBM_OBJ_PRESSURE_DROP;
  for (int i = 0; i < 6; ++i) {
    cfg.obj_in[i] = in.box[i];
    cfg.obj_out[i] = out.box[i];
  }
  cfg.obj_weight = 1. / nsteps;

  lbmgpu::IsothermalLBSolver solver;
  int ierr = solver.make(cfg);
  if (ierr) {
    std::fprintf(stderr, "make: %s\n", solver.lastError().c_str());
    return 1;
  }
  if ((ierr = solver.setFieldFromDesignVec(gamma))) return 1;

  // forward sweep with the objective, reference style
  if ((ierr = solver.initializeAtEquilibrium())) return 1;
  double J = 0.;
  if ((ierr = solver.collideAndStream(nsteps, &J))) return 1;
  std::vector<double> f;
  if ((ierr = solver.getDistributions(&f))) return 1;

  // checkpointed forward + reverse sweep
  lbmgpu::LBDynamicCheckpointing check(8, solver);
  double Jg = 0.;
  std::vector<double> sens;
  lbm_gradient_stats st;
  if ((ierr = check.objectiveAndGradient(nsteps, &Jg, &sens, &st))) {
    std::fprintf(stderr, "gradient: %s\n", solver.lastError().c_str());
    return 1;
  }
  // the same with the static placement, constructed as applications/pump2d/pump2d.cc:146
  lbmgpu::LBStaticCheckpointing scheck(8, nsteps + 1, solver);
  double Js = 0.;
  std::vector<double> ssens;
  lbm_gradient_stats sst;
  if ((ierr = scheck.objectiveAndGradient(nsteps, &Js, &ssens, &sst))) {
    std::fprintf(stderr, "static gradient: %s\n", solver.lastError().c_str());
    return 1;
  }
  const bool same = Js == Jg && ssens == sens;
  std::printf("J %.17g\nJgrad %.17g\nrecomputed %lld\n", J, Jg, (long long)st.recomputed_steps);
  std::printf("static_same %d\nstatic_recomputed %lld\n", same ? 1 : 0,
              (long long)sst.recomputed_steps);
  std::printf("sens");
  for (double s : sens) std::printf(" %.17g", s);
  std::printf("\nf");
  for (double v : f) std::printf(" %.17g", v);
  std::printf("\n");
  return 0;
}
