// Test driver for the C++ shim (include/cfdgb.hpp): the reference's call sequence of one
// projection step (src/RUN_CPU.cpp:257-436) written as a reference driver would write it,
// plus get_Cfl, SmagorinskyModel and a Plot3D write / QfileRead round trip.  Prints the
// numbers the test compares with the oracle.
#include <cstdio>
#include <string>

#include "cfdgb.hpp"

int main(int argc, char **argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";
  cfdgb_config cfg;
  cfdgb_config_default(&cfg);  // the reference's 96x48x4 case
  cfg.tol = 1e-12;
  cfdgb::Context ctx(cfg);
  cfdgb::velocity T0, T1, T3;
  cfdgb::pressure t1;
  cfdgb::DfibArray Dfib;
  cfdgb::MxClass Mx;
  ctx.resize(T0);
  ctx.resize(t1);
  for (auto &x : T0.u) x = 1.0;  // iniU(1, 0, 0)
  T1 = T0;                       // src/RUN_CPU.cpp:104-109
  T3 = T0;
  cfdgb::DFIB_CylinderZ(ctx, Dfib);
  cfdgb::BC_staggered_main(ctx, T0, t1);
  cfdgb::BC_staggered_copy(ctx, T0, T1);
  cfdgb::bicgstabRe2 solver(ctx);
  solver.setTolerance(cfg.tol);
  for (int loop = 1; loop <= 3; ++loop) {
    cfdgb::ConvectionDifussion(ctx, T0, T1);
    if (loop > 1) {
      cfdgb::createBMatrix_omp(ctx, T1, Mx);
      Mx.X_result.resize(ctx.iceltotCal(), 0.0);
      solver.solve(Mx.matB, Mx.X_result);
      cfdgb::Pressure_transform_X_result(ctx, t1, Mx);
    }
    cfdgb::update_UandF_omp(ctx, Dfib, t1, T1, T3);
    T0 = T3;  // copyVel
    cfdgb::BC_staggered_main(ctx, T0, t1);
    cfdgb::BC_staggered_copy(ctx, T0, T1);
    std::printf("cd %d %.17g\n", loop, Dfib.cD);
  }
  const cfdgb::Cfl c = cfdgb::get_Cfl(ctx, T1);
  std::printf("cfl %.17g\n", c.cfl_max);
  cfdgb::SmagorinskyModel(ctx, T0);
  double vmax = 0.0;
  for (double x : T0.Viseff) vmax = x > vmax ? x : vmax;
  std::printf("viseff_max %.17g\n", vmax);
  // the Plot3D file of a state and the reference's reader of it
  cfdgb::runSeqOmp(ctx, T0, t1, 2);
  const std::string q = dir + "/shim.q";
  cfdgb::OutputPLOT3D_Qfile(ctx, 0.5, q);
  auto [nb, mach, alpha, reyn, time, p, u, v, w, eta] = cfdgb::QfileRead(ctx, q);
  std::printf("qfile %d %.9g %.9g %zu\n", nb, (double)reyn, (double)time, u.size());
  return 0;
}
