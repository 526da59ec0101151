// cfdgb_run: command-line driver over the C ABI, the counterpart of the reference's
// `mx` executable (src/CFD_MX.cpp:12 -> runSeqOmp).  Parameters are key=value pairs
// instead of compile-time constants:
//
//   cfdgb_run nx=96 ny=48 nz=4 lx=24 ly=12 lz=1 cx=6 cy=6 Re=100 dt=0.005 steps=200 \
//             solver=bicgstab|jacobi|rbsor|cg precision=fp64|mixed tol=1e-8 [out=Information]
//             [solver=cg amp=1e-3 seed=1234 project_rhs=1 inner_tol=0 max_outer=400 maxit=5000]
//             [p3d=N: Plot3D grid file <out>/P3D.x and a solution file <out>/P3D<nn>.q
//              every N steps, byte-compatible with the reference's writers]
//             [scheme=quick|lud|ud: the convection switch (inc/0_General.hpp:114-118);
//              les=1: the Smagorinsky model (TERBULENCE_SMAGORINSKY);
//              walls=free_slip: the free-slip y-wall rows of the boundary table;
//              bc_z=periodic: periodic z; outflow=convective: the convective outflow with
//              the mass-flux correction (neither is in the reference);
//              precond=multigrid: the FP32 multigrid V-cycle preconditioning the MIXED
//              BiCGSTAB sweeps]
//             [restart=<file.q>: start from a Plot3D solution file of this grid (QfileRead,
//              the restart the reference leaves commented out at src/RUN_CPU.cpp:88-99);
//              the simulated time continues from the file's header]
//             [adjoint=first:last:ckpt: instead of the step loop, cfdgb_forward over `steps`
//              steps (drag averaged over steps first..last, a checkpoint every ckpt steps)
//              and cfdgb_backward; prints J, the gradients' norms and both wall times]
//
// Per step it prints the reference's lines ("[SPE (BICG)] iter:...", "[cD, cL] : ...")
// and appends the drag/lift series to <out>/Time_cDcL.dat in the reference's Tecplot
// layout (inc/dfib/virtualForceIntergrator.hpp:113-145).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "cfdgb.hpp"

int main(int argc, char **argv) {
  cfdgb_config cfg;
  cfdgb_config_default(&cfg);
  std::map<std::string, std::string> kv;
  for (int a = 1; a < argc; ++a) {
    const char *eq = std::strchr(argv[a], '=');
    if (!eq) {
      std::fprintf(stderr, "expected key=value, got %s\n", argv[a]);
      return 2;
    }
    kv[std::string(argv[a], (size_t)(eq - argv[a]))] = eq + 1;
  }
  auto num = [&](const char *k, double d) { return kv.count(k) ? std::atof(kv[k].c_str()) : d; };
  cfg.nx = (int)num("nx", cfg.nx); cfg.ny = (int)num("ny", cfg.ny); cfg.nz = (int)num("nz", cfg.nz);
  cfg.lx = num("lx", cfg.lx); cfg.ly = num("ly", cfg.ly); cfg.lz = num("lz", cfg.lz);
  cfg.cx = num("cx", cfg.cx); cfg.cy = num("cy", cfg.ly / 2.0); cfg.radius = num("radius", cfg.radius);
  cfg.Re = num("Re", cfg.Re); cfg.dt = num("dt", cfg.dt); cfg.tol = num("tol", cfg.tol);
  cfg.maxit = (int)num("maxit", cfg.maxit); cfg.omega = num("omega", cfg.omega);
  cfg.inner_tol = num("inner_tol", cfg.inner_tol); cfg.max_outer = (int)num("max_outer", cfg.max_outer);
  cfg.amp = num("amp", 0.0); cfg.seed = (uint64_t)num("seed", 0.0);
  cfg.project_rhs = (int)num("project_rhs", 0.0);
  const std::string scheme = kv.count("scheme") ? kv["scheme"] : "quick";
  cfg.scheme = scheme == "lud" ? CFDGB_LUD : scheme == "ud" ? CFDGB_UD : CFDGB_QUICK;
  cfg.les = (int)num("les", 0.0);
  cfg.walls = (kv.count("walls") && kv["walls"] == "free_slip") ? CFDGB_WALLS_FREE_SLIP : CFDGB_WALLS_ZERO_GRADIENT;
  cfg.precond = (kv.count("precond") && kv["precond"] == "multigrid") ? CFDGB_PRECOND_MULTIGRID : CFDGB_PRECOND_NONE;
  cfg.bc_z = (kv.count("bc_z") && kv["bc_z"] == "periodic") ? CFDGB_Z_PERIODIC : CFDGB_Z_ZERO_GRADIENT;
  cfg.outflow = (kv.count("outflow") && kv["outflow"] == "convective") ? CFDGB_OUTFLOW_CONVECTIVE
                                                                         : CFDGB_OUTFLOW_ZERO_GRADIENT;
  const std::string solver = kv.count("solver") ? kv["solver"] : "bicgstab";
  cfg.solver = solver == "jacobi" ? CFDGB_BICGSTAB_JACOBI
               : solver == "rbsor"  ? CFDGB_RBSOR
               : solver == "cg"     ? CFDGB_CG
                                    : CFDGB_BICGSTAB;
  cfg.precision = (kv.count("precision") && kv["precision"] == "mixed") ? CFDGB_MIXED : CFDGB_FP64;
  const int steps = (int)num("steps", 200);
  const int p3d = (int)num("p3d", 0);  // Plot3D solution file every p3d steps (0: none)
  const std::string out = kv.count("out") ? kv["out"] : "Information";
  try {
    cfdgb::Context ctx(cfg);
    cfdgb::velocity T0;
    cfdgb::pressure t1;
    ctx.resize(T0);
    ctx.resize(t1);
    std::fill(T0.u.begin(), T0.u.end(), 1.0);  // iniU(1, 0, 0), RUN_CPU.cpp:66-76
    cfdgb::check(cfdgb_init_fields(ctx.handle(), nullptr, nullptr, nullptr, nullptr));
    double time = 0.0;
    if (kv.count("restart")) {  // head: blocks, mach, alpha, Re, time
      double head[5];
      cfdgb::check(cfdgb_read_plot3d(ctx.handle(), kv["restart"].c_str(), head));
      time = head[4];
    }
    if (kv.count("adjoint")) {  // first:last:ckpt
      cfdgb_objective obj{};
      obj.nsteps = steps;
      if (std::sscanf(kv["adjoint"].c_str(), "%d:%d:%d", &obj.first, &obj.last, &obj.ckpt_every) != 3) {
        std::fprintf(stderr, "adjoint=first:last:ckpt expected\n");
        return 2;
      }
      double J = 0.0;
      const auto t0 = std::chrono::steady_clock::now();
      const int rf = cfdgb_forward(ctx.handle(), &obj, &J);
      if (rf != CFDGB_OK && rf != CFDGB_ENOCONV) cfdgb::check(rf);
      const auto t1 = std::chrono::steady_clock::now();
      std::vector<double> gin((size_t)cfg.ny * cfg.nz), geta((size_t)(cfg.nx + 4) * (cfg.ny + 4) * (cfg.nz + 4));
      const int rb = cfdgb_backward(ctx.handle(), gin.data(), geta.data());
      if (rb != CFDGB_OK && rb != CFDGB_ENOCONV) cfdgb::check(rb);
      const auto t2 = std::chrono::steady_clock::now();
      double ni = 0.0, ne = 0.0;
      for (double x : gin) ni += x * x;
      for (double x : geta) ne += x * x;
      const double tf = std::chrono::duration<double>(t1 - t0).count(), tb = std::chrono::duration<double>(t2 - t1).count();
      std::printf("J %.12g |dJ/dinlet| %.9g |dJ/deta| %.9g forward %.3f s backward %.3f s ratio %.3f\n", J,
                  std::sqrt(ni), std::sqrt(ne), tf, tb, tb / tf);
      return rf == CFDGB_OK && rb == CFDGB_OK ? 0 : 3;
    }
    mkdir(out.c_str(), 0755);
    FILE *f = std::fopen((out + "/Time_cDcL.dat").c_str(), "w");
    if (f) std::fprintf(f, "TITLE     = \"\"\nVARIABLES = \"simulation time\",\"C<sub>D</sub>\",\"C<sub>L</sub>\"\nZONE T=\"%s\"",
                        solver == "rbsor" ? "SOR" : solver == "jacobi" ? "CSR (BICG)" : solver == "cg" ? "ELL (CG)" : "SPE (BICG)");
    int worst = 0;
    if (p3d > 0) cfdgb::check(cfdgb_write_plot3d(ctx.handle(), (out + "/P3D.x").c_str(), nullptr, 0.0));
    for (int s = 0; s < steps; ++s) {
      cfdgb_step_stats st{};
      const int rc = cfdgb_step(ctx.handle(), 1, &st);
      if (rc != CFDGB_OK && rc != CFDGB_ENOCONV) cfdgb::check(rc);
      if (rc < worst) worst = rc;
      std::printf("[%s] iter:%d, error %g\n[cD, cL] : %g, %g\n", solver.c_str(), st.iters, st.relres, st.cd, st.cl);
      if (f) std::fprintf(f, "\n%.17g %.17g %.17g", time, st.cd, st.cl);
      time += cfg.dt;
      if (p3d > 0 && (s + 1) % p3d == 0) {  // qfile.hpp: P3D<nn>.q, nn the file counter
        char name[64];
        std::snprintf(name, sizeof(name), "/P3D%02d.q", (s + 1) / p3d);
        cfdgb::check(cfdgb_write_plot3d(ctx.handle(), nullptr, (out + name).c_str(), time));
      }
    }
    if (f) std::fclose(f);
    return worst == CFDGB_OK ? 0 : 3;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
}
