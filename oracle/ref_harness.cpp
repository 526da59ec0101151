// Oracle harness: drives the reference solver's OWN functions (headers compiled from the
// patched copy that oracle/build_ref.py stages under oracle/_ref/src) and dumps FP64
// fields as raw little-endian arrays.  Test infrastructure only.
//
//   ref_<grid> run  <steps> <Re> <dt> <tol> <spe|csr|sor> <omega> <seed> <amp> <outdir> [cap]
// (cap: optional BiCGSTAB iteration cap in place of the reference's 5000, for bounded
// timing samples; stats.txt then also carries per-step wall times of the whole step and
// of the pressure solve.)
//   ref_<grid> unit <seed> <Re> <dt> <outdir>
//
// "run" replays runSeqOmp (src/RUN_CPU.cpp:9-436) step by step: set-up :50-236, then
// per step ConvectionDifussion (:268), pressure only when loop > 1 (:287/:303),
// update_UandF_omp (:369), copyVel (:391), BC_staggered_main + BC_staggered_copy
// (:399-400) and CD_CL (:407).  Diagnostics that only print (get_Cfl, the p min/max,
// CheckSteadyStatebyMaxVal) and file output are left out; they do not feed back.
// Added hooks: a seeded perturbation of the initial interior velocity (splitmix64,
// defined identically in oracle/cfd_oracle.c and the CUDA library's host code), an
// explicit step count and tolerance, and the dumps.
//
// "unit" calls each hot-path function once on seeded random fields of this grid and
// dumps inputs and outputs (golden vectors for the per-function parity tests).
// Built with the convection switch set to LUD or UD, or with TERBULENCE_SMAGORINSKY (the
// reference's Smagorinsky model, called before ConvectionDifussion as at
// src/RUN_CPU.cpp:261-263), both modes use those instead.
// Standard headers first, so that the access override below reaches only the
// reference's own classes: it lets the bounded CPU-baseline sample set bicgstabRe2's
// private iteration cap (iters_max_, bicgstabRe2.hpp:47); no arithmetic changes.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <tuple>
#include <unordered_set>
#include <utility>
#include <vector>
#include <omp.h>
#define private public
#include "0_General.hpp"
#include "run/general.hpp"
#undef private

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>

namespace {

uint64_t splitmix64(uint64_t &s) {
  s += 0x9E3779B97F4A7C15ULL;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
// uniform in [-1, 1): 53 random bits
double sym_uniform(uint64_t &s) {
  const double r = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
  return 2.0 * r - 1.0;
}

void copy_bytes(const std::string &from, const std::string &to) {
  std::ifstream in(from, std::ios::binary);
  std::ofstream o(to, std::ios::binary);
  if (!in || !o) { std::fprintf(stderr, "copy %s -> %s failed\n", from.c_str(), to.c_str()); std::exit(3); }
  o << in.rdbuf();
}

void dump(const std::string &dir, const std::string &name, const std::vector<double> &a) {
  std::string p = dir + "/" + name + ".f64";
  FILE *f = std::fopen(p.c_str(), "wb");
  if (!f) { std::perror(p.c_str()); std::exit(3); }
  std::fwrite(a.data(), sizeof(double), a.size(), f);
  std::fclose(f);
}

void perturb(velocity &T, grid &gA, uint64_t seed, double amp) {
  uint64_t s = seed;
  std::vector<double> *fs[3] = {&T.u, &T.v, &T.w};
  for (auto *f : fs)
    for (int i = gA.gC; i < gA.nx - gA.gC; ++i)
      for (int j = gA.gC; j < gA.ny - gA.gC; ++j)
        for (int k = gA.gC; k < gA.nz - gA.gC; ++k)
          (*f)[gA.icel(i, j, k)] += amp * sym_uniform(s);
}

void fill_random(std::vector<double> &a, uint64_t &s, double offset, double scale) {
  for (auto &x : a) x = offset + scale * sym_uniform(s);
}

int run_mode(int argc, char **argv) {
  if (argc < 11) { std::fprintf(stderr, "run: bad args\n"); return 2; }
  const int steps = std::atoi(argv[2]);
  const double Re = std::atof(argv[3]), dt = std::atof(argv[4]), tol = std::atof(argv[5]);
  const std::string solver = argv[6];
  const double omega = std::atof(argv[7]);
  const uint64_t seed = std::strtoull(argv[8], nullptr, 10);
  const double amp = std::atof(argv[9]);
  const std::string out = argv[10];
  const int cap = argc > 11 ? std::atoi(argv[11]) : 0;

  grid gA;
  simpulationVariable simu;
  simu.set_time_max(steps * dt);
  simu.set_dt(dt);
  simu.set_Re(Re);
  simu.p_criteria = tol;
  simu.p_sor_omega = omega;
  simu.DfibMethod = "DFIB_Cylinder-Z";
  simu.Locality = 1;

  DfibArray Dfib; pressure t1; velocity T0, T1, T3;
  SORcoefficient Sor; shareMenory ShareM; MxClass Mx;
  divideLocal Lo;
  std::vector<int> grid_size{gA.nx, gA.ny, gA.nz}, dims{1, 1, 1};
  Lo.initTable(grid_size, dims);
  Lo.initLocal(0, 0, 0);
  resize_variable(gA, simu, t1, T0, T1, T3, Dfib);
  T0.iniU_omp(1.0, 0.0, 0.0); T1.iniU_omp(1.0, 0.0, 0.0); T3.iniU_omp(1.0, 0.0, 0.0);
  t1.init_p(0.0);
  generateGride(simu, ShareM, Lo, gA);
  if (amp != 0.0) perturb(T0, gA, seed, amp);
  T1.u = T3.u = T0.u; T1.v = T3.v = T0.v; T1.w = T3.w = T0.w;
  BC_staggered_main(Lo, T0, t1, gA);
  BC_staggered_copy(Lo, T0, T1, gA);
  dump(out, "u0", T0.u); dump(out, "v0", T0.v); dump(out, "w0", T0.w);

  Mx.X_result.resize(gA.iceltotCal, 0.0);
  std::unique_ptr<solver::bicgstabRe2<mat::SPE_matrix<double>>> spe;
  std::unique_ptr<solver::bicgstabRe2<mat::CSR_matrix<double>>> csr;
  if (solver == "spe") {
    Mx.matA_spe.resize(gA.nxCal, gA.nyCal, gA.nzCal);
    Mx.matA_spe.setupPressure(gA.gC, gA.Dx, gA.Dy, gA.Dz, gA.Dxs, gA.Dys, gA.Dzs);
    spe.reset(new solver::bicgstabRe2<mat::SPE_matrix<double>>(Mx.matA_spe));
    spe->setTolerance(tol);
    if (cap > 0) spe->iters_max_ = cap;
  } else if (solver == "csr") {
    Mx.matA_csr.set(gA.createPressureMatrixCSR());
    csr.reset(new solver::bicgstabRe2<mat::CSR_matrix<double>>(Mx.matA_csr));
    csr->setTolerance(tol);
    if (cap > 0) csr->iters_max_ = cap;
  } else if (solver != "sor") {
    std::fprintf(stderr, "unknown solver %s\n", solver.c_str()); return 2;
  }

  std::fill(Dfib.eta.begin(), Dfib.eta.end(), 0.0);
  DFIB_CylinderZ(Dfib, Lo, gA);
  dump(out, "eta", Dfib.eta);

  std::string stats = out + "/stats.txt";
  FILE *fs = std::fopen(stats.c_str(), "w");
  std::fprintf(fs, "# step time iters err cd cl t_step_s t_solve_s\n");
  using clk = std::chrono::steady_clock;
  for (int s = 1; s <= steps; ++s) {
    const auto t0 = clk::now();
    simu.loop = s;
#ifdef TERBULENCE_SMAGORINSKY
    SmagorinskyModel(ShareM, simu, T0, t1, Lo, gA);  // src/RUN_CPU.cpp:261-263
#endif
    ConvectionDifussion(simu, T0, T1, Lo, gA);
    simu.iters = 0; simu.error = 0.0;
    auto ts0 = clk::now(), ts1 = ts0;
    if (simu.loop > 1) {
      if (solver == "sor") {
        SorPipeLine_omp(ShareM, Sor, simu, T1, t1, Lo, gA);
      } else {
        createBMatrix_omp(T1, Mx, simu, Lo, gA);
        ts0 = clk::now();
        if (spe) std::tie(simu.iters, simu.error) = spe->solve(Mx.matB, Mx.X_result);
        else std::tie(simu.iters, simu.error) = csr->solve(Mx.matB, Mx.X_result);
        ts1 = clk::now();
        Pressure_transform_X_result(t1, Mx, Lo, gA);
      }
    }
    update_UandF_omp(Dfib, simu, t1, T1, T3, Lo, gA);
    copyVel(T3, T0);
    BC_staggered_main(Lo, T0, t1, gA);
    BC_staggered_copy(Lo, T0, T1, gA);
    // CD_CL (virtualForceIntergrator.hpp:92-109) without its file output
    virtualF_Int(Dfib, Lo, gA, 0);
    virtualF_Int(Dfib, Lo, gA, 1);
    const double cD = -2.0 * Dfib.ValSum[0] / gA.lz;
    const double cL = -2.0 * Dfib.ValSum[1] / gA.lz;
    const double t_step = std::chrono::duration<double>(clk::now() - t0).count();
    const double t_solve = std::chrono::duration<double>(ts1 - ts0).count();
    std::fprintf(fs, "%d %.17g %d %.17g %.17g %.17g %.6e %.6e\n", s, simu.time, simu.iters, simu.error, cD, cL,
                 t_step, t_solve);
    std::fflush(fs);
    simu.finishloop();
  }
  std::fclose(fs);
  dump(out, "u", T0.u); dump(out, "v", T0.v); dump(out, "w", T0.w);
  dump(out, "p", t1.p);
  dump(out, "us", T1.u); dump(out, "vs", T1.v); dump(out, "ws", T1.w);
  if (!Mx.X_result.empty()) dump(out, "x", Mx.X_result);
  return 0;
}

int unit_mode(int argc, char **argv) {
  if (argc < 6) { std::fprintf(stderr, "unit: bad args\n"); return 2; }
  uint64_t s = std::strtoull(argv[2], nullptr, 10);
  const double Re = std::atof(argv[3]), dt = std::atof(argv[4]);
  const std::string out = argv[5];

  grid gA;
  simpulationVariable simu;
  simu.set_time_max(1.0);
  simu.set_dt(dt);
  simu.set_Re(Re);
  simu.Locality = 1;
  DfibArray Dfib; pressure t1; velocity T0, T1, T3;
  SORcoefficient Sor; shareMenory ShareM; MxClass Mx;
  divideLocal Lo;
  std::vector<int> grid_size{gA.nx, gA.ny, gA.nz}, dims{1, 1, 1};
  Lo.initTable(grid_size, dims);
  Lo.initLocal(0, 0, 0);
  resize_variable(gA, simu, t1, T0, T1, T3, Dfib);
  generateGride(simu, ShareM, Lo, gA);

  // inputs: u has a mean so both QUICK branches occur; everything padded
  fill_random(T0.u, s, 0.3, 1.0); fill_random(T0.v, s, 0.0, 1.0); fill_random(T0.w, s, 0.0, 1.0);
  fill_random(T1.u, s, 0.0, 1.0); fill_random(T1.v, s, 0.0, 1.0); fill_random(T1.w, s, 0.0, 1.0);
  fill_random(T3.u, s, 0.0, 1.0); fill_random(T3.v, s, 0.0, 1.0); fill_random(T3.w, s, 0.0, 1.0);
  fill_random(t1.p, s, 0.0, 1.0);
  fill_random(Dfib.eta, s, 0.5, 0.5);
  std::vector<double> x(gA.iceltotCal);
  fill_random(x, s, 0.0, 1.0);
  dump(out, "in_u", T0.u); dump(out, "in_v", T0.v); dump(out, "in_w", T0.w);
  dump(out, "in_us", T1.u); dump(out, "in_vs", T1.v); dump(out, "in_ws", T1.w);
  dump(out, "in_u3", T3.u); dump(out, "in_v3", T3.v); dump(out, "in_w3", T3.w);
  dump(out, "in_p", t1.p); dump(out, "in_eta", Dfib.eta); dump(out, "in_x", x);

  // 1. convection-diffusion T0 -> copy of T1
  {
    velocity C = T1;
#ifdef TERBULENCE_SMAGORINSKY
    SmagorinskyModel(ShareM, simu, T0, t1, Lo, gA);  // eddy viscosity of T0 (compact)
    dump(out, "les_nut", T0.Viseff);
#endif
    ConvectionDifussion(simu, T0, C, Lo, gA);
    dump(out, "cd_u", C.u); dump(out, "cd_v", C.v); dump(out, "cd_w", C.w);
  }
  // 2. ghost fill of velocity and pressure
  {
    velocity B = T0; pressure P = t1;
    BC_staggered_main(Lo, B, P, gA);
    dump(out, "bc_u", B.u); dump(out, "bc_v", B.v); dump(out, "bc_w", B.w); dump(out, "bc_p", P.p);
    // 3. copy of ghosts + last faces into u*
    velocity C = T1;
    BC_staggered_copy(Lo, B, C, gA);
    dump(out, "bcc_u", C.u); dump(out, "bcc_v", C.v); dump(out, "bcc_w", C.w);
  }
  // 4. right-hand side, unscaled (SPE path) and Jacobi-scaled (CSR path)
  createBMatrix_omp(T1, Mx, simu, Lo, gA);
  dump(out, "b_spe", Mx.matB);
  auto csr_tuple = gA.createPressureMatrixCSR();  // also fills gA.jp
  createBMatrix_omp(T1, Mx, simu, Lo, gA);
  dump(out, "b_jac", Mx.matB);
  dump(out, "jp", gA.jp);
  // 5. operators
  std::vector<double> y(gA.iceltotCal);
  Mx.matA_spe.resize(gA.nxCal, gA.nyCal, gA.nzCal);
  Mx.matA_spe.setupPressure(gA.gC, gA.Dx, gA.Dy, gA.Dz, gA.Dxs, gA.Dys, gA.Dzs);
  Mx.matA_spe.multiply_omp(x, y);
  dump(out, "y_spe", y);
  Mx.matA_csr.set(csr_tuple);
  Mx.matA_csr.multiply_omp(x, y);
  dump(out, "y_csr", y);
  gA.jp.clear();
  // 6. velocity correction + DFIB forcing
  {
    velocity C = T3;
    std::fill(Dfib.f.begin(), Dfib.f.end(), 0.0);
    update_UandF_omp(Dfib, simu, t1, T1, C, Lo, gA);
    dump(out, "uf_u", C.u); dump(out, "uf_v", C.v); dump(out, "uf_w", C.w); dump(out, "uf_f", Dfib.f);
    virtualF_Int(Dfib, Lo, gA, 0);
    virtualF_Int(Dfib, Lo, gA, 1);
    std::vector<double> cdcl{-2.0 * Dfib.ValSum[0] / gA.lz, -2.0 * Dfib.ValSum[1] / gA.lz};
    dump(out, "cdcl", cdcl);
  }
  // 7. solid fraction of the cylinder
  {
    DfibArray D = Dfib;
    std::fill(D.eta.begin(), D.eta.end(), 0.0);
    DFIB_CylinderZ(D, Lo, gA);
    dump(out, "eta_cyl", D.eta);
  }
  // 8. BiCGSTAB (SPE operator) on a consistent right-hand side, warm start 0
  {
    std::vector<double> xt(gA.iceltotCal), rhs(gA.iceltotCal), sol(gA.iceltotCal, 0.0);
    fill_random(xt, s, 0.0, 1.0);
    Mx.matA_spe.multiply_omp(xt, rhs);
    solver::bicgstabRe2<mat::SPE_matrix<double>> bs(Mx.matA_spe);
    bs.setTolerance(1e-10);
    auto [it, err] = bs.solve(rhs, sol);
    dump(out, "bicg_rhs", rhs); dump(out, "bicg_x", sol);
    std::vector<double> ie{(double)it, err};
    dump(out, "bicg_it", ie);
  }
  // 9. SOR sweeps on u* (lexicographic at one thread), capped
  {
    pressure P = t1;
    simu.p_criteria = 1e-30;   // never met: run exactly the cap
    simu.p_sor_omega = 1.7;
    simu.p_sor_iter_max = 7;
    SorPipeLine_omp(ShareM, Sor, simu, T1, P, Lo, gA);
    dump(out, "sor_p", P.p);
    std::vector<double> ie{(double)simu.iters, simu.error};
    dump(out, "sor_it", ie);
  }
  // 10. CFL diagnostic on u* (get_Cfl, src/RUN_CPU.cpp:274): cfl, U_max[3], U_min[3]
  {
    simu.cfl_max = 0.0;
    get_Cfl(T1, Lo, gA, simu);
    std::vector<double> c{simu.cfl_max,  simu.U_max[0], simu.U_max[1], simu.U_max[2],
                          simu.U_min[0], simu.U_min[1], simu.U_min[2]};
    dump(out, "cfl", c);
  }
  // 11. Plot3D grid and solution files (OutputPlot3D_Xfile, OutputPLOT3D_Qfile of T3, p,
  // eta at time 0), written by the reference into ./mx_out; it also wants ../mx_out
  {
    mkdir("../mx_out", 0755);
    mkdir("mx_out", 0755);
    OutputPlot3D_Xfile(simu, gA);
    simu.currentFile = 0;
    OutputPLOT3D_Qfile(Dfib, simu, t1, T3, Lo, gA);
    copy_bytes("mx_out/P3D.x", out + "/p3d_x.bin");
    copy_bytes("mx_out/P3D00.q", out + "/p3d_q.bin");
  }
  // 12. the same .q file read back by QfileRead (the restart reader, its use commented out
  // at src/RUN_CPU.cpp:88-99): header and the padded p, u, v, w, eta it rebuilds
  {
    auto [nb, mach, alpha, reyn, time, rp, ru, rv, rw, reta] = QfileRead(gA, "mx_out/P3D00.q");
    dump(out, "p3d_read_head", std::vector<double>{(double)nb, mach, alpha, reyn, time});
    dump(out, "p3d_read_p", rp);
    dump(out, "p3d_read_u", ru);
    dump(out, "p3d_read_v", rv);
    dump(out, "p3d_read_w", rw);
    dump(out, "p3d_read_eta", reta);
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) { std::fprintf(stderr, "usage: run|unit ...\n"); return 2; }
  // keep the reference's chatter (printf/cout) off stdout's consumers
  std::string mode = argv[1];
  if (mode == "run") return run_mode(argc, argv);
  if (mode == "unit") return unit_mode(argc, argv);
  std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
