// C++ host shim over the C ABI (cfdgb.h) with the reference's own interface shapes, so a
// driver written against jimmy3769tw/CFD_NSsolver_forHPC_flowPassingCylinder keeps its
// call sites: the same function names, argument meaning (fields by reference, written in
// place) and error behaviour (configuration errors throw std::invalid_argument,
// non-convergence is returned, not thrown: inc/solver/bicgstabRe2.hpp:179).
//
//   reference (file:line)                                   shim
//   runSeqOmp(grid&, clockstruct&, simpulationVariable&,..)  cfdgb::runSeqOmp(Context&, velocity&, pressure&, ...)
//     (src/RUN_CPU.cpp:9)
//   ConvectionDifussion(simu, oldVel, curtVel, Lo, gA)      cfdgb::ConvectionDifussion(ctx, oldVel, curtVel)
//     (inc/source/Convection_Difussion.hpp:174)
//   BC_staggered_main(Lo, vel, pre, gA)                     cfdgb::BC_staggered_main(ctx, vel, pre)
//     (inc/BoundaryCondition/Boundary_Condition.hpp:37)
//   BC_staggered_copy(Lo, oldVel, curtVel, gA)              cfdgb::BC_staggered_copy(ctx, oldVel, curtVel)
//     (inc/BoundaryCondition/updateBC.hpp:6)
//   createBMatrix_omp(T1, Mx, simu, Lo, gA)                 cfdgb::createBMatrix_omp(ctx, T1, Mx, jacobi)
//     (inc/matrix/b_matrix.hpp:35)
//   solver::bicgstabRe2<M>::setTolerance / solve            cfdgb::bicgstabRe2::setTolerance / solve
//     (inc/solver/bicgstabRe2.hpp:38,84)
//   Pressure_transform_X_result(t1, Mx, Lo, gA)             cfdgb::Pressure_transform_X_result(ctx, t1, Mx)
//     (inc/pressure/Transform.hpp:8)
//   update_UandF_omp(Dfib, simu, t1, T1, T3, Lo, gA)         cfdgb::update_UandF_omp(ctx, Dfib, t1, T1, T3)
//     (inc/dfib/updateUandF.hpp:90)
//   DFIB_CylinderZ(Dfib, Lo, gA)                            cfdgb::DFIB_CylinderZ(ctx, Dfib)
//     (inc/dfib/setEta.hpp:136)
//   CD_CL(simu, Lo, Dfib, gA)                               returned by update_UandF_omp / runSeqOmp stats
//     (inc/dfib/virtualForceIntergrator.hpp:92)
//   SmagorinskyModel(ShareM, simu, TX, t1, Lo, gridA)       cfdgb::SmagorinskyModel(ctx, TX)
//     (inc/source/SmagorinskyModel.hpp:30)
//   get_Cfl(T1, Lo, gA, simu)                               cfdgb::get_Cfl(ctx, T1)
//     (inc/analyses/cfl.hpp:3)
//   OutputPLOT3D_Qfile / OutputPlot3D_Xfile                 cfdgb::OutputPLOT3D_Qfile / OutputPlot3D_Xfile
//     (inc/io/Plot3D/qfile.hpp:6, xfileWrite.hpp:6)         (files of the context's current state)
//   QfileRead(gA, filename)                                 cfdgb::QfileRead(ctx, filename)
//     (inc/io/Plot3D/qfileRead.hpp:6)
#pragma once

#include <cstdio>
#include <initializer_list>
#include <stdexcept>
#include <tuple>
#include <string>
#include <utility>
#include <vector>

#include "cfdgb.h"

namespace cfdgb {

struct velocity {  // inc/0_0_PhisicalVaribal.hpp:5
  std::vector<double> u, v, w;
  std::vector<double> Viseff;  // Smagorinsky eddy viscosity per compact cell (:11)
};
struct pressure {  // :75
  std::vector<double> p;
};
struct DfibArray {  // :92 (f is 3 x padded, as there)
  std::vector<double> f, eta;
  double cD = 0.0, cL = 0.0;
};
struct MxClass {  // inc/0_7_PossionEquationStruct.hpp:12
  std::vector<double> matB, X_result;
};

inline void check(int rc) {
  if (rc == CFDGB_OK || rc == CFDGB_ENOCONV) return;
  const std::string msg = std::string("cfdgb: ") + cfdgb_last_error();
  if (rc == CFDGB_EINVAL) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

// Owns one device context: the runtime equivalent of the reference's compile-time
// `grid` constants plus its `simpulationVariable` run parameters.
class Context {
 public:
  explicit Context(const cfdgb_config &cfg) : cfg_(cfg) {
    check(cfdgb_create(&cfg_, &h_));
    check(cfdgb_padded_dims(h_, &nx_, &ny_, &nz_));
  }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  ~Context() { cfdgb_destroy(h_); }
  cfdgb_ctx *handle() const { return h_; }
  const cfdgb_config &config() const { return cfg_; }
  size_t iceltot() const { return (size_t)nx_ * ny_ * nz_; }
  size_t iceltotCal() const { return (size_t)cfg_.nx * cfg_.ny * cfg_.nz; }
  void resize(velocity &v) const { v.u.resize(iceltot()); v.v.resize(iceltot()); v.w.resize(iceltot()); }
  void resize(pressure &p) const { p.p.resize(iceltot()); }

 private:
  cfdgb_config cfg_;
  cfdgb_ctx *h_ = nullptr;
  int nx_ = 0, ny_ = 0, nz_ = 0;
};

inline void need(const Context &c, const std::vector<double> &a, size_t n, const char *what) {
  if (a.size() != n) throw std::invalid_argument(std::string("cfdgb: wrong size for ") + what);
}

inline bool ConvectionDifussion(Context &c, const velocity &oldVel, velocity &curtVel) {
  for (auto *a : {&oldVel.u, &oldVel.v, &oldVel.w}) need(c, *a, c.iceltot(), "oldVel");
  c.resize(curtVel);
  check(cfdgb_op_convection_diffusion(c.handle(), oldVel.u.data(), oldVel.v.data(), oldVel.w.data(),
                                      curtVel.u.data(), curtVel.v.data(), curtVel.w.data()));
  return true;
}

inline bool BC_staggered_main(Context &c, velocity &vel, pressure &pre) {
  for (const std::vector<double> *a : {&vel.u, &vel.v, &vel.w, &pre.p}) need(c, *a, c.iceltot(), "field");
  check(cfdgb_op_bc_main(c.handle(), vel.u.data(), vel.v.data(), vel.w.data(), pre.p.data()));
  return true;
}

inline bool BC_staggered_copy(Context &c, const velocity &oldVel, velocity &curtVel) {
  for (auto *a : {&oldVel.u, &oldVel.v, &oldVel.w}) need(c, *a, c.iceltot(), "oldVel");
  c.resize(curtVel);
  check(cfdgb_op_bc_copy(c.handle(), oldVel.u.data(), oldVel.v.data(), oldVel.w.data(), curtVel.u.data(),
                         curtVel.v.data(), curtVel.w.data()));
  return true;
}

inline void createBMatrix_omp(Context &c, const velocity &T1, MxClass &Mx, bool jacobi = false) {
  for (auto *a : {&T1.u, &T1.v, &T1.w}) need(c, *a, c.iceltot(), "T1");
  Mx.matB.resize(c.iceltotCal());
  check(cfdgb_op_rhs(c.handle(), jacobi ? 1 : 0, T1.u.data(), T1.v.data(), T1.w.data(), Mx.matB.data()));
}

// bicgstabRe2 on the context's operator (SPE, or the Jacobi-scaled CSR rows).
class bicgstabRe2 {
 public:
  explicit bicgstabRe2(Context &c, bool jacobi = false) : c_(c), jacobi_(jacobi) {}
  void setTolerance(double t) { tol_ = t; }
  std::pair<int, double> solve(const std::vector<double> &rhs, std::vector<double> &x) {
    need(c_, rhs, c_.iceltotCal(), "rhs");
    x.resize(c_.iceltotCal(), 0.0);
    int it = 0;
    double rr = 0.0;
    check(cfdgb_op_bicgstab(c_.handle(), jacobi_ ? CFDGB_BICGSTAB_JACOBI : CFDGB_BICGSTAB, tol_, 5000, rhs.data(),
                            x.data(), &it, &rr));
    return {it, rr};
  }

 private:
  Context &c_;
  bool jacobi_;
  double tol_ = 1e-3;  // bicgstabRe2.hpp:51
};

inline void Pressure_transform_X_result(const Context &c, pressure &t1, const MxClass &Mx) {
  need(c, Mx.X_result, c.iceltotCal(), "X_result");
  c.resize(t1);
  const auto &g = c.config();
  const int ny = g.ny + 4, nz = g.nz + 4;
  size_t row = 0;
  for (int i = 2; i < g.nx + 2; ++i)
    for (int j = 2; j < g.ny + 2; ++j)
      for (int k = 2; k < g.nz + 2; ++k) t1.p[((size_t)i * ny + j) * nz + k] = Mx.X_result[row++];
}

inline bool update_UandF_omp(Context &c, DfibArray &Dfib, const pressure &t1, const velocity &oldVel,
                             velocity &curtVel) {
  for (const std::vector<double> *a : std::initializer_list<const std::vector<double> *>{
           &oldVel.u, &oldVel.v, &oldVel.w, &t1.p, &Dfib.eta})
    need(c, *a, c.iceltot(), "field");
  c.resize(curtVel);
  Dfib.f.resize(3 * c.iceltot());
  check(cfdgb_op_update_uf(c.handle(), Dfib.eta.data(), t1.p.data(), oldVel.u.data(), oldVel.v.data(),
                           oldVel.w.data(), curtVel.u.data(), curtVel.v.data(), curtVel.w.data(), Dfib.f.data(),
                           &Dfib.cD, &Dfib.cL));
  return true;
}

inline void DFIB_CylinderZ(Context &c, DfibArray &Dfib) {
  Dfib.eta.resize(c.iceltot());
  check(cfdgb_op_solid_fraction(c.handle(), Dfib.eta.data()));
}

// TX.Viseff = the Smagorinsky eddy viscosity of TX (the context need not have les on).
inline void SmagorinskyModel(Context &c, velocity &TX) {
  for (auto *a : {&TX.u, &TX.v, &TX.w}) need(c, *a, c.iceltot(), "TX");
  TX.Viseff.resize(c.iceltotCal());
  check(cfdgb_op_smagorinsky(c.handle(), TX.u.data(), TX.v.data(), TX.w.data(), TX.Viseff.data()));
}

// get_Cfl's outputs (simu.cfl_max, U_max, U_min) for u* = T1.
struct Cfl {
  double cfl_max, U_max[3], U_min[3];
};
inline Cfl get_Cfl(Context &c, const velocity &T1) {
  for (auto *a : {&T1.u, &T1.v, &T1.w}) need(c, *a, c.iceltot(), "T1");
  double o[7];
  check(cfdgb_op_cfl(c.handle(), T1.u.data(), T1.v.data(), T1.w.data(), o));
  return {o[0], {o[1], o[2], o[3]}, {o[4], o[5], o[6]}};
}

// The reference's Plot3D writers, for the context's current state.
inline void OutputPLOT3D_Qfile(Context &c, double time, const std::string &path) {
  check(cfdgb_write_plot3d(c.handle(), nullptr, path.c_str(), time));
}
inline void OutputPlot3D_Xfile(Context &c, const std::string &path) {
  check(cfdgb_write_plot3d(c.handle(), path.c_str(), nullptr, 0.0));
}

// QfileRead: (Nblock, mach, alpha, reyn, time, p, u, v, w, eta), the fields padded as the
// reference returns them (zero outside the interior).  Throws if the file is not a Plot3D
// solution of the context's grid.
inline auto QfileRead(Context &c, const std::string &path) {
  const auto &g = c.config();
  const size_t n = c.iceltotCal();
  std::FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::invalid_argument("cfdgb: cannot open " + path);
  int ih[4] = {0, 0, 0, 0};
  float fh[4] = {0, 0, 0, 0};
  std::vector<float> q(5 * n);
  const bool ok = std::fread(ih, sizeof(int), 4, f) == 4 && std::fread(fh, sizeof(float), 4, f) == 4 &&
                  ih[1] == g.nx && ih[2] == g.ny && ih[3] == g.nz && std::fread(q.data(), sizeof(float), 5 * n, f) == 5 * n;
  std::fclose(f);
  if (!ok) throw std::invalid_argument("cfdgb: " + path + " is not a Plot3D solution of this grid");
  std::vector<double> p(c.iceltot()), u(c.iceltot()), v(c.iceltot()), w(c.iceltot()), eta(c.iceltot());
  check(cfdgb_op_plot3d_read(c.handle(), q.data(), p.data(), u.data(), v.data(), w.data(), eta.data()));
  return std::make_tuple(ih[0], fh[0], fh[1], fh[2], fh[3], std::move(p), std::move(u), std::move(v), std::move(w),
                         std::move(eta));
}

// The time loop of runSeqOmp (src/RUN_CPU.cpp:257-436) on the device: T0/t1 in as the
// initial state (before the first ghost fill), out as the state after `steps` steps.
inline bool runSeqOmp(Context &c, velocity &T0, pressure &t1, int steps, std::vector<cfdgb_step_stats> *stats = nullptr) {
  for (auto *a : {&T0.u, &T0.v, &T0.w}) need(c, *a, c.iceltot(), "T0");
  c.resize(t1);
  check(cfdgb_init_fields(c.handle(), T0.u.data(), T0.v.data(), T0.w.data(), t1.p.data()));
  std::vector<cfdgb_step_stats> st(steps > 0 ? steps : 1);
  const int rc = cfdgb_step(c.handle(), steps, st.data());
  check(rc);
  check(cfdgb_get_fields(c.handle(), T0.u.data(), T0.v.data(), T0.w.data(), t1.p.data()));
  if (stats) stats->assign(st.begin(), st.begin() + steps);
  return rc == CFDGB_OK;
}

}  // namespace cfdgb
