// cfdgb_poisson_solve_static: the BiCGSTAB pressure solve for callers that cannot
// allocate device memory.
//
// Who needs it: callers inside a host framework that owns all device memory through its
// own pool and forbids raw allocations, and real-time or long-running services that must
// not allocate after start-up.  Such a caller passes its own device buffers for the
// right-hand side and the solution; every work vector, block partial and solver scalar
// lives in one file-scope static device array, so the call makes no cudaMalloc/cudaFree
// and no allocating library call.
//
// Limits and sharing:
//   - at most kStaticMaxCells unknowns (2^18, e.g. 64^3); larger grids are rejected with
//     CFDGB_EINVAL;
//   - the array is reserved on every GPU that loads the library, until the process exits:
//     8 work vectors of 2 MiB, 256 KiB of block partials and 256 B of solver scalars,
//     17,039,616 bytes (about 17.0 MB, kScratchBytes);
//   - all calls share it and it keeps the last call's contents: each call clears the
//     solver scalars and reduction tickets it relies on before it starts, but two calls
//     whose work overlaps on the GPU (different streams or threads at the same time) race
//     on it and must not be issued;
//   - the call polls the solver's convergence from the host every 8 iterations (a
//     device-to-host copy and a wait on `stream`), so `stream` must not be capturing into a
//     CUDA graph: a capturing stream is rejected with CFDGB_EINVAL before any work;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, cached).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "cfdgb_internal.cuh"
#include "kernels.h"

namespace {

using namespace cfdgb;

constexpr long long kStaticMaxCells = 1LL << 18;  // 262,144 unknowns, e.g. 64 x 64 x 64
constexpr int kStaticMaxBlocks = 4096;            // reduction partials per vector
constexpr int kStaticVectors = 8;                 // x-history x2, r0 r1 p1 s ap as
constexpr size_t kVecBytes = kStaticMaxCells * sizeof(double);
constexpr size_t kPartBytes = 8 * kStaticMaxBlocks * sizeof(double);
constexpr size_t kScalBytes = (sizeof(SolverScal) + 255) / 256 * 256;
constexpr size_t kScratchBytes = kStaticVectors * kVecBytes + kPartBytes + kScalBytes;
static_assert(kScalBytes == 256 && kScratchBytes == 17039616, "the documented size of the static array");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {nullptr};

// Device address of g_scratch on the current device (looked up once per device).
cudaError_t scratch_address(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = static_cast<unsigned char *>(p);
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

// The 27 operator row classes of a uniform grid, with the reference's entry values
// (SPE_sparseMatrix.hpp:42-126; CSR rows scaled by jp, structureGrid.hpp:557-645).
void uniform_stencils(int nx, int ny, int nz, double dx, double dy, double dz, Stencil<double> &spe,
                      Stencil<double> &jac) {
  const double cx = 1.0 / dx / dx, cy = 1.0 / dy / dy, cz = 1.0 / dz / dz;
  auto rep = [](int cls, int n) { return cls == 0 ? 0 : (cls == 2 ? n - 1 : 1); };
  for (int bx = 0; bx < 3; ++bx)
    for (int by = 0; by < 3; ++by)
      for (int bz = 0; bz < 3; ++bz) {
        const int cls = bx * 9 + by * 3 + bz;
        const int i = rep(bx, nx), j = rep(by, ny), k = rep(bz, nz);
        double ijk = cx + cy + cz + cx + cy + cz;
        if (i == 0) ijk -= cx;
        if (i == nx - 1) ijk -= cx;
        if (j == 0) ijk -= cy;
        if (j == ny - 1) ijk -= cy;
        if (k == 0) ijk -= cz;
        if (k == nz - 1) ijk -= cz;
        double *s = spe.c[cls];
        s[0] = i != 0 ? -cx : 0.0;
        s[1] = j != 0 ? -cy : 0.0;
        s[2] = k != 0 ? -cz : 0.0;
        s[3] = ijk;
        s[4] = k != nz - 1 ? -cz : 0.0;
        s[5] = j != ny - 1 ? -cy : 0.0;
        s[6] = i != nx - 1 ? -cx : 0.0;
        s[7] = 1.0 / ijk;
        spe.dg[cls] = jac.dg[cls] = ijk;
        double aa = 0.0, bb = 0.0, cc = 0.0;
        if (i == 0) aa = -cx;
        if (i == nx - 1) aa = -cx;
        if (j == 0) bb = -cy;
        if (j == ny - 1) bb = -cy;
        if (k == 0) cc = -cz;
        if (k == nz - 1) cc = -cz;
        const double dj = cx + cy + cz + cx + cy + cz + aa + bb + cc;
        const double jp = 1.0 / dj;
        double *q = jac.c[cls];
        q[0] = i != 0 ? -cx * jp : 0.0;
        q[1] = j != 0 ? -cy * jp : 0.0;
        q[2] = k != 0 ? -cz * jp : 0.0;
        q[3] = dj * jp;
        q[4] = k != nz - 1 ? -cz * jp : 0.0;
        q[5] = j != ny - 1 ? -cy * jp : 0.0;
        q[6] = i != nx - 1 ? -cx * jp : 0.0;
        q[7] = jp;
      }
}

}  // namespace

extern "C" int cfdgb_poisson_solve_static(int nx, int ny, int nz, double dx, double dy, double dz, int solver,
                                          double tol, int maxit, const double *d_rhs, double *d_x, void *stream,
                                          int *iters, double *relres) {
  if (nx < 3 || ny < 3 || nz < 3 || !(dx > 0 && dy > 0 && dz > 0) || !d_rhs || !d_x || !(tol > 0) || maxit < 1 ||
      (solver != CFDGB_BICGSTAB && solver != CFDGB_BICGSTAB_JACOBI))
    return CFDGB_EINVAL;
  const long long n = (long long)nx * ny * nz;
  if (n > kStaticMaxCells) return CFDGB_EINVAL;  // the static work array holds 2^18 unknowns
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the convergence polls wait on the stream: a stream that is being captured cannot run them
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return CFDGB_ECUDA;
  if (cap != cudaStreamCaptureStatusNone) return CFDGB_EINVAL;
  unsigned char *base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return CFDGB_ECUDA;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return CFDGB_ECUDA;
  // geometry: the launch shape of the context driver's solver kernels (k_block_width and
  // the same grid), so the reductions sum in the same order
  Geo g{};
  g.nxc = nx; g.nyc = ny; g.nzc = nz;
  g.nx = nx + 4; g.ny = ny + 4; g.nz = nz + 4;
  g.sx = (long long)g.ny * g.nz; g.sy = g.nz;
  g.ncell = n;
  g.lbx = k_block_width(nz);
  g.lby = kBlock / g.lbx;
  g.lgx = (nz + g.lbx - 1) / g.lbx;
  g.lgy = (ny + g.lby - 1) / g.lby;
  g.lgz = std::max(1, std::min(nx, nsm * 8 / std::max(1, g.lgx * g.lgy)));
  if ((long long)g.lgx * g.lgy * g.lgz > kStaticMaxBlocks) return CFDGB_EINVAL;
  Stencil<double> spe, jac;
  uniform_stencils(nx, ny, nz, dx, dy, dz, spe, jac);
  const Stencil<double> &st = solver == CFDGB_BICGSTAB_JACOBI ? jac : spe;
  // carve the static array
  double *vec[kStaticVectors];
  for (int q = 0; q < kStaticVectors; ++q) vec[q] = reinterpret_cast<double *>(base + q * kVecBytes);
  double *part = reinterpret_cast<double *>(base + kStaticVectors * kVecBytes);
  SolverScal *sc = reinterpret_cast<SolverScal *>(base + kStaticVectors * kVecBytes + kPartBytes);
  KrylovVecs<double> v{};
  v.x = d_x;
  v.r0 = vec[2]; v.r1 = vec[3]; v.p1 = vec[4]; v.s = vec[5]; v.ap = vec[6]; v.as = vec[7];
  double *px1 = vec[0], *px2 = vec[1];
  // clear what must start at zero: solver scalars and tickets; history = the warm start
  SolverScal init{};
  init.tol = tol;
  init.restart_thr = tol * 1e-7;  // bicgstabRe2.hpp:53
  init.maxit = maxit;
  if (cudaMemcpyAsync(sc, &init, sizeof(SolverScal), cudaMemcpyHostToDevice, s) != cudaSuccess) return CFDGB_ECUDA;
  if (cudaMemsetAsync(px1, 0, n * sizeof(double), s) != cudaSuccess) return CFDGB_ECUDA;
  launch_bicg_setup64(s, 0, g, st, v, d_rhs, px1, px2, part, sc);
  SolverScal h{};
  bool done = false;
  for (long long q = 0; q < (long long)maxit / 8 + 3 && !done; ++q) {
    for (int m = 0; m < 8; ++m)
      for (int k = 0; k < 5; ++k) launch_bicg64_part(s, k, g, st, v, part, sc);
    if (cudaMemcpyAsync(&h, sc, sizeof(SolverScal), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return CFDGB_ECUDA;
    done = h.done != 0;
  }
  if (!done) return CFDGB_ECUDA;
  if (h.status == CFDGB_ENOCONV) launch_bicg_nan_reset(s, 0, g, d_x, px1, px2, part, sc);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return CFDGB_ECUDA;
  if (iters) *iters = h.iter;
  if (relres) *relres = h.relres;
  return h.status;
}
