// Geometric multigrid V-cycle in FP32: the preconditioner of the FP32 BiCGSTAB sweep
// inside the FP64 refinement (the reference has no multigrid; its Poisson operator on a
// uniform grid is the 7-point Neumann Laplacian of SPE_sparseMatrix.hpp:42-85, which every
// level here rediscretises at its own spacing).
//
// Cell-centred hierarchy: a coarse cell is the union of 2 cells along each halved axis.
// Restriction averages the fine residual over a coarse cell's children; prolongation is
// the cell-centred trilinear interpolation (weights 3/4 and 1/4 per halved axis, the
// parent's value standing in for a neighbour beyond a Neumann wall, the wrapped cell
// across a periodic z end); the smoother is
// red-black Gauss-Seidel, one sweep before and one after the coarse correction; the
// coarsest level (at most kMgSharedCells cells) is solved by red-black sweeps in the
// shared memory of one block.  The V-cycle is a fixed linear map, as a right
// preconditioner of BiCGSTAB requires.  Every kernel is pointwise or a stencil over one
// level and reads sc->done first, so a captured chunk of iterations idles once the sweep
// has stopped.
#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

#include "cfdgb_internal.cuh"
#include "kernels.h"

namespace cfdgb {

// Programmatic dependent launch (griddepcontrol): a V-cycle kernel is launched so that it
// may be scheduled while its predecessor finishes.  It waits for the predecessor's
// completion and memory (pdl_wait) before reading anything, and lets its successor be
// scheduled once its own results are stored (pdl_trigger); a block that returns early
// counts as triggered.  The small levels' kernels are launch-latency-bound.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

#define FOR_LEVEL(L)                                   \
  const int k = blockIdx.x * blockDim.x + threadIdx.x; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y; \
  const bool on_ = (k < (L).nz) && (j < (L).ny);       \
  for (int i = blockIdx.z; on_ && i < (L).nx; i += gridDim.z)

template <typename T>
__device__ __forceinline__ long long lrow(const MgLevelT<T> &L, int i, int j, int k) {
  return ((long long)i * L.ny + j) * L.nz + k;
}

// Rounded operations the compiler does not contract: the quad smoother, the pair transfers
// and the marching kernels form each value by the same explicit sequence, so that they give
// identical results.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
// wx a + wy e + wz f (the weighted neighbour sums of lnb's three axes)
template <typename T>
__device__ __forceinline__ T wsum(const MgLevelT<T> &L, T a, T e, T f) {
  return fma_rn(L.wz, f, fma_rn(L.wy, e, mul_rn(L.wx, a)));
}
// one child's residual b - d x + (neighbour sum), b already scaled
template <typename T>
__device__ __forceinline__ T resid(T bb, T d, T x, T nb) { return add_rn(fma_rn(-d, x, bb), nb); }

// z neighbours of a cell: those that exist (Neumann), or both across the wrap (periodic z,
// none on a level one cell thick, whose wrapped neighbours are the cell itself)
template <typename T>
__device__ __forceinline__ int zcount(const MgLevelT<T> &L, int k) {
  return L.pz ? (L.nz > 1 ? 2 : 0) : (k > 0) + (k < L.nz - 1);
}

// diagonal of a row: the weights of the neighbours that exist
template <typename T>
__device__ __forceinline__ T ldiag(const MgLevelT<T> &L, int i, int j, int k) {
  return L.wx * (T)((i > 0) + (i < L.nx - 1)) + L.wy * (T)((j > 0) + (j < L.ny - 1)) + L.wz * (T)zcount(L, k);
}

// 1/diag of the row (ldiag's reciprocal, from the level's table)
template <typename T>
__device__ __forceinline__ T linv(const MgLevelT<T> &L, int i, int j, int k) {
  return L.idg[9 * ((i > 0) + (i < L.nx - 1)) + 3 * ((j > 0) + (j < L.ny - 1)) + zcount(L, k)];
}

// weighted sum of the neighbours' values (minus the off-diagonal part of the row)
template <typename T>
__device__ __forceinline__ T lnb(const MgLevelT<T> &L, const T *x, int i, int j, int k, long long r) {
  const long long sx = (long long)L.ny * L.nz;
  T a = T(0), b = T(0), c = T(0);
  if (i > 0) a += x[r - sx];
  if (i < L.nx - 1) a += x[r + sx];
  if (j > 0) b += x[r - L.nz];
  if (j < L.ny - 1) b += x[r + L.nz];
  if (L.pz) {
    if (L.nz > 1) {
      c += x[k > 0 ? r - 1 : r + L.nz - 1];
      c += x[k < L.nz - 1 ? r + 1 : r + 1 - L.nz];
    }
  } else {
    if (k > 0) c += x[r - 1];
    if (k < L.nz - 1) c += x[r + 1];
  }
  return L.wx * a + L.wy * b + L.wz * c;
}

// One colour of a red-black Gauss-Seidel sweep (colour = (i + j + k) & 1).  zero: x starts
// at zero, so the cells of this colour take b / diag and the others are set to zero.
// bscale: b holds Jacobi-scaled rows (b / diag), which are unscaled first.
template <typename T>
__global__ void __launch_bounds__(kBlock) k_mg_smooth(MgLevelT<T> L, int colour, int zero, int bscale,
                                                      const T *__restrict__ b, T *x, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  FOR_LEVEL(L) {
    const long long r = lrow(L, i, j, k);
    if (((i + j + k) & 1) != colour) {
      if (zero) x[r] = T(0);
      continue;
    }
    T bb = b[r];
    if (bscale) bb *= ldiag(L, i, j, k);
    const T num = zero ? bb : bb + lnb(L, x, i, j, k, r);
    x[r] = num * linv(L, i, j, k);
  }
}

// The same colour pass on quads of four consecutive k cells (nz % 4 == 0): a thread updates
// the two cells of the colour in its quad and stores the whole quad, the other two
// unchanged (no thread writes them in this pass, so rewriting them races with nothing).
// 3-D launch (quads along x, rows along y, planes strided over z: no index division), the
// row's neighbour counts along x and y taken once per quad.  Neighbour sums in the order
// of lnb, diagonals as ldiag / linv form them.
__global__ void __launch_bounds__(kBlock) k_mg_smooth4(MgLevel L, int colour, int zero, int bscale,
                                                       const float *__restrict__ b, float *x, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  const int kq = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (kq >= (L.nz >> 2) || j >= L.ny) return;  // no barrier below
  const long long sx = (long long)L.ny * L.nz;
  const int k0 = 4 * kq;
  const bool jm = j > 0, jp = j < L.ny - 1;
  const int cy = (int)jm + (int)jp;
  int cz[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) cz[c] = zcount(L, k0 + c);
  for (int i = blockIdx.z; i < L.nx; i += gridDim.z) {
    const long long r = lrow(L, i, j, k0);
    const bool im = i > 0, ip = i < L.nx - 1;
    const int cx = (int)im + (int)ip, cxy = 9 * cx + 3 * cy;
    const float dxy = L.wx * (float)cx + L.wy * (float)cy;  // ldiag's first two terms, in its order
    const int t0 = (i + j + k0 + colour) & 1;  // first cell of the colour in the quad
    const float4 bq = *reinterpret_cast<const float4 *>(b + r);
    const float bv[4] = {bq.x, bq.y, bq.z, bq.w};
    float o[4];
    if (zero) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if ((c & 1) != t0) {
          o[c] = 0.f;
          continue;
        }
        const float bb = bscale ? mul_rn(bv[c], dxy + L.wz * (float)cz[c]) : bv[c];
        o[c] = mul_rn(bb, L.idg[cxy + cz[c]]);
      }
    } else {
      const float4 xq = *reinterpret_cast<const float4 *>(x + r);
      const float xv[4] = {xq.x, xq.y, xq.z, xq.w};
      const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 xm = im ? *reinterpret_cast<const float4 *>(x + r - sx) : z4;
      const float4 xp = ip ? *reinterpret_cast<const float4 *>(x + r + sx) : z4;
      const float4 ym = jm ? *reinterpret_cast<const float4 *>(x + r - L.nz) : z4;
      const float4 yp = jp ? *reinterpret_cast<const float4 *>(x + r + L.nz) : z4;
      const float xmv[4] = {xm.x, xm.y, xm.z, xm.w}, xpv[4] = {xp.x, xp.y, xp.z, xp.w};
      const float ymv[4] = {ym.x, ym.y, ym.z, ym.w}, ypv[4] = {yp.x, yp.y, yp.z, yp.w};
      // the cells left and right of the quad (periodic z: across the wrap)
      const float kl = k0 > 0 ? x[r - 1] : (L.pz ? x[r + L.nz - 1] : 0.f);
      const float kr = k0 + 4 < L.nz ? x[r + 4] : (L.pz ? x[r + 4 - L.nz] : 0.f);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        o[c] = xv[c];
        if ((c & 1) != t0) continue;
        const int k = k0 + c;
        float a = 0.f, e = 0.f, f = 0.f;
        if (im) a += xmv[c];
        if (ip) a += xpv[c];
        if (jm) e += ymv[c];
        if (jp) e += ypv[c];
        if (k > 0 || L.pz) f += c == 0 ? kl : xv[c - 1];
        if (k < L.nz - 1 || L.pz) f += c == 3 ? kr : xv[c + 1];
        const float bb = bscale ? mul_rn(bv[c], dxy + L.wz * (float)cz[c]) : bv[c];
        o[c] = mul_rn(add_rn(bb, wsum(L, a, e, f)), L.idg[cxy + cz[c]]);
      }
    }
    *reinterpret_cast<float4 *>(x + r) = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// bc = average over each coarse cell's children of the fine residual b - A x
template <typename T>
__global__ void __launch_bounds__(kBlock) k_mg_restrict(MgLevelT<T> F, MgLevelT<T> Cl, int bscale,
                                                        const T *__restrict__ bf, const T *__restrict__ xf,
                                                        T *__restrict__ bc, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  const T inv = T(1) / (T)(F.fx * F.fy * F.fz);
  FOR_LEVEL(Cl) {
    T sum = T(0);
    for (int a = 0; a < F.fx; ++a)
      for (int e = 0; e < F.fy; ++e)
        for (int c = 0; c < F.fz; ++c) {
          const int fi = i * F.fx + a, fj = j * F.fy + e, fk = k * F.fz + c;
          const long long r = lrow(F, fi, fj, fk);
          const T d = ldiag(F, fi, fj, fk);
          T bb = bf[r];
          if (bscale) bb *= d;
          sum += bb - d * xf[r] + lnb(F, xf, fi, fj, fk, r);
        }
    bc[lrow(Cl, i, j, k)] = sum * inv;
  }
}

// the two coarse cells a fine cell interpolates from along one axis, and their weights;
// per: the axis is periodic
template <typename T>
__device__ __forceinline__ void axis_taps(int i, int f, int n, int (&c)[2], T (&w)[2], bool per = false) {
  if (f == 1) {
    c[0] = c[1] = i;
    w[0] = T(1);
    w[1] = T(0);
    return;
  }
  const int p = i >> 1;
  int q = p + ((i & 1) ? 1 : -1);
  // beyond a wall: the parent's value (zero normal gradient); periodic: the wrapped cell
  if (q < 0 || q >= n) q = per ? (q + n) % n : p;
  c[0] = p;
  c[1] = q;
  w[0] = T(0.75);
  w[1] = T(0.25);
}

// (P xc) at fine cell (i, j, k): cell-centred trilinear interpolation
template <typename T>
__device__ __forceinline__ T prolong_at(const MgLevelT<T> &F, const MgLevelT<T> &Cl, const T *__restrict__ xc, int i,
                                        int j, int k) {
  int ci[2], cj[2], ck[2];
  T wi[2], wj[2], wk[2];
  axis_taps(i, F.fx, Cl.nx, ci, wi);
  axis_taps(j, F.fy, Cl.ny, cj, wj);
  axis_taps(k, F.fz, Cl.nz, ck, wk, F.pz != 0);
  T v = T(0);
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const T w = wi[a] * wj[e] * wk[c];
        if (w != T(0)) v += w * xc[lrow(Cl, ci[a], cj[e], ck[c])];
      }
  return v;
}

// xf += P xc
template <typename T>
__global__ void __launch_bounds__(kBlock) k_mg_prolong(MgLevelT<T> F, MgLevelT<T> Cl, const T *__restrict__ xc,
                                                       T *__restrict__ xf, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  FOR_LEVEL(F) {
    xf[lrow(F, i, j, k)] += prolong_at(F, Cl, xc, i, j, k);
  }
}

// ---- transfers when every axis halves (fx = fy = fz = 2): one thread per coarse cell,
// its eight children loaded once (pairs along k as one vector load) and their neighbours
// shared, the arithmetic and summation order of k_mg_restrict / k_mg_prolong ----
template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };
template <typename T>
__device__ __forceinline__ void ld2(const T *p, T &a, T &b) {
  const typename Vec2<T>::type v = *reinterpret_cast<const typename Vec2<T>::type *>(p);
  a = v.x;
  b = v.y;
}
template <typename T>
__device__ __forceinline__ void st2(T *p, T a, T b) {
  typename Vec2<T>::type v;
  v.x = a;
  v.y = b;
  *reinterpret_cast<typename Vec2<T>::type *>(p) = v;
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_mg_restrict8(MgLevelT<T> F, MgLevelT<T> Cl, int bscale,
                                                         const T *__restrict__ bf, const T *__restrict__ xf,
                                                         T *__restrict__ bc, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  const T inv = T(1) / T(8);
  const long long sx = (long long)F.ny * F.nz, sy = F.nz;
  FOR_LEVEL(Cl) {
    const int i0 = 2 * i, j0 = 2 * j, k0 = 2 * k;
    const long long r0 = lrow(F, i0, j0, k0);
    T xv[2][2][2], bv[2][2][2], xim[2][2], xip[2][2], xjm[2][2], xjp[2][2], xkm[2][2], xkp[2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const long long r = r0 + a * sx + e * sy;
        ld2(xf + r, xv[a][e][0], xv[a][e][1]);
        ld2(bf + r, bv[a][e][0], bv[a][e][1]);
        xkm[a][e] = k0 > 0 ? xf[r - 1] : (F.pz ? xf[r + F.nz - 1] : T(0));
        xkp[a][e] = k0 + 2 < F.nz ? xf[r + 2] : (F.pz ? xf[r + 2 - F.nz] : T(0));
      }
#pragma unroll
    for (int e = 0; e < 2; ++e) {  // x neighbours of the i0 and i0+1 planes
      if (i0 > 0) ld2(xf + r0 - sx + e * sy, xim[e][0], xim[e][1]);
      else xim[e][0] = xim[e][1] = T(0);
      if (i0 + 2 < F.nx) ld2(xf + r0 + 2 * sx + e * sy, xip[e][0], xip[e][1]);
      else xip[e][0] = xip[e][1] = T(0);
    }
#pragma unroll
    for (int a = 0; a < 2; ++a) {  // y neighbours
      if (j0 > 0) ld2(xf + r0 + a * sx - sy, xjm[a][0], xjm[a][1]);
      else xjm[a][0] = xjm[a][1] = T(0);
      if (j0 + 2 < F.ny) ld2(xf + r0 + a * sx + 2 * sy, xjp[a][0], xjp[a][1]);
      else xjp[a][0] = xjp[a][1] = T(0);
    }
    T sum = T(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int fi = i0 + a, fj = j0 + e, fk = k0 + c;
          T ax = T(0), ay = T(0), az = T(0);  // lnb's terms in its order
          if (fi > 0) ax += a ? xv[0][e][c] : xim[e][c];
          if (fi < F.nx - 1) ax += a ? xip[e][c] : xv[1][e][c];
          if (fj > 0) ay += e ? xv[a][0][c] : xjm[a][c];
          if (fj < F.ny - 1) ay += e ? xjp[a][c] : xv[a][1][c];
          if (fk > 0 || F.pz) az += c ? xv[a][e][0] : xkm[a][e];
          if (fk < F.nz - 1 || F.pz) az += c ? xkp[a][e] : xv[a][e][1];
          const T d = ldiag(F, fi, fj, fk);
          const T bb = bscale ? mul_rn(bv[a][e][c], d) : bv[a][e][c];
          sum = add_rn(sum, resid(bb, d, xv[a][e][c], wsum(F, ax, ay, az)));
        }
    bc[lrow(Cl, i, j, k)] = mul_rn(sum, inv);
  }
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_mg_prolong8(MgLevelT<T> F, MgLevelT<T> Cl, const T *__restrict__ xc,
                                                        T *__restrict__ xf, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  const long long sx = (long long)F.ny * F.nz, sy = F.nz;
  FOR_LEVEL(Cl) {
    // the 3 x 3 x 3 coarse neighbourhood; beyond a wall the parent's value (axis_taps)
    T cv[3][3][3];
    const int ci[3] = {i > 0 ? i - 1 : i, i, i < Cl.nx - 1 ? i + 1 : i};
    const int cj[3] = {j > 0 ? j - 1 : j, j, j < Cl.ny - 1 ? j + 1 : j};
    const int ck[3] = {k > 0 ? k - 1 : (Cl.pz ? Cl.nz - 1 : k), k, k < Cl.nz - 1 ? k + 1 : (Cl.pz ? 0 : k)};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int e = 0; e < 3; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) cv[a][e][c] = xc[lrow(Cl, ci[a], cj[e], ck[c])];
    const T w0 = T(0.75), w1 = T(0.25);
    const long long r0 = lrow(F, 2 * i, 2 * j, 2 * k);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        T out[2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          // taps: the parent (index 1) and the neighbour on the child's side (0 or 2), in
          // k_mg_prolong's order (parent first on every axis) and weights
          const int ti[2] = {1, a ? 2 : 0}, tj[2] = {1, e ? 2 : 0}, tk[2] = {1, c ? 2 : 0};
          const T wa[2] = {w0, w1};
          T v = T(0);
#pragma unroll
          for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int q = 0; q < 2; ++q)
#pragma unroll
              for (int t = 0; t < 2; ++t) v = fma_rn(wa[p] * wa[q] * wa[t], cv[ti[p]][tj[q]][tk[t]], v);
          out[c] = v;
        }
        T *dst = xf + r0 + a * sx + e * sy;
        T x0, x1;
        ld2(dst, x0, x1);
        st2(dst, add_rn(x0, out[0]), add_rn(x1, out[1]));
      }
  }
}

// ---- a level whose every axis halves, FP32 quads (nz / 4 a power of two up to 16): its
// V-cycle work in two marching kernels instead of six per-pass launches.  A block of
// nz / 4 x (mty + 4) threads owns a band of mty rows and two halo rows on each side (a
// thread: one quad of one row) and marches along x over a segment of msx planes and two halo
// planes on each side.  A thread keeps its planes in registers (rings of three, rotated by
// unrolling); each stage's plane passes through shared memory for the y neighbours (three
// buffers per stage, so one barrier a plane; rows outside the level hold zeros there) and
// the z neighbours across quads by shuffles.  The arithmetic runs on cell pairs (FP32x2).
//   k_mg_down4: the pre-smoothing from zero (colour 0: b / diag; colour 1 from those), the
//     residual and its restriction to the next level's b.  The level's x is not stored: the
//     only part of it read later, colour 0's, is b / diag again.
//   k_mg_up4: colour 0 = b / diag + P xc, then the colour-1 and colour-0 passes of the
//     post-smoothing; x stored.
// Neighbours beyond a wall enter as zeros (the registers of planes and the shared rows
// outside the level hold zeros).  Each value is otherwise formed by the rounded sequence of
// k_mg_smooth4, k_mg_restrict8 or k_mg_prolong8 (the pair operations round each component
// as the scalar ones do), so a V-cycle gives the per-pass kernels' result (equal as
// numbers: a sum of two zeros may differ in sign).
constexpr int kMgMarchThreads = 320;

__device__ __forceinline__ float2 pr(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
// wsum of two cells
__device__ __forceinline__ float2 wsum2(const MgLevel &L, float2 a, float2 e, float2 f) {
  return __ffma2_rn(bc2(L.wz), f, __ffma2_rn(bc2(L.wy), e, __fmul2_rn(bc2(L.wx), a)));
}

// a thread's row and quad, and what does not change along the march
struct MarchRow {
  unsigned mask;      // the lanes of this warp that exist
  int left, right;    // lanes of the quads before and after this one in its row (wrapping)
  int q, tj, j, k0;
  bool jin, jm, jp;   // the row exists; its neighbours along y exist
  bool zl, zr;        // the quad has a z neighbour before / after it (or across the wrap)
  float wycy;         // wy cy (exact: cy in 0..2)
  float2 wz01, wz23;  // wz cz of the quad's cells (exact)
  int cy3, cz0, cz3;  // 3 cy; cz of the end cells (the middle ones have cz = 2)
  // 1/diag of the quad's cells on a plane with 9 cx = c9
  __device__ __forceinline__ float2 idg01(const MgLevel &L, int c9) const {
    return pr(L.idg[c9 + cy3 + cz0], L.idg[c9 + cy3 + 2]);
  }
  __device__ __forceinline__ float2 idg23(const MgLevel &L, int c9) const {
    return pr(L.idg[c9 + cy3 + 2], L.idg[c9 + cy3 + cz3]);
  }
};

template <int NQ>
__device__ __forceinline__ MarchRow march_row(const MgLevel &L) {
  MarchRow R;
  const int w0 = threadIdx.x & ~31, n = min(32, (int)blockDim.x - w0);
  R.mask = n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
  R.q = threadIdx.x % NQ;
  R.tj = threadIdx.x / NQ;
  R.k0 = 4 * R.q;
  const int row0 = (threadIdx.x & 31) - R.q;  // a row's NQ lanes lie in one warp (NQ divides 32)
  R.left = row0 + ((R.q - 1) & (NQ - 1));
  R.right = row0 + ((R.q + 1) & (NQ - 1));
  R.j = blockIdx.y * L.mty - 2 + R.tj;
  R.jin = R.j >= 0 && R.j < L.ny;
  R.jm = R.j > 0;
  R.jp = R.j < L.ny - 1;
  R.zl = R.q > 0 || L.pz;
  R.zr = R.q < NQ - 1 || L.pz;
  const int cy = (int)R.jm + (int)R.jp;
  R.wycy = L.wy * (float)cy;
  R.cy3 = 3 * cy;
  R.cz0 = zcount(L, R.k0);
  R.cz3 = zcount(L, R.k0 + 3);
  R.wz01 = pr(L.wz * (float)R.cz0, 2.f * L.wz);
  R.wz23 = pr(2.f * L.wz, L.wz * (float)R.cz3);
  return R;
}

__device__ __forceinline__ void unq(const float4 v, float (&o)[4]) {
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
}
__device__ __forceinline__ float4 mkq(const float (&o)[4]) { return make_float4(o[0], o[1], o[2], o[3]); }

// wx cx + wy cy of plane i (the diagonal less its z part) and 9 cx
__device__ __forceinline__ float march_dxy(const MgLevel &L, const MarchRow &R, int i, int &c9) {
  const int cx = (int)(i > 0) + (int)(i < L.nx - 1);
  c9 = 9 * cx;
  return fma_rn(L.wx, (float)cx, R.wycy);
}

// the z neighbours of a quad's end cells from the neighbouring lanes (every lane calls it)
__device__ __forceinline__ void march_kz(const MarchRow &R, const float (&v)[4], float &kl, float &kr) {
  const float l = __shfl_sync(R.mask, v[3], R.left), r = __shfl_sync(R.mask, v[0], R.right);
  kl = R.zl ? l : 0.f;
  kr = R.zr ? r : 0.f;
}

// b of a quad's cell pairs, times the diagonal for Jacobi-scaled rows (BS).  The product
// stays scalar: its FP32x2 form gave results different from the per-pass kernels on the
// Jacobi-scaled runs (measured; the pair operations alone round as the scalar ones do, and
// the cause was not found), the scalar form gives identical ones.
template <bool BS>
__device__ __forceinline__ void march_bb(const MarchRow &R, float dxy, const float (&bv)[4], float2 &b01,
                                         float2 &b23) {
  if (BS) {
    b01 = pr(mul_rn(bv[0], dxy + R.wz01.x), mul_rn(bv[1], dxy + R.wz01.y));
    b23 = pr(mul_rn(bv[2], dxy + R.wz23.x), mul_rn(bv[3], dxy + R.wz23.y));
  } else {
    b01 = pr(bv[0], bv[1]);
    b23 = pr(bv[2], bv[3]);
  }
}

// colour 0 of a quad after the pre-smoothing from zero (k_mg_smooth4's zero pass): b / diag
// on colour 0, zero on colour 1
template <bool BS>
__device__ __forceinline__ void march_zero(const MgLevel &L, const MarchRow &R, float dxy, int c9, int t0,
                                           const float (&bv)[4], float (&o)[4]) {
  float2 b01, b23;
  march_bb<BS>(R, dxy, bv, b01, b23);
  const float2 v01 = __fmul2_rn(b01, R.idg01(L, c9)), v23 = __fmul2_rn(b23, R.idg23(L, c9));
  o[0] = t0 ? 0.f : v01.x;
  o[1] = t0 ? v01.y : 0.f;
  o[2] = t0 ? 0.f : v23.x;
  o[3] = t0 ? v23.y : 0.f;
}

// One colour pass of k_mg_smooth4 on a quad (its non-zero form): the cells of colour t0's
// parity (t0: the first such cell) from the neighbours' values, the others kept.  xm, xp:
// the quad on the planes before and after; ym, yp: rows j -1, j + 1; kl, kr: the cells
// beyond the quad's ends.
template <bool BS>
__device__ __forceinline__ void march_pass(const MgLevel &L, const MarchRow &R, float dxy, int c9, int t0,
                                           const float (&bv)[4], const float (&xv)[4], const float (&xm)[4],
                                           const float (&xp)[4], const float4 ym, const float4 yp, float kl, float kr,
                                           float (&o)[4]) {
  float2 b01, b23;
  march_bb<BS>(R, dxy, bv, b01, b23);
  const float2 s01 = wsum2(L, __fadd2_rn(pr(xm[0], xm[1]), pr(xp[0], xp[1])), __fadd2_rn(pr(ym.x, ym.y), pr(yp.x, yp.y)),
                           __fadd2_rn(pr(kl, xv[0]), pr(xv[1], xv[2])));
  const float2 s23 = wsum2(L, __fadd2_rn(pr(xm[2], xm[3]), pr(xp[2], xp[3])), __fadd2_rn(pr(ym.z, ym.w), pr(yp.z, yp.w)),
                           __fadd2_rn(pr(xv[1], xv[2]), pr(xv[3], kr)));
  const float2 v01 = __fmul2_rn(__fadd2_rn(b01, s01), R.idg01(L, c9));
  const float2 v23 = __fmul2_rn(__fadd2_rn(b23, s23), R.idg23(L, c9));
  o[0] = t0 ? xv[0] : v01.x;
  o[1] = t0 ? v01.y : xv[1];
  o[2] = t0 ? xv[2] : v23.x;
  o[3] = t0 ? v23.y : xv[3];
}

template <int NQ, bool BS>
__global__ void __launch_bounds__(kMgMarchThreads, 2)
    k_mg_down4(MgLevel F, MgLevel Cl, const float *__restrict__ b, float *__restrict__ bc, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  constexpr int NZ = 4 * NQ;
  const int RY = F.mty + 4, PL = RY * NQ;
  extern __shared__ float4 msm[];
  float4 *const sa = msm + threadIdx.x, *const sb = msm + 3 * PL + threadIdx.x;  // colour 0 / both
  const MarchRow R = march_row<NQ>(F);
  const int is = blockIdx.x * F.msx, ie = min(F.nx, is + F.msx);
  const bool blk = R.jin && R.tj >= 1 && R.tj < RY - 1;  // colour 1: the band and one halo row
  const bool res = R.jin && R.tj >= 2 && R.tj < RY - 2;  // residual: the band
  const bool even = !(R.j & 1);
  const int sx = F.ny * NZ, o = (R.jin ? R.j : 0) * NZ + R.k0;  // 32-bit: under 2^31 cells
  auto ldb = [&](int p) -> float4 {
    return R.jin && p >= 0 && p < F.nx ? __ldg(reinterpret_cast<const float4 *>(b + (o + p * sx)))
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  float4 bn1 = ldb(is - 2), bn2 = ldb(is - 1);
  float bA[4] = {}, bB[4] = {}, bC[4] = {};  // b of planes p, p-1, p-2 (rotating)
  float xA[4] = {}, xB[4] = {}, xC[4] = {};  // colour 0 from zero, planes p, p-1, p-2
  float fA[4] = {}, fB[4] = {}, fC[4] = {};  // both colours, planes p-1, p-2, p-3
  float sA = 0.f, sB = 0.f;  // the restriction sums of the quad's two coarse cells (even rows)
  // s0, s1, s2: the shared slots of planes p, p - 1, p - 2
  auto step = [&](int p, float(&b0)[4], float(&b1)[4], float(&b2)[4], float(&x0)[4], float(&x1)[4],
                  float(&x2)[4], float(&f1)[4], float(&f2)[4], float(&f3)[4], int s0, int s1, int s2) {
    // plane p: b, and colour 0 from zero (zeros outside the level)
    unq(bn1, b0);
    bn1 = bn2;
    bn2 = ldb(p + 2);
    {
      int c9;
      const float dxy = march_dxy(F, R, p, c9);
      march_zero<BS>(F, R, dxy, c9, (p + R.j) & 1, b0, x0);
      sa[s0 * PL] = mkq(x0);
    }
    __syncthreads();
    {  // plane p - 1: colour 1 from colour 0
      const int i = p - 1;
      float kl, kr;
      march_kz(R, x1, kl, kr);
      if (blk && i >= 0 && i < F.nx) {
        int c9;
        const float dxy = march_dxy(F, R, i, c9);
        const float4 *s = sa + s1 * PL;
        march_pass<BS>(F, R, dxy, c9, (i + R.j + 1) & 1, b1, x1, x2, x0, s[-NQ], s[NQ], kl, kr, f1);
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) f1[c] = x1[c];
      }
      sb[s1 * PL] = mkq(f1);
    }
    {  // plane p - 2: the residual b - A x, restricted (k_mg_restrict8's sums)
      const int i = p - 2;
      float kl, kr;
      march_kz(R, f2, kl, kr);
      const bool act = res && i >= is && i < ie;
      float2 r01 = make_float2(0.f, 0.f), r23 = r01;
      if (act) {
        int c9;
        const float dxy = march_dxy(F, R, i, c9);
        const float4 *s = sb + s2 * PL;
        const float4 ym = s[-NQ], yp = s[NQ];
        float2 b01, b23;
        march_bb<BS>(R, dxy, b2, b01, b23);
        const float2 d01 = __fadd2_rn(bc2(dxy), R.wz01), d23 = __fadd2_rn(bc2(dxy), R.wz23);  // ldiag
        const float2 s01 = wsum2(F, __fadd2_rn(pr(f3[0], f3[1]), pr(f1[0], f1[1])),
                                 __fadd2_rn(pr(ym.x, ym.y), pr(yp.x, yp.y)), __fadd2_rn(pr(kl, f2[0]), pr(f2[1], f2[2])));
        const float2 s23 = wsum2(F, __fadd2_rn(pr(f3[2], f3[3]), pr(f1[2], f1[3])),
                                 __fadd2_rn(pr(ym.z, ym.w), pr(yp.z, yp.w)), __fadd2_rn(pr(f2[1], f2[2]), pr(f2[3], kr)));
        r01 = __fadd2_rn(__ffma2_rn(pr(-d01.x, -d01.y), pr(f2[0], f2[1]), b01), s01);
        r23 = __fadd2_rn(__ffma2_rn(pr(-d23.x, -d23.y), pr(f2[2], f2[3]), b23), s23);
      }
      // children (a, e, c) of a coarse cell summed in k_mg_restrict8's order: the odd row's
      // residuals by shuffle
      const float o0 = __shfl_down_sync(R.mask, r01.x, NQ), o1 = __shfl_down_sync(R.mask, r01.y, NQ);
      const float o2 = __shfl_down_sync(R.mask, r23.x, NQ), o3 = __shfl_down_sync(R.mask, r23.y, NQ);
      if (act && even) {
        if (!(i & 1)) {
          sA = 0.f;
          sB = 0.f;
        }
        sA = add_rn(add_rn(add_rn(add_rn(sA, r01.x), r01.y), o0), o1);
        sB = add_rn(add_rn(add_rn(add_rn(sB, r23.x), r23.y), o2), o3);
        if (i & 1) {
          const float inv = 1.f / 8.f;
          *reinterpret_cast<float2 *>(bc + lrow(Cl, i >> 1, R.j >> 1, 2 * R.q)) =
              make_float2(mul_rn(sA, inv), mul_rn(sB, inv));
        }
      }
    }
  };
  for (int p = is - 2;;) {
    step(p, bA, bC, bB, xA, xC, xB, fA, fC, fB, 0, 2, 1);
    if (++p > ie + 1) break;
    step(p, bB, bA, bC, xB, xA, xC, fB, fA, fC, 1, 0, 2);
    if (++p > ie + 1) break;
    step(p, bC, bB, bA, xC, xB, xA, fC, fB, fA, 2, 1, 0);
    if (++p > ie + 1) break;
  }
}

// a coarse plane's values for a quad's prolongation: rows pj, nj (the parent row and the
// neighbour on the child's side) x coarse z 2q - 1, 2q, 2q + 1, 2q + 2, the ends the parent
// beyond a wall or wrapped (k_mg_prolong8's taps); raw: the float2 pairs of the two rows
__device__ __forceinline__ void march_zext(const MarchRow &R, float4 raw, float (&o)[2][4]) {
  const float l0 = __shfl_sync(R.mask, raw.y, R.left), l1 = __shfl_sync(R.mask, raw.w, R.left);
  const float r0 = __shfl_sync(R.mask, raw.x, R.right), r1 = __shfl_sync(R.mask, raw.z, R.right);
  o[0][0] = R.zl ? l0 : raw.x;
  o[0][1] = raw.x;
  o[0][2] = raw.y;
  o[0][3] = R.zr ? r0 : raw.y;
  o[1][0] = R.zl ? l1 : raw.z;
  o[1][1] = raw.z;
  o[1][2] = raw.w;
  o[1][3] = R.zr ? r1 : raw.w;
}

template <int NQ, bool BS>
__global__ void __launch_bounds__(kMgMarchThreads, 2)
    k_mg_up4(MgLevel F, MgLevel Cl, const float *__restrict__ b, const float *__restrict__ xc, float *__restrict__ x,
             const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  constexpr int NZ = 4 * NQ;
  const int RY = F.mty + 4, PL = RY * NQ;
  extern __shared__ float4 msm[];
  float4 *const sa = msm + threadIdx.x, *const sb = msm + 3 * PL + threadIdx.x;  // colour 0 / both
  const MarchRow R = march_row<NQ>(F);
  const int is = blockIdx.x * F.msx, ie = min(F.nx, is + F.msx);
  const bool one = R.jin && R.tj >= 1 && R.tj < RY - 1;   // colour 1: the band and one halo row
  const bool zero = R.jin && R.tj >= 2 && R.tj < RY - 2;  // colour 0, stored: the band
  // 32-bit offsets: a marching level has fewer than 2^31 cells (mg_plan)
  const int sx = F.ny * NZ, o = (R.jin ? R.j : 0) * NZ + R.k0;
  auto ldb = [&](int p) -> float4 {
    return R.jin && p >= 0 && p < F.nx ? __ldg(reinterpret_cast<const float4 *>(b + (o + p * sx)))
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  // prolongation taps along y: the parent row and the neighbour on the child's side
  const int jc = min(max(R.j, 0), F.ny - 1), pj = jc >> 1;
  const int nj = (jc & 1) ? min(pj + 1, Cl.ny - 1) : max(pj - 1, 0);
  const int co = pj * Cl.nz + 2 * R.q, cd = (nj - pj) * Cl.nz, csx = Cl.ny * Cl.nz;
  auto ldc = [&](int m) -> float4 {  // coarse plane m (clamped to the level), rows pj and nj
    const int r = min(max(m, 0), Cl.nx - 1) * csx + co;
    const float2 u = __ldg(reinterpret_cast<const float2 *>(xc + r));
    const float2 v = __ldg(reinterpret_cast<const float2 *>(xc + (r + cd)));
    return make_float4(u.x, u.y, v.x, v.y);
  };
  // coarse planes m - 1 and m around the parent plane m = p / 2 of the fine plane p (raw
  // pairs, extended at each use), and m + 1 in flight during the parent's first child (is - 2
  // is even: the march starts on a first child)
  const int m0 = (is - 2) >> 1;
  float4 ca = ldc(m0 - 1), cb = ldc(m0), cn = cb;
  float4 bn1 = ldb(is - 2), bn2 = ldb(is - 1);
  float bA[4] = {}, bB[4] = {}, bC[4] = {};  // b of planes p, p-1, p-2 (rotating)
  // the earlier planes of both stages are read back from this thread's own shared slots
  // (registers are this kernel's limit); zeros before the march, as the planes before it
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    sa[q * PL] = make_float4(0.f, 0.f, 0.f, 0.f);
    sb[q * PL] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  auto step = [&](int p, float(&b0)[4], float(&b1)[4], float(&b2)[4], int s0, int s1, int s2) {
    const bool odd = p & 1;
    float x0[4], x1[4], x2[4], y1[4], y2[4], y3[4];  // colour 0 + P xc of p, p-1, p-2; after colour 1, p-1..p-3
    // plane p: colour 0 = b / diag + P xc (k_mg_prolong8: parent first on every axis)
    unq(bn1, b0);
    bn1 = bn2;
    bn2 = ldb(p + 2);
    {
      int c9;
      const float dxy = march_dxy(F, R, p, c9);
      const int t0 = (p + R.j) & 1;
      march_zero<BS>(F, R, dxy, c9, t0, b0, x0);
      // cells (0, 1) and (2, 3): z taps parent (1, 1), (2, 2), child's side (0, 2), (1, 3);
      // the parent plane (a = 0), then the plane on the child's side
      const float wa[2] = {0.75f, 0.25f};
      float2 v01 = make_float2(0.f, 0.f), v23 = v01;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        float cv[2][4];
        march_zext(R, a == 0 ? cb : (odd ? cn : ca), cv);
#pragma unroll
        for (int e = 0; e < 2; ++e)
#pragma unroll
          for (int t = 0; t < 2; ++t) {
            const float2 w = bc2(wa[a] * wa[e] * wa[t]);
            v01 = __ffma2_rn(w, t == 0 ? pr(cv[e][1], cv[e][1]) : pr(cv[e][0], cv[e][2]), v01);
            v23 = __ffma2_rn(w, t == 0 ? pr(cv[e][2], cv[e][2]) : pr(cv[e][1], cv[e][3]), v23);
          }
      }
      const float2 s01 = __fadd2_rn(pr(x0[0], x0[1]), v01), s23 = __fadd2_rn(pr(x0[2], x0[3]), v23);
      // outside the level: zeros, as the neighbours beyond a wall
      const bool in = R.jin && p >= 0 && p < F.nx;
      x0[0] = in && !t0 ? s01.x : 0.f;
      x0[1] = in && t0 ? s01.y : 0.f;
      x0[2] = in && !t0 ? s23.x : 0.f;
      x0[3] = in && t0 ? s23.y : 0.f;
      sa[s0 * PL] = mkq(x0);
      if (odd) {  // the next plane has the next parent
        ca = cb;
        cb = cn;
      } else {
        cn = ldc((p >> 1) + 1);
      }
    }
    __syncthreads();
    unq(sa[s1 * PL], x1);
    unq(sa[s2 * PL], x2);
    unq(sb[s2 * PL], y2);
    unq(sb[s0 * PL], y3);  // plane p - 3 (the slot that takes plane p in the next step)
    {  // plane p - 1: colour 1 of the post-smoothing
      const int i = p - 1;
      float kl, kr;
      march_kz(R, x1, kl, kr);
      if (one && i >= 0 && i < F.nx) {
        int c9;
        const float dxy = march_dxy(F, R, i, c9);
        const float4 *s = sa + s1 * PL;
        march_pass<BS>(F, R, dxy, c9, (i + R.j + 1) & 1, b1, x1, x2, x0, s[-NQ], s[NQ], kl, kr, y1);
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) y1[c] = x1[c];
      }
      sb[s1 * PL] = mkq(y1);
    }
    {  // plane p - 2: colour 0, stored
      const int i = p - 2;
      float kl, kr;
      march_kz(R, y2, kl, kr);
      if (zero && i >= is && i < ie) {
        int c9;
        const float dxy = march_dxy(F, R, i, c9);
        const float4 *s = sb + s2 * PL;
        float ov[4];
        march_pass<BS>(F, R, dxy, c9, (i + R.j) & 1, b2, y2, y3, y1, s[-NQ], s[NQ], kl, kr, ov);
        *reinterpret_cast<float4 *>(x + (o + i * sx)) = mkq(ov);
      }
    }
  };
  for (int p = is - 2;;) {
    step(p, bA, bC, bB, 0, 2, 1);
    if (++p > ie + 1) break;
    step(p, bB, bA, bC, 1, 0, 2);
    if (++p > ie + 1) break;
    step(p, bC, bB, bA, 2, 1, 0);
    if (++p > ie + 1) break;
  }
}

// coarsest level: x = 0, then `sweeps` red-black sweeps in shared memory, one block
// x = M b on the coarsest level with the precomputed pseudo-inverse M (n x n, row-major):
// one dot product of length n per cell (the block's shared copies of b, x)
template <typename T>
__device__ void blk_dense(int n, const T *__restrict__ M, const T *bs, T *xs) {
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const T *row = M + (long long)q * n;
    T v = T(0);
    for (int c = 0; c < n; ++c) v += row[c] * bs[c];
    xs[q] = v;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(1024) k_mg_coarse(MgLevelT<T> L, int sweeps, const T *__restrict__ M, int bscale,
                                                    const T *__restrict__ b, T *__restrict__ x, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smraw[];
  T *sm = reinterpret_cast<T *>(smraw);
  const int n = L.nx * L.ny * L.nz;
  T *xs = sm, *bs = sm + n;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int k = q % L.nz, t = q / L.nz, j = t % L.ny, i = t / L.ny;
    T bb = b[q];
    if (bscale) bb *= ldiag(L, i, j, k);
    bs[q] = bb;
    xs[q] = T(0);
  }
  __syncthreads();
  if (M) {
    blk_dense(n, M, bs, xs);
    sweeps = 0;
  }
  for (int s = 0; s < sweeps; ++s)
    for (int colour = 0; colour < 2; ++colour) {
      for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int k = q % L.nz, t = q / L.nz, j = t % L.ny, i = t / L.ny;
        if (((i + j + k) & 1) != colour) continue;
        xs[q] = (bs[q] + lnb(L, xs, i, j, k, q)) * linv(L, i, j, k);
      }
      __syncthreads();
    }
  for (int q = threadIdx.x; q < n; q += blockDim.x) x[q] = xs[q];
}

// ---- the small levels in one block: levels t..nlev-1 together hold at most
// kMgTailBytes / (2 sizeof(T)) cells, x and b of each in shared memory; the same smoothing,
// transfers and coarsest solve as the per-level kernels (same arithmetic, same order), a
// barrier between phases where the per-level path has a launch ----
// 48 KB: one block working on more cells per barrier (a 16K-cell level, 192 KB) ran slower
// than the same level's launched kernels (measured on 512x256x64)
constexpr int kMgTailBytes = 48 * 1024;
template <typename T>
constexpr int tail_cells_max() { return kMgTailBytes / (2 * (int)sizeof(T)); }

// Unsigned division by an invariant d >= 1 (Granlund and Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994, the round-up method): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (t + ((n - t) >> 1)) >> (l - 1), t = mulhi(m, n),
// for every 32-bit n (d = 1: l = 0 and the quotient is n).
static inline void div_magic(unsigned d, unsigned *m, int *l) {
  int ll = 0;
  while ((1ull << ll) < d) ++ll;
  *l = ll;
  *m = (unsigned)((((1ull << ll) - d) << 32) / d + 1);
}
__device__ __forceinline__ unsigned udiv_inv(unsigned n, unsigned m, int l) {
  if (l == 0) return n;
  const unsigned t = __umulhi(m, n);
  return (t + ((n - t) >> 1)) >> (l - 1);
}

template <typename T>
__device__ __forceinline__ void cell_ijk(const MgLevelT<T> &L, int q, int &i, int &j, int &k) {
  const unsigned t = udiv_inv((unsigned)q, L.dz_m, L.dz_l), u = udiv_inv(t, L.dy_m, L.dy_l);
  k = q - (int)t * L.nz;
  j = (int)t - (int)u * L.ny;
  i = (int)u;
}

template <typename T>
__device__ void blk_smooth(const MgLevelT<T> &L, int colour, int zero, const T *b, T *x) {
  const int n = L.nx * L.ny * L.nz;
  if (L.nz % 2 == 0) {
    // the cells of a row pair up along k, one of each colour: a thread per pair updates the
    // one of the colour (and, from zero, clears the other)
    const int half = L.nz / 2, np = n / 2;
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
      const unsigned r = udiv_inv((unsigned)p, L.dh_m, L.dh_l), ii = udiv_inv(r, L.dy_m, L.dy_l);
      const int i = (int)ii, j = (int)r - i * L.ny, d = (i + j + colour) & 1;
      const int k = 2 * (p - (int)r * half) + d, q = (int)r * L.nz + k;
      if (zero) x[q + 1 - 2 * d] = T(0);
      const T num = zero ? b[q] : b[q] + lnb(L, x, i, j, k, q);
      x[q] = num * linv(L, i, j, k);
    }
    __syncthreads();
    return;
  }
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, k;
    cell_ijk(L, q, i, j, k);
    if (((i + j + k) & 1) != colour) {
      if (zero) x[q] = T(0);
      continue;
    }
    const T num = zero ? b[q] : b[q] + lnb(L, x, i, j, k, q);
    x[q] = num * linv(L, i, j, k);
  }
  __syncthreads();
}

template <typename T>
__device__ void blk_restrict(const MgLevelT<T> &F, const MgLevelT<T> &Cl, const T *bf, const T *xf, T *bc) {
  const T inv = T(1) / (T)(F.fx * F.fy * F.fz);
  const int n = Cl.nx * Cl.ny * Cl.nz;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, k;
    cell_ijk(Cl, q, i, j, k);
    T sum = T(0);
    for (int a = 0; a < F.fx; ++a)
      for (int e = 0; e < F.fy; ++e)
        for (int c = 0; c < F.fz; ++c) {
          const int fi = i * F.fx + a, fj = j * F.fy + e, fk = k * F.fz + c;
          const long long r = lrow(F, fi, fj, fk);
          const T d = ldiag(F, fi, fj, fk);
          sum += bf[r] - d * xf[r] + lnb(F, xf, fi, fj, fk, r);
        }
    bc[q] = sum * inv;
  }
  __syncthreads();
}

template <typename T>
__device__ void blk_prolong(const MgLevelT<T> &F, const MgLevelT<T> &Cl, const T *xc, T *xf) {
  const int n = F.nx * F.ny * F.nz;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, k;
    cell_ijk(F, q, i, j, k);
    xf[q] += prolong_at(F, Cl, xc, i, j, k);
  }
  __syncthreads();
}

// x_t = V-cycle of levels t..nlev-1 on b_t (both in global memory, level t >= 1)
template <typename T>
__global__ void __launch_bounds__(1024) k_mg_tail(MgPlanT<T> mg, int t, const SolverScal *sc) {
  pdl_wait();
  if (sc->done) return;
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smraw[];
  T *sm = reinterpret_cast<T *>(smraw);
  const int n = mg.nlev;
  T *xs[kMgMaxLevels], *bs[kMgMaxLevels];
  int off = 0;
  for (int l = t; l < n; ++l) {
    const int c = mg.lev[l].nx * mg.lev[l].ny * mg.lev[l].nz;
    xs[l] = sm + off;
    bs[l] = sm + off + c;
    off += 2 * c;
  }
  const int nt = mg.lev[t].nx * mg.lev[t].ny * mg.lev[t].nz;
  for (int q = threadIdx.x; q < nt; q += blockDim.x) bs[t][q] = mg.lev[t].b[q];
  __syncthreads();
  for (int l = t; l + 1 < n; ++l) {
    blk_smooth(mg.lev[l], 0, 1, bs[l], xs[l]);
    blk_smooth(mg.lev[l], 1, 0, bs[l], xs[l]);
    blk_restrict(mg.lev[l], mg.lev[l + 1], bs[l], xs[l], bs[l + 1]);
  }
  {  // coarsest: the dense pseudo-inverse, or x = 0 and red-black sweeps (k_mg_coarse)
    const MgLevelT<T> &C = mg.lev[n - 1];
    const int nc = C.nx * C.ny * C.nz;
    if (mg.cinv) {
      blk_dense(nc, mg.cinv, bs[n - 1], xs[n - 1]);
    } else {
      for (int q = threadIdx.x; q < nc; q += blockDim.x) xs[n - 1][q] = T(0);
      __syncthreads();
      for (int s = 0; s < mg.coarse_sweeps; ++s) {
        blk_smooth(C, 0, 0, bs[n - 1], xs[n - 1]);
        blk_smooth(C, 1, 0, bs[n - 1], xs[n - 1]);
      }
    }
  }
  for (int l = n - 2; l >= t; --l) {
    blk_prolong(mg.lev[l], mg.lev[l + 1], xs[l + 1], xs[l]);
    blk_smooth(mg.lev[l], 1, 0, bs[l], xs[l]);
    blk_smooth(mg.lev[l], 0, 0, bs[l], xs[l]);
  }
  for (int q = threadIdx.x; q < nt; q += blockDim.x) mg.lev[t].x[q] = xs[t][q];
}

template <typename T>
static void level_geometry(MgLevelT<T> &L, int nsm, bool quads) {
  L.bx = 1;
  while (L.bx < L.nz && L.bx < 32) L.bx *= 2;
  L.by = kBlock / L.bx;
  L.gx = (L.nz + L.bx - 1) / L.bx;
  L.gy = (L.ny + L.by - 1) / L.by;
  L.gz = std::max(1, std::min(L.nx, nsm * 8 / std::max(1, L.gx * L.gy)));
  // the quad smoother is FP32 (float4 loads): quads along x, rows along y, planes over z
  L.qgrid = quads && sizeof(T) == sizeof(float) && L.nz % 4 == 0 ? 1 : 0;
  if (L.qgrid) {
    const int nq = L.nz / 4;
    L.qbx = 1;
    while (L.qbx < nq && L.qbx < 32) L.qbx *= 2;
    L.qby = kBlock / L.qbx;
    L.qgx = (nq + L.qbx - 1) / L.qbx;
    L.qgy = (L.ny + L.qby - 1) / L.qby;
    L.qgz = std::max(1, std::min(L.nx, nsm * 8 / std::max(1, L.qgx * L.qgy)));
  }
}

template <typename T>
bool mg_plan(int nx, int ny, int nz, double hx, double hy, double hz, int nsm, bool quads, MgPlanT<T> *mg,
             bool pz) {
  *mg = MgPlanT<T>{};
  int l = 0;
  for (;;) {
    MgLevelT<T> &L = mg->lev[l];
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.pz = pz ? 1 : 0;
    // periodic z: red-black colouring holds across the wrap only for an even nz (or one
    // cell, which has no z neighbours)
    if (pz && nz % 2 && nz > 1) return false;
    L.wx = (T)(1.0 / (hx * hx));
    L.wy = (T)(1.0 / (hy * hy));
    L.wz = (T)(1.0 / (hz * hz));
    for (int q = 0; q < 27; ++q) {  // the diagonal as ldiag sums it, then its reciprocal
      const T d = L.wx * (T)(q / 9) + L.wy * (T)((q / 3) % 3) + L.wz * (T)(q % 3);
      L.idg[q] = d > T(0) ? T(1) / d : T(0);
    }
    level_geometry(L, nsm, quads);
    div_magic((unsigned)nz, &L.dz_m, &L.dz_l);
    div_magic((unsigned)ny, &L.dy_m, &L.dy_l);
    div_magic((unsigned)std::max(1, nz / 2), &L.dh_m, &L.dh_l);
    const long long cells = (long long)nx * ny * nz;
    const int fx = nx % 2 == 0 ? 2 : 1, fy = ny % 2 == 0 ? 2 : 1, fz = nz % 2 == 0 ? 2 : 1;
    if (cells <= kMgCoarseCells || fx * fy * fz == 1 || l + 1 == kMgMaxLevels) {
      L.fx = L.fy = L.fz = 1;
      break;
    }
    L.fx = fx;
    L.fy = fy;
    L.fz = fz;
    // the marching kernels: a band of 256 / (nz / 4) rows (at most ny), the segments sized so
    // that about two blocks per SM run
    const int nq = nz / 4;
    if (L.qgrid && fx == 2 && fy == 2 && fz == 2 && nq <= 16 && (nq & (nq - 1)) == 0 && cells < (1LL << 31)) {
      L.march = 1;
      L.mty = std::min(256 / nq, ny);
      L.mgy = (ny + L.mty - 1) / L.mty;
      const long long want = 2LL * nsm;
      L.msx = 2 * (int)std::max(1LL, ((long long)nx * L.mgy + 2 * want - 1) / (2 * want));
      L.mgx = (nx + L.msx - 1) / L.msx;
    }
    nx /= fx;
    ny /= fy;
    nz /= fz;
    hx *= fx;
    hy *= fy;
    hz *= fz;
    ++l;
  }
  mg->nlev = l + 1;
  // first level of the one-block tail: the smallest t >= 1 whose levels t..nlev-1 fit
  mg->tail = mg->nlev;  // none
  long long tail_cells = 0;
  for (int t = mg->nlev - 1; t >= 1; --t) {
    tail_cells += (long long)mg->lev[t].nx * mg->lev[t].ny * mg->lev[t].nz;
    if (tail_cells > tail_cells_max<T>()) break;
    mg->tail = t;
  }
  const MgLevelT<T> &C = mg->lev[l];
  mg->coarse_sweeps = std::min(256, 16 + 2 * std::max(C.nx, std::max(C.ny, C.nz)));
  return (long long)C.nx * C.ny * C.nz <= kMgSharedCells;
}

// per level above the tail (or the coarsest): 2 smooths + restrict, prolong + 2 smooths, or
// the two marching kernels; then one tail (or coarsest) kernel
template <typename T>
int mg_vcycle_launches(const MgPlanT<T> &mg) {
  const int m = mg.tail < mg.nlev ? mg.tail : mg.nlev - 1;
  int n = 1;
  for (int l = 0; l < m; ++l) n += mg.lev[l].march ? 2 : 6;
  return n;
}

// The pseudo-inverse of the coarsest level's operator (symmetric, singular on constants
// only): A+ = (A + J/n)^-1 - J/n with J the all-ones matrix, inverted by Gauss-Jordan with
// partial pivoting in double.  False when the level is larger than kMgDenseCells.
template <typename T>
bool mg_dense_inverse(const MgPlanT<T> &mg, std::vector<T> &M) {
  const MgLevelT<T> &C = mg.lev[mg.nlev - 1];
  const int n = C.nx * C.ny * C.nz;
  if (n > kMgDenseCells) return false;
  std::vector<double> A((size_t)n * n, 0.0), I((size_t)n * n, 0.0);
  const double wx = (double)C.wx, wy = (double)C.wy, wz = (double)C.wz;
  for (int i = 0; i < C.nx; ++i)
    for (int j = 0; j < C.ny; ++j)
      for (int k = 0; k < C.nz; ++k) {
        const int r = (i * C.ny + j) * C.nz + k;
        auto link = [&](int q, double w) {
          A[(size_t)r * n + q] -= w;
          A[(size_t)r * n + r] += w;
        };
        if (i > 0) link(r - C.ny * C.nz, wx);
        if (i < C.nx - 1) link(r + C.ny * C.nz, wx);
        if (j > 0) link(r - C.nz, wy);
        if (j < C.ny - 1) link(r + C.nz, wy);
        if (C.pz) {
          if (C.nz > 1) {
            link(k > 0 ? r - 1 : r + C.nz - 1, wz);
            link(k < C.nz - 1 ? r + 1 : r + 1 - C.nz, wz);
          }
        } else {
          if (k > 0) link(r - 1, wz);
          if (k < C.nz - 1) link(r + 1, wz);
        }
      }
  for (size_t q = 0; q < A.size(); ++q) A[q] += 1.0 / n;
  for (int r = 0; r < n; ++r) I[(size_t)r * n + r] = 1.0;
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (std::fabs(A[(size_t)r * n + col]) > std::fabs(A[(size_t)piv * n + col])) piv = r;
    if (!(std::fabs(A[(size_t)piv * n + col]) > 0.0)) return false;
    if (piv != col)
      for (int c = 0; c < n; ++c) {
        std::swap(A[(size_t)piv * n + c], A[(size_t)col * n + c]);
        std::swap(I[(size_t)piv * n + c], I[(size_t)col * n + c]);
      }
    const double inv = 1.0 / A[(size_t)col * n + col];
    for (int c = 0; c < n; ++c) {
      A[(size_t)col * n + c] *= inv;
      I[(size_t)col * n + c] *= inv;
    }
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const double f = A[(size_t)r * n + col];
      if (f == 0.0) continue;
      for (int c = 0; c < n; ++c) {
        A[(size_t)r * n + c] -= f * A[(size_t)col * n + c];
        I[(size_t)r * n + c] -= f * I[(size_t)col * n + c];
      }
    }
  }
  M.resize((size_t)n * n);
  for (size_t q = 0; q < M.size(); ++q) M[q] = (T)(I[q] - 1.0 / n);
  return true;
}

template <typename T>
void mg_prepare() {
  // the one-block kernels of the FP64 hierarchy need more than the default 48 KB
  cudaFuncSetAttribute(k_mg_coarse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(2 * sizeof(T) * kMgSharedCells));
  cudaFuncSetAttribute(k_mg_tail<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMgTailBytes);
}

template <typename T>
void launch_mg_vcycle(cudaStream_t s, const MgPlanT<T> &mg, int jacobi, const T *b0, T *x0, const SolverScal *sc) {
  const int n = mg.nlev;
  auto B = [&](int l) -> const T * { return l == 0 ? b0 : mg.lev[l].b; };
  auto X = [&](int l) -> T * { return l == 0 ? x0 : mg.lev[l].x; };
  auto grid = [&](int l) { return dim3(mg.lev[l].gx, mg.lev[l].gy, mg.lev[l].gz); };
  auto block = [&](int l) { return dim3(mg.lev[l].bx, mg.lev[l].by, 1); };
  auto smooth = [&](int l, int colour, int zero) {
    if constexpr (sizeof(T) == sizeof(float)) {
      if (mg.lev[l].qgrid > 0) {
        const MgLevelT<T> &Q = mg.lev[l];
        launch_pdl(k_mg_smooth4, dim3(Q.qgx, Q.qgy, Q.qgz), dim3(Q.qbx, Q.qby, 1), 0, s, Q, colour, zero,
                   l == 0 ? jacobi : 0, B(l), X(l), sc);
        return;
      }
    }
    launch_pdl(k_mg_smooth<T>, grid(l), block(l), 0, s, mg.lev[l], colour, zero, l == 0 ? jacobi : 0, B(l), X(l), sc);
  };
  // pre-smoothing from zero and restriction to level l + 1.  (Both colour passes in one
  // kernel, each black cell recomputing its red neighbours' start values, was measured at
  // 80 us on the 512x256x64 level against 36 us for the two quad passes: not kept.)
  // the marching kernels of a level (FP32 only; nz / 4 a power of two up to 16)
  auto march = [&](int l, bool up) {
    if constexpr (sizeof(T) == sizeof(float)) {
      const MgLevelT<T> &F = mg.lev[l], &Cl = mg.lev[l + 1];
      const int bs = l == 0 ? jacobi : 0, nq = F.nz / 4;
      const dim3 grid(F.mgx, F.mgy), block(nq * (F.mty + 4));
      const size_t smem = 6 * sizeof(float4) * (size_t)block.x;
#define CFDGB_MARCH(NQ)                                                                                      \
  case NQ:                                                                                                 \
    if (up && bs)                                                                                          \
      launch_pdl(k_mg_up4<NQ, true>, grid, block, smem, s, F, Cl, B(l), (const T *)X(l + 1), X(l), sc);     \
    else if (up)                                                                                           \
      launch_pdl(k_mg_up4<NQ, false>, grid, block, smem, s, F, Cl, B(l), (const T *)X(l + 1), X(l), sc);    \
    else if (bs)                                                                                           \
      launch_pdl(k_mg_down4<NQ, true>, grid, block, smem, s, F, Cl, B(l), Cl.b, sc);                        \
    else                                                                                                   \
      launch_pdl(k_mg_down4<NQ, false>, grid, block, smem, s, F, Cl, B(l), Cl.b, sc);                       \
    break;
      switch (nq) {
        CFDGB_MARCH(1)
        CFDGB_MARCH(2)
        CFDGB_MARCH(4)
        CFDGB_MARCH(8)
        CFDGB_MARCH(16)
      }
#undef CFDGB_MARCH
    }
  };
  auto down = [&](int l) {
    if (mg.lev[l].march) {
      march(l, false);
      return;
    }
    const int bs = l == 0 ? jacobi : 0;
    smooth(l, 0, 1);
    smooth(l, 1, 0);
    const MgLevelT<T> &F = mg.lev[l];
    if (F.fx == 2 && F.fy == 2 && F.fz == 2)
      launch_pdl(k_mg_restrict8<T>, grid(l + 1), block(l + 1), 0, s, F, mg.lev[l + 1], bs, B(l), X(l),
                 mg.lev[l + 1].b, sc);
    else
      launch_pdl(k_mg_restrict<T>, grid(l + 1), block(l + 1), 0, s, F, mg.lev[l + 1], bs, B(l), X(l),
                 mg.lev[l + 1].b, sc);
  };
  const int m = std::min(mg.tail, n);  // levels m..n-1 run in one block (m < n), or none
  for (int l = 0; l + 1 < m; ++l) down(l);
  if (m < n) {
    down(m - 1);  // levels m-1 -> m as above, then the tail
    size_t cells = 0;
    for (int l = m; l < n; ++l) cells += (size_t)mg.lev[l].nx * mg.lev[l].ny * mg.lev[l].nz;
    launch_pdl(k_mg_tail<T>, dim3(1), dim3(1024), 2 * sizeof(T) * cells, s, mg, m, sc);
  } else {
    const MgLevelT<T> &C = mg.lev[n - 1];
    const size_t smem = 2 * sizeof(T) * (size_t)C.nx * C.ny * C.nz;
    launch_pdl(k_mg_coarse<T>, dim3(1), dim3(1024), smem, s, C, mg.coarse_sweeps, mg.cinv, n == 1 ? jacobi : 0,
               B(n - 1), X(n - 1), sc);
  }
  for (int l = (m < n ? m : n - 1) - 1; l >= 0; --l) {
    const MgLevelT<T> &F = mg.lev[l];
    if (F.march) {
      march(l, true);
      continue;
    }
    if (F.fx == 2 && F.fy == 2 && F.fz == 2)
      launch_pdl(k_mg_prolong8<T>, grid(l + 1), block(l + 1), 0, s, F, mg.lev[l + 1], (const T *)X(l + 1), X(l), sc);
    else
      launch_pdl(k_mg_prolong<T>, grid(l), block(l), 0, s, F, mg.lev[l + 1], (const T *)X(l + 1), X(l), sc);
    smooth(l, 1, 0);
    smooth(l, 0, 0);
  }
}

template bool mg_plan<float>(int, int, int, double, double, double, int, bool, MgPlanT<float> *, bool);
template bool mg_plan<double>(int, int, int, double, double, double, int, bool, MgPlanT<double> *, bool);
template int mg_vcycle_launches<float>(const MgPlanT<float> &);
template bool mg_dense_inverse<float>(const MgPlanT<float> &, std::vector<float> &);
template bool mg_dense_inverse<double>(const MgPlanT<double> &, std::vector<double> &);
template int mg_vcycle_launches<double>(const MgPlanT<double> &);
template void mg_prepare<float>();
template void mg_prepare<double>();
template void launch_mg_vcycle<float>(cudaStream_t, const MgPlanT<float> &, int, const float *, float *,
                                      const SolverScal *);
template void launch_mg_vcycle<double>(cudaStream_t, const MgPlanT<double> &, int, const double *, double *,
                                       const SolverScal *);

}  // namespace cfdgb
