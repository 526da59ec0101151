// Geometric multigrid V-cycle in FP32: the preconditioner of the FP32 BiCGSTAB sweep
// inside the FP64 refinement (the reference has no multigrid; its Poisson operator on a
// uniform grid is the 7-point Neumann Laplacian of SPE_sparseMatrix.hpp:42-85, which every
// level here rediscretises at its own spacing).
//
// Cell-centred hierarchy: a coarse cell is the union of 2 cells along each halved axis.
// Restriction averages the fine residual over a coarse cell's children; prolongation is
// the cell-centred trilinear interpolation (weights 3/4 and 1/4 per halved axis, the
// parent's value standing in for a neighbour beyond a Neumann wall); the smoother is
// red-black Gauss-Seidel, one sweep before and one after the coarse correction; the
// coarsest level (at most kMgSharedCells cells) is solved by red-black sweeps in the
// shared memory of one block.  The V-cycle is a fixed linear map, as a right
// preconditioner of BiCGSTAB requires.  Every kernel is pointwise or a stencil over one
// level and reads sc->done first, so a captured chunk of iterations idles once the sweep
// has stopped.
#include <algorithm>

#include "cfdgb_internal.cuh"
#include "kernels.h"

namespace cfdgb {

#define FOR_LEVEL(L)                                   \
  const int k = blockIdx.x * blockDim.x + threadIdx.x; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y; \
  const bool on_ = (k < (L).nz) && (j < (L).ny);       \
  for (int i = blockIdx.z; on_ && i < (L).nx; i += gridDim.z)

__device__ __forceinline__ long long lrow(const MgLevel &L, int i, int j, int k) {
  return ((long long)i * L.ny + j) * L.nz + k;
}

// diagonal of a Neumann row: the weights of the neighbours that exist
__device__ __forceinline__ float ldiag(const MgLevel &L, int i, int j, int k) {
  return L.wx * (float)((i > 0) + (i < L.nx - 1)) + L.wy * (float)((j > 0) + (j < L.ny - 1)) +
         L.wz * (float)((k > 0) + (k < L.nz - 1));
}

// weighted sum of the neighbours' values (minus the off-diagonal part of the row)
__device__ __forceinline__ float lnb(const MgLevel &L, const float *x, int i, int j, int k, long long r) {
  const long long sx = (long long)L.ny * L.nz;
  float a = 0.f, b = 0.f, c = 0.f;
  if (i > 0) a += x[r - sx];
  if (i < L.nx - 1) a += x[r + sx];
  if (j > 0) b += x[r - L.nz];
  if (j < L.ny - 1) b += x[r + L.nz];
  if (k > 0) c += x[r - 1];
  if (k < L.nz - 1) c += x[r + 1];
  return L.wx * a + L.wy * b + L.wz * c;
}

// One colour of a red-black Gauss-Seidel sweep (colour = (i + j + k) & 1).  zero: x starts
// at zero, so the cells of this colour take b / diag and the others are set to zero.
// bscale: b holds Jacobi-scaled rows (b / diag), which are unscaled first.
__global__ void __launch_bounds__(kBlock) k_mg_smooth(MgLevel L, int colour, int zero, int bscale,
                                                      const float *__restrict__ b, float *x, const SolverScal *sc) {
  if (sc->done) return;
  FOR_LEVEL(L) {
    const long long r = lrow(L, i, j, k);
    if (((i + j + k) & 1) != colour) {
      if (zero) x[r] = 0.f;
      continue;
    }
    const float d = ldiag(L, i, j, k);
    float bb = b[r];
    if (bscale) bb *= d;
    const float num = zero ? bb : bb + lnb(L, x, i, j, k, r);
    x[r] = d > 0.f ? num / d : 0.f;
  }
}

// The same colour pass on quads of four consecutive k cells (nz % 4 == 0): a thread updates
// the two cells of the colour in its quad and stores the whole quad, the other two
// unchanged (no thread writes them in this pass, so rewriting them races with nothing).
// Neighbour sums in the order of lnb.
__global__ void __launch_bounds__(kBlock) k_mg_smooth4(MgLevel L, int colour, int zero, int bscale,
                                                       const float *__restrict__ b, float *x, const SolverScal *sc) {
  if (sc->done) return;
  const unsigned nq = (unsigned)L.nz >> 2, nquads = (unsigned)L.nx * L.ny * nq;
  const long long sx = (long long)L.ny * L.nz;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < nquads; q += gridDim.x * blockDim.x) {
    const unsigned t = q / nq, kq = q - t * nq, j = t % (unsigned)L.ny, i = t / (unsigned)L.ny;
    const int k0 = (int)(4 * kq);
    const long long r = lrow(L, (int)i, (int)j, k0);
    const int t0 = ((int)i + (int)j + k0 + colour) & 1;  // first cell of the colour in the quad
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
        const float d = ldiag(L, (int)i, (int)j, k0 + c);
        const float bb = bscale ? bv[c] * d : bv[c];
        o[c] = d > 0.f ? bb / d : 0.f;
      }
    } else {
      const float4 xq = *reinterpret_cast<const float4 *>(x + r);
      const float xv[4] = {xq.x, xq.y, xq.z, xq.w};
      const bool im = i > 0, ip = (int)i < L.nx - 1, jm = j > 0, jp = (int)j < L.ny - 1;
      const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 xm = im ? *reinterpret_cast<const float4 *>(x + r - sx) : z4;
      const float4 xp = ip ? *reinterpret_cast<const float4 *>(x + r + sx) : z4;
      const float4 ym = jm ? *reinterpret_cast<const float4 *>(x + r - L.nz) : z4;
      const float4 yp = jp ? *reinterpret_cast<const float4 *>(x + r + L.nz) : z4;
      const float xmv[4] = {xm.x, xm.y, xm.z, xm.w}, xpv[4] = {xp.x, xp.y, xp.z, xp.w};
      const float ymv[4] = {ym.x, ym.y, ym.z, ym.w}, ypv[4] = {yp.x, yp.y, yp.z, yp.w};
      const float kl = k0 > 0 ? x[r - 1] : 0.f, kr = k0 + 4 < L.nz ? x[r + 4] : 0.f;
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
        if (k > 0) f += c == 0 ? kl : xv[c - 1];
        if (k < L.nz - 1) f += c == 3 ? kr : xv[c + 1];
        const float d = ldiag(L, (int)i, (int)j, k);
        const float bb = bscale ? bv[c] * d : bv[c];
        o[c] = d > 0.f ? (bb + (L.wx * a + L.wy * e + L.wz * f)) / d : 0.f;
      }
    }
    *reinterpret_cast<float4 *>(x + r) = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// bc = average over each coarse cell's children of the fine residual b - A x
__global__ void __launch_bounds__(kBlock) k_mg_restrict(MgLevel F, MgLevel Cl, int bscale, const float *__restrict__ bf,
                                                        const float *__restrict__ xf, float *__restrict__ bc,
                                                        const SolverScal *sc) {
  if (sc->done) return;
  const float inv = 1.0f / (float)(F.fx * F.fy * F.fz);
  FOR_LEVEL(Cl) {
    float sum = 0.f;
    for (int a = 0; a < F.fx; ++a)
      for (int e = 0; e < F.fy; ++e)
        for (int c = 0; c < F.fz; ++c) {
          const int fi = i * F.fx + a, fj = j * F.fy + e, fk = k * F.fz + c;
          const long long r = lrow(F, fi, fj, fk);
          const float d = ldiag(F, fi, fj, fk);
          float bb = bf[r];
          if (bscale) bb *= d;
          sum += bb - d * xf[r] + lnb(F, xf, fi, fj, fk, r);
        }
    bc[lrow(Cl, i, j, k)] = sum * inv;
  }
}

// the two coarse cells a fine cell interpolates from along one axis, and their weights
__device__ __forceinline__ void axis_taps(int i, int f, int n, int (&c)[2], float (&w)[2]) {
  if (f == 1) {
    c[0] = c[1] = i;
    w[0] = 1.f;
    w[1] = 0.f;
    return;
  }
  const int p = i >> 1;
  int q = p + ((i & 1) ? 1 : -1);
  if (q < 0 || q >= n) q = p;  // beyond a wall: the parent's value (zero normal gradient)
  c[0] = p;
  c[1] = q;
  w[0] = 0.75f;
  w[1] = 0.25f;
}

// xf += P xc
__global__ void __launch_bounds__(kBlock) k_mg_prolong(MgLevel F, MgLevel Cl, const float *__restrict__ xc,
                                                       float *__restrict__ xf, const SolverScal *sc) {
  if (sc->done) return;
  FOR_LEVEL(F) {
    int ci[2], cj[2], ck[2];
    float wi[2], wj[2], wk[2];
    axis_taps(i, F.fx, Cl.nx, ci, wi);
    axis_taps(j, F.fy, Cl.ny, cj, wj);
    axis_taps(k, F.fz, Cl.nz, ck, wk);
    float v = 0.f;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const float w = wi[a] * wj[e] * wk[c];
          if (w != 0.f) v += w * xc[lrow(Cl, ci[a], cj[e], ck[c])];
        }
    xf[lrow(F, i, j, k)] += v;
  }
}

// coarsest level: x = 0, then `sweeps` red-black sweeps in shared memory, one block
__global__ void __launch_bounds__(1024) k_mg_coarse(MgLevel L, int sweeps, int bscale, const float *__restrict__ b,
                                                    float *__restrict__ x, const SolverScal *sc) {
  if (sc->done) return;
  extern __shared__ float sm[];
  const int n = L.nx * L.ny * L.nz;
  float *xs = sm, *bs = sm + n;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int k = q % L.nz, t = q / L.nz, j = t % L.ny, i = t / L.ny;
    float bb = b[q];
    if (bscale) bb *= ldiag(L, i, j, k);
    bs[q] = bb;
    xs[q] = 0.f;
  }
  __syncthreads();
  for (int s = 0; s < sweeps; ++s)
    for (int colour = 0; colour < 2; ++colour) {
      for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int k = q % L.nz, t = q / L.nz, j = t % L.ny, i = t / L.ny;
        if (((i + j + k) & 1) != colour) continue;
        const float d = ldiag(L, i, j, k);
        xs[q] = d > 0.f ? (bs[q] + lnb(L, xs, i, j, k, q)) / d : 0.f;
      }
      __syncthreads();
    }
  for (int q = threadIdx.x; q < n; q += blockDim.x) x[q] = xs[q];
}

// ---- the small levels in one block: levels t..nlev-1 together hold at most kMgTailCells
// cells, x and b of each in shared memory; the same smoothing, transfers and coarsest solve
// as the per-level kernels (same arithmetic, same order), a barrier between phases where
// the per-level path has a launch ----
constexpr int kMgTailCells = 6144;  // 2 arrays of floats: 48 KB of shared memory

__device__ __forceinline__ void cell_ijk(const MgLevel &L, int q, int &i, int &j, int &k) {
  k = q % L.nz;
  const int t = q / L.nz;
  j = t % L.ny;
  i = t / L.ny;
}

__device__ void blk_smooth(const MgLevel &L, int colour, int zero, const float *b, float *x) {
  const int n = L.nx * L.ny * L.nz;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, k;
    cell_ijk(L, q, i, j, k);
    if (((i + j + k) & 1) != colour) {
      if (zero) x[q] = 0.f;
      continue;
    }
    const float d = ldiag(L, i, j, k);
    const float num = zero ? b[q] : b[q] + lnb(L, x, i, j, k, q);
    x[q] = d > 0.f ? num / d : 0.f;
  }
  __syncthreads();
}

__device__ void blk_restrict(const MgLevel &F, const MgLevel &Cl, const float *bf, const float *xf, float *bc) {
  const float inv = 1.0f / (float)(F.fx * F.fy * F.fz);
  const int n = Cl.nx * Cl.ny * Cl.nz;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, k;
    cell_ijk(Cl, q, i, j, k);
    float sum = 0.f;
    for (int a = 0; a < F.fx; ++a)
      for (int e = 0; e < F.fy; ++e)
        for (int c = 0; c < F.fz; ++c) {
          const int fi = i * F.fx + a, fj = j * F.fy + e, fk = k * F.fz + c;
          const long long r = lrow(F, fi, fj, fk);
          const float d = ldiag(F, fi, fj, fk);
          sum += bf[r] - d * xf[r] + lnb(F, xf, fi, fj, fk, r);
        }
    bc[q] = sum * inv;
  }
  __syncthreads();
}

__device__ void blk_prolong(const MgLevel &F, const MgLevel &Cl, const float *xc, float *xf) {
  const int n = F.nx * F.ny * F.nz;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, k;
    cell_ijk(F, q, i, j, k);
    int ci[2], cj[2], ck[2];
    float wi[2], wj[2], wk[2];
    axis_taps(i, F.fx, Cl.nx, ci, wi);
    axis_taps(j, F.fy, Cl.ny, cj, wj);
    axis_taps(k, F.fz, Cl.nz, ck, wk);
    float v = 0.f;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const float w = wi[a] * wj[e] * wk[c];
          if (w != 0.f) v += w * xc[lrow(Cl, ci[a], cj[e], ck[c])];
        }
    xf[q] += v;
  }
  __syncthreads();
}

// x_t = V-cycle of levels t..nlev-1 on b_t (both in global memory, level t >= 1)
__global__ void __launch_bounds__(1024) k_mg_tail(MgPlan mg, int t, const SolverScal *sc) {
  if (sc->done) return;
  extern __shared__ float sm[];
  const int n = mg.nlev;
  float *xs[kMgMaxLevels], *bs[kMgMaxLevels];
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
  {  // coarsest: x = 0, then red-black sweeps (k_mg_coarse)
    const MgLevel &C = mg.lev[n - 1];
    const int nc = C.nx * C.ny * C.nz;
    for (int q = threadIdx.x; q < nc; q += blockDim.x) xs[n - 1][q] = 0.f;
    __syncthreads();
    for (int s = 0; s < mg.coarse_sweeps; ++s) {
      blk_smooth(C, 0, 0, bs[n - 1], xs[n - 1]);
      blk_smooth(C, 1, 0, bs[n - 1], xs[n - 1]);
    }
  }
  for (int l = n - 2; l >= t; --l) {
    blk_prolong(mg.lev[l], mg.lev[l + 1], xs[l + 1], xs[l]);
    blk_smooth(mg.lev[l], 1, 0, bs[l], xs[l]);
    blk_smooth(mg.lev[l], 0, 0, bs[l], xs[l]);
  }
  for (int q = threadIdx.x; q < nt; q += blockDim.x) mg.lev[t].x[q] = xs[t][q];
}

static void level_geometry(MgLevel &L, int nsm, bool quads) {
  L.bx = 1;
  while (L.bx < L.nz && L.bx < 32) L.bx *= 2;
  L.by = kBlock / L.bx;
  L.gx = (L.nz + L.bx - 1) / L.bx;
  L.gy = (L.ny + L.by - 1) / L.by;
  L.gz = std::max(1, std::min(L.nx, nsm * 8 / std::max(1, L.gx * L.gy)));
  const long long nquads = (long long)L.nx * L.ny * (L.nz / 4);
  L.qgrid = quads && L.nz % 4 == 0 ? (int)std::max(1LL, std::min((nquads + kBlock - 1) / kBlock, 8LL * nsm)) : 0;
}

bool mg_plan(int nx, int ny, int nz, double hx, double hy, double hz, int nsm, bool quads, MgPlan *mg) {
  *mg = MgPlan{};
  int l = 0;
  for (;;) {
    MgLevel &L = mg->lev[l];
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.wx = (float)(1.0 / (hx * hx));
    L.wy = (float)(1.0 / (hy * hy));
    L.wz = (float)(1.0 / (hz * hz));
    level_geometry(L, nsm, quads);
    const long long cells = (long long)nx * ny * nz;
    const int fx = nx % 2 == 0 ? 2 : 1, fy = ny % 2 == 0 ? 2 : 1, fz = nz % 2 == 0 ? 2 : 1;
    if (cells <= kMgCoarseCells || fx * fy * fz == 1 || l + 1 == kMgMaxLevels) {
      L.fx = L.fy = L.fz = 1;
      break;
    }
    L.fx = fx;
    L.fy = fy;
    L.fz = fz;
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
    if (tail_cells > kMgTailCells) break;
    mg->tail = t;
  }
  const MgLevel &C = mg->lev[l];
  mg->coarse_sweeps = std::min(256, 16 + 2 * std::max(C.nx, std::max(C.ny, C.nz)));
  return (long long)C.nx * C.ny * C.nz <= kMgSharedCells;
}

// per level above the tail (or the coarsest): 2 smooths + restrict, prolong + 2 smooths;
// then one tail (or coarsest) kernel
int mg_vcycle_launches(const MgPlan &mg) {
  return mg.tail < mg.nlev ? 6 * mg.tail + 1 : 6 * (mg.nlev - 1) + 1;
}

void launch_mg_vcycle(cudaStream_t s, const MgPlan &mg, int jacobi, const float *b0, float *x0, const SolverScal *sc) {
  const int n = mg.nlev;
  auto B = [&](int l) -> const float * { return l == 0 ? b0 : mg.lev[l].b; };
  auto X = [&](int l) -> float * { return l == 0 ? x0 : mg.lev[l].x; };
  auto grid = [&](int l) { return dim3(mg.lev[l].gx, mg.lev[l].gy, mg.lev[l].gz); };
  auto block = [&](int l) { return dim3(mg.lev[l].bx, mg.lev[l].by, 1); };
  auto smooth = [&](int l, int colour, int zero) {
    if (mg.lev[l].qgrid > 0)
      k_mg_smooth4<<<mg.lev[l].qgrid, kBlock, 0, s>>>(mg.lev[l], colour, zero, l == 0 ? jacobi : 0, B(l), X(l), sc);
    else
      k_mg_smooth<<<grid(l), block(l), 0, s>>>(mg.lev[l], colour, zero, l == 0 ? jacobi : 0, B(l), X(l), sc);
  };
  const int m = std::min(mg.tail, n);  // levels m..n-1 run in one block (m < n), or none
  for (int l = 0; l + 1 < m; ++l) {
    smooth(l, 0, 1);
    smooth(l, 1, 0);
    k_mg_restrict<<<grid(l + 1), block(l + 1), 0, s>>>(mg.lev[l], mg.lev[l + 1], l == 0 ? jacobi : 0, B(l), X(l),
                                                         mg.lev[l + 1].b, sc);
  }
  if (m < n) {
    // levels m-1 -> m: smooth and restrict as above, then the tail
    smooth(m - 1, 0, 1);
    smooth(m - 1, 1, 0);
    k_mg_restrict<<<grid(m), block(m), 0, s>>>(mg.lev[m - 1], mg.lev[m], m == 1 ? jacobi : 0, B(m - 1), X(m - 1),
                                                 mg.lev[m].b, sc);
    size_t cells = 0;
    for (int l = m; l < n; ++l) cells += (size_t)mg.lev[l].nx * mg.lev[l].ny * mg.lev[l].nz;
    k_mg_tail<<<1, 1024, 2 * sizeof(float) * cells, s>>>(mg, m, sc);
  } else {
    const MgLevel &C = mg.lev[n - 1];
    const size_t smem = 2 * sizeof(float) * (size_t)C.nx * C.ny * C.nz;
    k_mg_coarse<<<1, 1024, smem, s>>>(C, mg.coarse_sweeps, n == 1 ? jacobi : 0, B(n - 1), X(n - 1), sc);
  }
  for (int l = (m < n ? m : n - 1) - 1; l >= 0; --l) {
    k_mg_prolong<<<grid(l), block(l), 0, s>>>(mg.lev[l], mg.lev[l + 1], X(l + 1), X(l), sc);
    smooth(l, 1, 0);
    smooth(l, 0, 0);
  }
}

}  // namespace cfdgb
