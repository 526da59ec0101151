// Deterministic two-stage FP64 reductions for kernels with a fixed grid (1-D or 3-D
// blocks of kBlock threads).
//
// Stage 1: each block reduces its NV per-thread values (warp shuffles + shared memory)
// and stores them to part[q * nblocks + block].  Stage 2: the last block to finish (atomic
// ticket) sums the partials in a fixed order, so results do not depend on block
// scheduling.  No block ever waits on another.
#pragma once

#include "cfdgb_internal.cuh"

namespace cfdgb {

__device__ __forceinline__ int lin_tid() { return (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int lin_bid() { return (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x; }
__device__ __forceinline__ int nblocks() { return gridDim.x * gridDim.y * gridDim.z; }

template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV]) {
#pragma unroll
  for (int q = 0; q < NV; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
}

// Reduce v over the block (whole warps, at most 32 of them); the result is valid in
// thread 0 only.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double sh[NV][32];
  const int t = lin_tid();
  const int lane = t & 31, wid = t >> 5;
  const int nw = (int)(blockDim.x * blockDim.y * blockDim.z) >> 5;
  warp_sum<NV>(v);
  __syncthreads();  // sh may still be read by a previous call
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) sh[q][wid] = v[q];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = lane < nw ? sh[q][lane] : 0.0;
    warp_sum<NV>(v);
  }
}

// Stage 1 + 2.  Returns true in every thread of the last block; out[] is then valid in
// all of its threads.  *ticket is reset for the next launch.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *part, unsigned *ticket,
                                         double (&out)[NV]) {
  __shared__ bool last;
  __shared__ double res[NV];
  block_sum<NV>(v);
  const int G = nblocks(), t = lin_tid();
  if (t == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) part[q * G + lin_bid()] = v[q];
    __threadfence();
    last = (atomicAdd(ticket, 1u) == (unsigned)(G - 1));
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double w[NV];
  const int nt = (int)(blockDim.x * blockDim.y * blockDim.z);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double s = 0.0;
    for (int b = t; b < G; b += nt) s += __ldcg(part + q * G + b);
    w[q] = s;
  }
  block_sum<NV>(w);
  if (t == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) res[q] = w[q];
    *ticket = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) out[q] = res[q];
  return true;
}

// Grid-wide maxima of NV values per thread, with the same last-block pattern as grid_sum
// (minima: pass the negated values).  Maxima are exact, so the result does not depend on
// the order either.
template <int NV>
__device__ __forceinline__ bool grid_max(double (&v)[NV], double *part, unsigned *ticket, double (&out)[NV]) {
  __shared__ double sh[NV][kBlock / 32];
  __shared__ bool last;
  __shared__ double res[NV];
  const int t = lin_tid(), lane = t & 31, wid = t >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[q] = fmax(v[q], __shfl_down_sync(0xffffffffu, v[q], off));
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) sh[q][wid] = v[q];
  __syncthreads();
  const int G = nblocks();
  if (t == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double m = sh[q][0];
      for (int w = 1; w < kBlock / 32; ++w) m = fmax(m, sh[q][w]);
      part[q * G + lin_bid()] = m;
    }
    __threadfence();
    last = (atomicAdd(ticket, 1u) == (unsigned)(G - 1));
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // the partials, strided over the block's threads, then over its warps (every thread of
  // the block takes part: a one-thread loop over the partials held the grid for a long tail)
  const int nt = (int)(blockDim.x * blockDim.y * blockDim.z);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double m = -INFINITY;
    for (int b = t; b < G; b += nt) m = fmax(m, __ldcg(part + q * G + b));
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
    v[q] = m;
  }
  __syncthreads();  // sh is reused below
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) sh[q][wid] = v[q];
  __syncthreads();
  if (t == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double m = sh[q][0];
      for (int w = 1; w < nt / 32; ++w) m = fmax(m, sh[q][w]);
      res[q] = m;
    }
    *ticket = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) out[q] = res[q];
  return true;
}

// FP32 products summed in short FP32 runs, each run added into an FP64 accumulator:
// global sums stay FP64 while the per-element work stays FP32.
struct AccF {
  double d = 0.0;
  float f = 0.0f;
  int n = 0;
  __device__ __forceinline__ void add(float x) {
    f += x;
    if (++n == 8) { d += (double)f; f = 0.0f; n = 0; }
  }
  __device__ __forceinline__ double get() const { return d + (double)f; }
};
// Compensated FP32 dot product (Ogita, Rump and Oishi's Dot2: the error-free product by
// FMA and Knuth's TwoSum): as accurate as a dot product in twice the working precision,
// at a few FP32 operations per term.
struct Dot2F {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);  // a*b - p exactly
    const float s = hi + p;
    const float bp = s - hi;
    const float se = (hi - (s - bp)) + (p - bp);  // hi + p - s exactly
    hi = s;
    lo += pe + se;
  }
  __device__ __forceinline__ double get() const { return (double)hi + (double)lo; }
};
// Plain FP32 running sum of products for the vectorised kernels: a thread covers a few
// dozen quads, and the sum over threads is FP64 (grid_sum).
struct SumF {
  float f = 0.0f;
  __device__ __forceinline__ void add(float a, float b) { f = fmaf(a, b, f); }
  __device__ __forceinline__ double get() const { return (double)f; }
};
struct AccD {
  double d = 0.0;
  __device__ __forceinline__ void add(double x) { d += x; }
  __device__ __forceinline__ double get() const { return d; }
};
template <typename T> struct AccFor;
template <> struct AccFor<double> { using type = AccD; };
template <> struct AccFor<float> { using type = AccF; };

}  // namespace cfdgb
