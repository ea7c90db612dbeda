// Device helpers of the two-stage deterministic reductions: every block writes its partial sums,
// takes a ticket, and the block that takes the last ticket adds the partials in block order. The
// result therefore does not depend on the order in which the blocks finish.
#pragma once

#include "common.cuh"

namespace ttgb {
namespace red {

constexpr int RT = 256;   // threads per reduction block

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum of one value per thread; result valid in thread 0
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Block sums of the first nv of N per-thread values with one barrier: each warp reduces its values
// by shuffles, then thread j < nv adds the warps' results (in warp order) and stores the block's
// sum at partial[(first + j) * G + blockIdx.x]. sh holds (blockDim.x / 32) * N doubles.
template <int N>
__device__ __forceinline__ void block_sums_to_partials(const double (&v)[N], int nv, double* sh,
                                                       double* partial, int first, int G) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    if (j < nv) {
      const double t = warp_sum(v[j]);
      if (lane == 0) sh[warp * N + j] = t;
    }
  }
  __syncthreads();
  if ((int)threadIdx.x < nv) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += sh[w * N + threadIdx.x];
    partial[(int64_t)(first + threadIdx.x) * G + blockIdx.x] = s;
  }
  __syncthreads();
}

// Called by every thread of every block after the block's partials are written. Returns true, in
// all threads of the block, only in the block that took the last ticket; that block then sees the
// partials of all the others. The caller of the last block resets the counter with reset_ticket().
__device__ __forceinline__ bool take_last_ticket(unsigned* counter) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(counter, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

__device__ __forceinline__ void reset_ticket(unsigned* counter) {
  if (threadIdx.x == 0) *counter = 0u;
}

// sum of partial[v * G + b] over b = 0..G-1, in block order (one thread)
__device__ __forceinline__ double sum_partials(const double* partial, int v, int G) {
  const volatile double* p = partial + (int64_t)v * G;
  double s = 0.0;
  for (int b = 0; b < G; ++b) s += p[b];
  return s;
}

// The same sum by one warp (all 32 lanes call it; the result is in every lane): lane l adds
// the blocks l, l + 32, ... in order, then the lanes' sums are combined by a fixed butterfly, so
// the result is the same on every run.
__device__ __forceinline__ double warp_sum_partials(const double* partial, int v, int G) {
  const volatile double* p = partial + (int64_t)v * G;
  double s = 0.0;
  for (int b = (int)(threadIdx.x & 31); b < G; b += 32) s += p[b];
  return warp_sum(s);
}

// Last-block epilogue for nvec sums of G partials each: out(v, sum) is called once per vector,
// by lane 0 of the warp that reduced it (warps take the vectors in turn).
template <typename F>
__device__ __forceinline__ void reduce_vectors(const double* partial, int nvec, int G, F out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int v = warp; v < nvec; v += nw) {
    const double s = warp_sum_partials(partial, v, G);
    if (lane == 0) out(v, s);
  }
}

}  // namespace red
}  // namespace ttgb
