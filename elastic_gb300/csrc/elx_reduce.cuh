// Deterministic block and grid reductions used by the solver kernels: each
// block reduces its threads in a fixed tree, writes one partial per block,
// and the last block to arrive (atomic ticket) sums the partials in a fixed
// order.  Same grid, same inputs -> bitwise the same result.
#pragma once

#include <cstdint>

namespace elx {

constexpr int kThreads = 256;

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

// Block-wide sum of NV values (fixed order); result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double sh[NV][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; i++) {
    v[i] = warp_sum(v[i]);
    if (lane == 0) sh[i][w] = v[i];
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int i = 0; i < NV; i++) {
      double t = lane < kThreads / 32 ? sh[i][lane] : 0.0;
      v[i] = warp_sum(t);
    }
  }
}

// Block-wide sum of NV per-thread values of type T (float in the FP32
// kernels): the warp stage adds in T, the per-warp sums are widened to double
// and added in a fixed order.  Keeps the FP32 kernels off the (narrow) FP64
// pipe except for a handful of additions per block.  Result in thread 0.
template <int NV, class T>
__device__ __forceinline__ void block_sum_widen(const T (&v)[NV], double (&out)[NV]) {
  __shared__ double sh[NV][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; i++) {
    const T s = warp_sum(v[i]);
    if (lane == 0) sh[i][w] = (double)s;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < NV; i++) out[i] = 0.0;
  if (w == 0) {
#pragma unroll
    for (int i = 0; i < NV; i++) {
      double t = lane < kThreads / 32 ? sh[i][lane] : 0.0;
      out[i] = warp_sum(t);
    }
  }
}

// Writes this block's NV partials and returns true in thread 0 of the last
// block to arrive, after which that thread may read every block's partials.
template <int NV>
__device__ __forceinline__ bool publish_partials(const double (&v)[NV], double *partials,
                                                 unsigned int *counter) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; i++) partials[(size_t)i * gridDim.x + blockIdx.x] = v[i];
    __threadfence();
    const unsigned int ticket = atomicAdd(counter, 1u);
    last = ticket == gridDim.x - 1;
  }
  __syncthreads();
  return last;
}

// In the last block: every thread sums a strided slice of the partials, then
// a fixed tree; thread 0 gets the totals and resets the counter.
template <int NV>
__device__ __forceinline__ void gather_partials(double (&tot)[NV], const double *partials,
                                                unsigned int *counter) {
  __threadfence();
#pragma unroll
  for (int i = 0; i < NV; i++) {
    double s = 0.0;
    // L2 loads (__ldcg: the partials were written by other blocks, ordered by
    // the fence + ticket); several in flight per thread
#pragma unroll 4
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads)
      s += __ldcg(partials + (size_t)i * gridDim.x + b);
    tot[i] = s;
  }
  block_sum<NV>(tot);
  if (threadIdx.x == 0) *counter = 0u;
}


}  // namespace elx
