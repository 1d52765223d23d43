// sweep_common.h -- pieces shared by the per-step sweep kernels (sweep.cu) and
// the streamed FP32 sweep (sweep_stream.cu), so both sum a tile's population
// partial in the same order with the same arithmetic.
#pragma once

#include "kgb_internal.h"

namespace kgb {
namespace {

// Compensated FP32 accumulator (Knuth TwoSum): the running error term keeps the
// sum of a tile's psi values accurate to FP64 level before it is widened.
struct F32Acc {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    const float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};
struct F64Acc {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};
template <typename T> struct AccOf;
template <> struct AccOf<double> { using type = F64Acc; };
template <> struct AccOf<float> { using type = F32Acc; };

__device__ __forceinline__ double blockSum128(double v) {
  __shared__ double part[kSweepThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kSweepThreads / 32; ++i) r += part[i];
  __syncthreads();  // part is reused by the block's next tile
  return r;
}

// The same for a block of any whole number of warps up to kSweepThreads (the
// streamed sweep's GB x Ds chains); with 128 threads it sums as blockSum128.
__device__ __forceinline__ double blockSumWarps(double v) {
  __shared__ double part[kSweepThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += part[i];
  __syncthreads();
  return r;
}

}  // namespace
}  // namespace kgb
