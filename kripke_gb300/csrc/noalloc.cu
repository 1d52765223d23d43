// noalloc.cu -- a population edit that allocates nothing.
//
// Some callers cannot call cudaMalloc when they need the particle count: a
// host framework that has reserved all device memory up front for its own pool
// allocator (a cudaMalloc would fail or fragment that pool), or a
// latency-bound control loop where an allocation's implicit device
// synchronisation is not acceptable.  For them
// kgb_population_noalloc computes the same sum as kgb_population (sum over
// d, g, z of w(d) * psi(d,g,z) * volume(z), FP64) from device arrays the caller
// owns, using a fixed scratch array that lives in this file's device image.
//
// Scratch: g_noalloc_partials, kNoallocMaxPartials doubles (128 KiB).  Each
// partial sums kNoallocRowsPerPartial (zone, group) rows, so at most
// kNoallocMaxPartials * kNoallocRowsPerPartial = 33,554,432 rows (zones x
// groups) per call; larger problems are rejected.  Every GPU that loads the
// library holds the array until the process exits.  All calls share it and it
// keeps the last call's contents; a call writes every slot it later reads, so
// nothing has to start at zero, but two calls that overlap on the GPU race on
// it.
//
// Host code cannot use the array's name as a device address, so the first
// call on each device (with that device current) looks it up with
// cudaGetSymbolAddress and caches it; that first call should come before any
// stream capture.  The address belongs to the device's primary context: a
// cudaDeviceReset ends that context, and the cached address with it, so a
// process that resets a device must not call this function on it afterwards.
#include <cstdio>
#include <mutex>

#include "kgb.h"

namespace {

constexpr int kNoallocMaxPartials = 16384;
constexpr int64_t kNoallocRowsPerPartial = 2048;
constexpr int kNoallocThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoallocMaxPartials];

std::mutex g_setup_mu;
double *g_scratch[kMaxDevices] = {};

__device__ __forceinline__ double blockSumOrdered(double v) {
  __shared__ double part[kNoallocThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kNoallocThreads / 32; ++i) r += part[i];
  return r;
}

// Block b sums rows [b*R, (b+1)*R) of the psi array [rows][D] (device nesting
// [zone][group][direction]) into partials[b].
__global__ void __launch_bounds__(kNoallocThreads)
noalloc_rows(const double *__restrict__ psi, const double *__restrict__ w, const double *__restrict__ vol,
             int64_t rows, int G, int D, double *__restrict__ partials) {
  const int64_t r0 = (int64_t)blockIdx.x * kNoallocRowsPerPartial;
  const int64_t r1 = min(rows, r0 + kNoallocRowsPerPartial);
  double acc = 0.0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += kNoallocThreads) {
    const double *p = psi + r * D;
    double s = 0.0;
    for (int d = 0; d < D; ++d) s += w[d] * p[d];
    acc += s * vol[r / G];
  }
  const double b = blockSumOrdered(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

__global__ void __launch_bounds__(kNoallocThreads)
noalloc_finish(const double *__restrict__ partials, int n, double *__restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kNoallocThreads) acc += partials[i];
  const double b = blockSumOrdered(acc);
  if (threadIdx.x == 0) *out = b;
}

void setError(char *err, int32_t len, const char *msg) {
  if (err && len > 0) std::snprintf(err, (size_t)len, "%s", msg);
}

}  // namespace

extern "C" int kgb_population_noalloc(const double *psi, const double *w, const double *volume, int64_t zones,
                                      int32_t groups, int32_t directions, double *out, void *stream, char *err,
                                      int32_t err_len) {
  if (!psi || !w || !volume || !out || zones < 1 || groups < 1 || directions < 1) {
    setError(err, err_len, "kgb_population_noalloc: null pointer or non-positive size");
    return KGB_ERR_ARG;
  }
  const int64_t limit = (int64_t)kNoallocMaxPartials * kNoallocRowsPerPartial;
  if (zones > limit / groups) {  // checked before the product, which could overflow
    char msg[240];
    std::snprintf(msg, sizeof msg,
                  "kgb_population_noalloc: zones*groups = %lld*%d exceeds the %lld-row limit of its static scratch",
                  (long long)zones, (int)groups, (long long)limit);
    setError(err, err_len, msg);
    return KGB_ERR_ARG;
  }
  const int64_t rows = zones * (int64_t)groups;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    setError(err, err_len, "kgb_population_noalloc: no usable current device");
    return KGB_ERR_CUDA;
  }
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch[dev]) {
      double *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_partials);
      if (e != cudaSuccess || !p) {
        setError(err, err_len, "kgb_population_noalloc: cudaGetSymbolAddress of the scratch array failed");
        return KGB_ERR_CUDA;
      }
      g_scratch[dev] = p;
    }
    scratch = g_scratch[dev];
  }
  const int nparts = (int)((rows + kNoallocRowsPerPartial - 1) / kNoallocRowsPerPartial);
  cudaStream_t s = (cudaStream_t)stream;
  noalloc_rows<<<nparts, kNoallocThreads, 0, s>>>(psi, w, volume, rows, groups, directions, scratch);
  noalloc_finish<<<1, kNoallocThreads, 0, s>>>(scratch, nparts, out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    setError(err, err_len, cudaGetErrorString(e));
    return KGB_ERR_CUDA;
  }
  return KGB_OK;
}
