// peak_probe.cu -- FP64 / FP32 FMA and divide issue rates of the current GPU.
//
// The plain form of the source iteration is bound by the FP64 pipe, whose
// rate is not among the measured peaks (HBM copy, bf16 GEMM), so the
// benchmark measures it with this probe: independent FMA chains per thread
// on a grid of 8 blocks per SM, timed with CUDA events.  Prints one JSON line.
// Every thread writes exactly one output element.
#include <cstdio>
#include <cuda_runtime.h>

template <typename T, int CH>
__global__ void fma_chains(T *out, int iters, T a, T b) {
  T x[CH];
  for (int c = 0; c < CH; ++c) x[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = x[c] * a + b;
  }
  T s = 0;
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T, int CH>
__global__ void div_chains(T *out, int iters, T a) {
  T x[CH];
  for (int c = 0; c < CH; ++c) x[c] = (T)(threadIdx.x + c + 1);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = a / (x[c] + (T)1.5);
  }
  T s = 0;
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename K>
float timeIt(K k) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;  // first launch is a warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

int main() {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) return 1;
  const int blocks = p.multiProcessorCount * 8, threads = 256, iters = 4096;
  double *dd = nullptr;
  float *df = nullptr;
  if (cudaMalloc(&dd, sizeof(double) * blocks * threads) != cudaSuccess) return 1;
  if (cudaMalloc(&df, sizeof(float) * blocks * threads) != cudaSuccess) return 1;
  const double n = (double)blocks * threads;
  float t64 = timeIt([&] { fma_chains<double, 8><<<blocks, threads>>>(dd, iters, 0.999, 0.001); });
  float d64 = timeIt([&] { div_chains<double, 4><<<blocks, threads>>>(dd, iters / 4, 3.0); });
  float t32 = timeIt([&] { fma_chains<float, 8><<<blocks, threads>>>(df, iters * 8, 0.999f, 0.001f); });
  float d32 = timeIt([&] { div_chains<float, 4><<<blocks, threads>>>(df, iters, 3.0f); });
  const cudaError_t e = cudaDeviceSynchronize();
  printf("{\"device\": \"%s\", \"sms\": %d, \"fp64_fma_gflops\": %.1f, \"fp64_div_gdiv\": %.2f, "
         "\"fp32_fma_gflops\": %.1f, \"fp32_div_gdiv\": %.2f, \"status\": \"%s\"}\n",
         p.name, p.multiProcessorCount, 2.0 * 8 * iters * n / t64 / 1e6, 4.0 * (iters / 4) * n / d64 / 1e6,
         2.0 * 8 * iters * 8 * n / t32 / 1e6, 4.0 * iters * n / d32 / 1e6, cudaGetErrorString(e));
  cudaFree(dd);
  cudaFree(df);
  return e == cudaSuccess ? 0 : 1;
}
