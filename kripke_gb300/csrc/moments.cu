// moments.cu -- discrete-to-moment (LTimes) and moment-to-discrete
// (LPlusTimes) transforms on GB300, SIMT form.
//
// Replaces Kernel::LTimes (src/Kripke/Kernel/LTimes.cpp:54-65) and
// Kernel::LPlusTimes (src/Kripke/Kernel/LPlusTimes.cpp:49-60).  With the
// device nesting psi[z][g][d], phi[z][g][m], both are one small matrix
// product per (zone, group) row against the shared L / L+ matrix, which sits in
// shared memory and is read as a broadcast.  Summation runs over directions
// (LTimes) or moments (LPlusTimes) in ascending order, as the reference loops.
#include "kgb_internal.h"

namespace kgb {

namespace {
constexpr int kMomThreads = 128;

template <typename T, int MB>
__global__ void __launch_bounds__(kMomThreads) ltimes_kernel(const T *__restrict__ psi, T *__restrict__ phi,
                                                            const T *__restrict__ ell_dm, int64_t rows, int D,
                                                            int M, int m0, int mc, bool accumulate) {
  extern __shared__ unsigned char smem_raw[];
  T *sell = reinterpret_cast<T *>(smem_raw);  // [D][MB]
  for (int i = threadIdx.x; i < D * MB; i += blockDim.x) {
    const int d = i / MB, m = i - d * MB;
    sell[i] = (m < mc) ? ell_dm[(int64_t)d * M + m0 + m] : T(0);
  }
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    T acc[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) acc[m] = T(0);
    const T *p = psi + r * D;
    for (int d = 0; d < D; ++d) {
      const T v = p[d];
      const T *e = sell + d * MB;
#pragma unroll
      for (int m = 0; m < MB; ++m) acc[m] += e[m] * v;
    }
    T *o = phi + r * M + m0;
#pragma unroll
    for (int m = 0; m < MB; ++m)
      if (m < mc) o[m] = accumulate ? o[m] + acc[m] : acc[m];
  }
}

template <typename T, int MB>
__global__ void __launch_bounds__(kMomThreads) lplustimes_kernel(const T *__restrict__ phi_out, T *__restrict__ rhs,
                                                                const T *__restrict__ ellp_dm, int64_t rows, int D,
                                                                int M, bool accumulate) {
  extern __shared__ unsigned char smem_raw[];
  T *sel = reinterpret_cast<T *>(smem_raw);  // [D][MB]
  for (int i = threadIdx.x; i < D * MB; i += blockDim.x) {
    const int d = i / MB, m = i - d * MB;
    sel[i] = (m < M) ? ellp_dm[(int64_t)d * M + m] : T(0);
  }
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    T po[MB];
    const T *src = phi_out + r * M;
#pragma unroll
    for (int m = 0; m < MB; ++m) po[m] = (m < M) ? src[m] : T(0);
    T *o = rhs + r * D;
    for (int d = 0; d < D; ++d) {
      const T *e = sel + d * MB;
      T acc = T(0);
#pragma unroll
      for (int m = 0; m < MB; ++m) acc += e[m] * po[m];
      o[d] = accumulate ? o[d] + acc : acc;
    }
  }
}

int gridFor(int64_t rows) {
  int64_t b = (rows + kMomThreads - 1) / kMomThreads;
  const int64_t cap = 152 * 16;  // grid-stride beyond 16 resident blocks per SM
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}
}  // namespace

template <typename T>
void launch_ltimes(const T *psi, T *phi, const T *ell_dm, int64_t rows, int D, int M, bool accumulate, cudaStream_t s) {
  constexpr int MB = 32;
  for (int m0 = 0; m0 < M; m0 += MB) {
    const int mc = (M - m0) < MB ? (M - m0) : MB;
    const size_t smem = sizeof(T) * (size_t)D * MB;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(ltimes_kernel<T, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    ltimes_kernel<T, MB><<<gridFor(rows), kMomThreads, smem, s>>>(psi, phi, ell_dm, rows, D, M, m0, mc, accumulate);
  }
}

template <typename T>
void launch_lplustimes(const T *phi_out, T *rhs, const T *ellp_dm, int64_t rows, int D, int M, bool accumulate,
                       cudaStream_t s) {
  if (M <= 32) {
    const size_t smem = sizeof(T) * (size_t)D * 32;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(lplustimes_kernel<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    lplustimes_kernel<T, 32><<<gridFor(rows), kMomThreads, smem, s>>>(phi_out, rhs, ellp_dm, rows, D, M, accumulate);
  } else {
    const size_t smem = sizeof(T) * (size_t)D * 64;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(lplustimes_kernel<T, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    lplustimes_kernel<T, 64><<<gridFor(rows), kMomThreads, smem, s>>>(phi_out, rhs, ellp_dm, rows, D, M, accumulate);
  }
}

template void launch_ltimes<double>(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t);
template void launch_ltimes<float>(const float *, float *, const float *, int64_t, int, int, bool, cudaStream_t);
template void launch_lplustimes<double>(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t);
template void launch_lplustimes<float>(const float *, float *, const float *, int64_t, int, int, bool, cudaStream_t);

}  // namespace kgb
