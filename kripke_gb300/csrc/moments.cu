// moments.cu -- discrete-to-moment (LTimes) and moment-to-discrete
// (LPlusTimes) transforms on GB300, SIMT form.
//
// Replaces Kernel::LTimes (src/Kripke/Kernel/LTimes.cpp:54-65) and
// Kernel::LPlusTimes (src/Kripke/Kernel/LPlusTimes.cpp:49-60).  With the
// device nesting psi[z][g][d], phi[z][g][m], both are one small matrix
// product per (zone, group) row against the shared L / L+ matrix, which sits in
// shared memory and is read as a broadcast, 16 bytes per load.  Summation runs
// over directions (LTimes) or moments (LPlusTimes) in ascending order, as the
// reference loops.
#include "kgb_internal.h"

namespace kgb {

namespace {
constexpr int kMomThreads = 128;

// 16-byte vector of T
template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };

template <typename T>
__device__ __forceinline__ void load16(T (&dst)[Vec16<T>::n], const T *src) {
  *reinterpret_cast<typename Vec16<T>::type *>(dst) = *reinterpret_cast<const typename Vec16<T>::type *>(src);
}
template <typename T>
__device__ __forceinline__ void store16(T *dst, const T (&src)[Vec16<T>::n]) {
  *reinterpret_cast<typename Vec16<T>::type *>(dst) = *reinterpret_cast<const typename Vec16<T>::type *>(src);
}

// VEC: every psi row starts on a 16-byte boundary (D*sizeof(T) % 16 == 0).
template <typename T, int MB, bool VEC>
__global__ void __launch_bounds__(kMomThreads) ltimes_kernel(const T *__restrict__ psi, T *__restrict__ phi,
                                                            const T *__restrict__ ell_dm, int64_t rows, int D,
                                                            int M, int m0, int mc, bool accumulate) {
  constexpr int V = Vec16<T>::n;
  extern __shared__ __align__(16) unsigned char smem_raw[];
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
    const int dv = VEC ? D - D % V : 0;
    for (int d0 = 0; d0 < dv; d0 += V) {
      T pv[V];
      load16(pv, p + d0);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const T *e = sell + (d0 + v) * MB;
#pragma unroll
        for (int m = 0; m < MB; m += V) {
          T ev[V];
          load16(ev, e + m);
#pragma unroll
          for (int u = 0; u < V; ++u) acc[m + u] += ev[u] * pv[v];
        }
      }
    }
    for (int d = dv; d < D; ++d) {
      const T pd = p[d];
      const T *e = sell + d * MB;
#pragma unroll
      for (int m = 0; m < MB; m += V) {
        T ev[V];
        load16(ev, e + m);
#pragma unroll
        for (int u = 0; u < V; ++u) acc[m + u] += ev[u] * pd;
      }
    }
    T *o = phi + r * M + m0;
#pragma unroll
    for (int m = 0; m < MB; ++m)
      if (m < mc) o[m] = accumulate ? o[m] + acc[m] : acc[m];
  }
}

template <typename T, int MB, bool VEC>
__global__ void __launch_bounds__(kMomThreads) lplustimes_kernel(const T *__restrict__ phi_out, T *__restrict__ rhs,
                                                                const T *__restrict__ ellp_dm, int64_t rows, int D,
                                                                int M, bool accumulate) {
  constexpr int V = Vec16<T>::n;
  extern __shared__ __align__(16) unsigned char smem_raw[];
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
    const int dv = VEC ? D - D % V : 0;
    for (int d0 = 0; d0 < dv; d0 += V) {
      T out[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const T *e = sel + (d0 + v) * MB;
        T acc = T(0);
#pragma unroll
        for (int m = 0; m < MB; m += V) {
          T ev[V];
          load16(ev, e + m);
#pragma unroll
          for (int u = 0; u < V; ++u) acc += ev[u] * po[m + u];
        }
        out[v] = acc;
      }
      if (accumulate) {
        T old[V];
        load16(old, o + d0);
#pragma unroll
        for (int v = 0; v < V; ++v) out[v] = old[v] + out[v];
      }
      store16(o + d0, out);
    }
    for (int d = dv; d < D; ++d) {
      const T *e = sel + d * MB;
      T acc = T(0);
#pragma unroll
      for (int m = 0; m < MB; m += V) {
        T ev[V];
        load16(ev, e + m);
#pragma unroll
        for (int u = 0; u < V; ++u) acc += ev[u] * po[m + u];
      }
      o[d] = accumulate ? o[d] + acc : acc;
    }
  }
}

int gridFor(int64_t rows) {
  int64_t b = (rows + kMomThreads - 1) / kMomThreads;
  const int64_t cap = 152 * 16;  // grid-stride beyond 16 resident blocks per SM
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

template <typename K>
void setSmem(K kernel, size_t smem) {
  if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
}  // namespace

// Moment-count instances: M = (L+1)^2 rounded up to a multiple of the 16-byte
// vector width, so at most one vector of padding is multiplied.
template <typename T, template <typename, int> class Launch>
void byMoments(int M, Launch<T, 4> l4, Launch<T, 12> l12, Launch<T, 16> l16, Launch<T, 28> l28, Launch<T, 36> l36,
               Launch<T, 52> l52, Launch<T, 64> l64) {
  if (M <= 4) l4();
  else if (M <= 12) l12();
  else if (M <= 16) l16();
  else if (M <= 28) l28();
  else if (M <= 36) l36();
  else if (M <= 52) l52();
  else l64();
}

template <typename T, int MB>
struct LPlusLaunch {
  const T *phi_out; T *rhs; const T *ellp; int64_t rows; int D, M; bool acc; cudaStream_t s;
  void operator()() const {
    // FP32 computes a 16-byte vector of directions per pass; FP64 (FP64-pipe bound) one at a time
    const bool vec = sizeof(T) == 4 && (D * sizeof(T)) % 16 == 0;
    const size_t smem = sizeof(T) * (size_t)D * MB;
    if (vec) {
      setSmem(lplustimes_kernel<T, MB, true>, smem);
      lplustimes_kernel<T, MB, true><<<gridFor(rows), kMomThreads, smem, s>>>(phi_out, rhs, ellp, rows, D, M, acc);
    } else {
      setSmem(lplustimes_kernel<T, MB, false>, smem);
      lplustimes_kernel<T, MB, false><<<gridFor(rows), kMomThreads, smem, s>>>(phi_out, rhs, ellp, rows, D, M, acc);
    }
  }
};

template <typename T, int MB>
struct LTimesLaunch {
  const T *psi; T *phi; const T *ell; int64_t rows; int D, M; bool acc; cudaStream_t s;
  void operator()() const {
    const bool vec = (D * sizeof(T)) % 16 == 0;
    const size_t smem = sizeof(T) * (size_t)D * MB;
    if (vec) {
      setSmem(ltimes_kernel<T, MB, true>, smem);
      ltimes_kernel<T, MB, true><<<gridFor(rows), kMomThreads, smem, s>>>(psi, phi, ell, rows, D, M, 0, M, acc);
    } else {
      setSmem(ltimes_kernel<T, MB, false>, smem);
      ltimes_kernel<T, MB, false><<<gridFor(rows), kMomThreads, smem, s>>>(psi, phi, ell, rows, D, M, 0, M, acc);
    }
  }
};

template <typename T>
void launch_ltimes(const T *psi, T *phi, const T *ell_dm, int64_t rows, int D, int M, bool accumulate, cudaStream_t s) {
#define KGB_L(MBV) LTimesLaunch<T, MBV>{psi, phi, ell_dm, rows, D, M, accumulate, s}
  byMoments<T, LTimesLaunch>(M, KGB_L(4), KGB_L(12), KGB_L(16), KGB_L(28), KGB_L(36), KGB_L(52), KGB_L(64));
#undef KGB_L
}

template <typename T>
void launch_lplustimes(const T *phi_out, T *rhs, const T *ellp_dm, int64_t rows, int D, int M, bool accumulate,
                       cudaStream_t s) {
#define KGB_L(MBV) LPlusLaunch<T, MBV>{phi_out, rhs, ellp_dm, rows, D, M, accumulate, s}
  byMoments<T, LPlusLaunch>(M, KGB_L(4), KGB_L(12), KGB_L(16), KGB_L(28), KGB_L(36), KGB_L(52), KGB_L(64));
#undef KGB_L
}

template void launch_ltimes<double>(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t);
template void launch_ltimes<float>(const float *, float *, const float *, int64_t, int, int, bool, cudaStream_t);
template void launch_lplustimes<double>(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t);
template void launch_lplustimes<float>(const float *, float *, const float *, int64_t, int, int, bool, cudaStream_t);

}  // namespace kgb
