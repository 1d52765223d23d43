// reduce.cu -- FP64 reductions of the source iteration on GB300.
//
// Kernel::population (src/Kripke/Kernel/Population.cpp:40-64,88-100):
//   sum over (d,g,z) of w(d) * psi(d,g,z) * volume(z)
// and the particle-balance terms (emission, collision, boundary leakage).
// Every reduction is two passes in a fixed order -- one partial per block
// written to a scratch array, then a single block sums the partials -- so
// results are bitwise reproducible run to run (the grid size is fixed).
#include "kgb_internal.h"

namespace kgb {

namespace {
constexpr int kRedThreads = 256;

__device__ __forceinline__ double blockSum(double v) {
  __shared__ double warp_part[kRedThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_part[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kRedThreads / 32; ++i) r += warp_part[i];
  __syncthreads();
  return r;
}

// One warp per (zone, group) row at a time, lanes over directions, so every
// load of the warp is one contiguous run of the row; each lane keeps its own
// volume-weighted partial, summed in the block's fixed order at the end.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) population_kernel(const T *__restrict__ psi, const double *__restrict__ w,
                                                                const double *__restrict__ vol, int64_t rows, int G,
                                                                int D, double *__restrict__ partials) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (int64_t r = warp0; r < rows; r += nwarps) {
    const T *p = psi + r * D;
    double s = 0.0;
    for (int d = lane; d < D; d += 32) s += w[d] * (double)p[d];
    acc += s * vol[r / G];
  }
  const double b = blockSum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// The same count from the moments: sum over (z,g) of scale * phi(0,g,z) * vol(z),
// with scale = w(d) / ell(0,d) (the quadrature's L has ell(0,d) proportional
// to w(d), so this equals the sum over d of w(d) psi(d,g,z)).
template <typename T>
__global__ void __launch_bounds__(kRedThreads) moment_population_kernel(const T *__restrict__ phi, int M,
                                                                       const double *__restrict__ vol, int64_t rows,
                                                                       int G, double scale,
                                                                       double *__restrict__ partials) {
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
    acc += (double)phi[r * M] * vol[r / G];
  const double b = blockSum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = b * scale;
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) balance_kernel(const T *__restrict__ psi, const T *__restrict__ rhs,
                                                             const T *__restrict__ sigt, const double *__restrict__ w,
                                                             const double *__restrict__ vol, int64_t rows, int G, int D,
                                                             double *__restrict__ partials) {
  double ae = 0.0, ac = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const T *p = psi + r * D;
    const T *q = rhs + r * D;
    double se = 0.0, sc = 0.0;
    for (int d = 0; d < D; ++d) {
      se += w[d] * (double)q[d];
      sc += w[d] * (double)p[d];
    }
    const double v = vol[r / G];
    ae += se * v;
    ac += sc * (double)sigt[r] * v;
  }
  const double be = blockSum(ae);
  const double bc = blockSum(ac);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = be;
    partials[2 * blockIdx.x + 1] = bc;
  }
}

// Outflow through one boundary plane chunk [nb][na][Gs][Ds]:
// sum of w(d) * |cos(d)| * wa(a) * wb(b) * plane.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) leakage_kernel(const T *__restrict__ plane, int64_t nelem, int Gs, int Ds,
                                                             int dlo, int na, const double *__restrict__ w,
                                                             const double *__restrict__ cosv,
                                                             const double *__restrict__ wa,
                                                             const double *__restrict__ wb,
                                                             double *__restrict__ partials) {
  double acc = 0.0;
  const int64_t nchain = (int64_t)Gs * Ds;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nelem; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = e / nchain;
    const int dl = (int)((e - cell * nchain) % Ds);
    const int64_t b = cell / na, a = cell - b * na;
    const int d = dlo + dl;
    acc += w[d] * cosv[d] * (wa[a] * wb[b]) * (double)plane[e];
  }
  const double bsum = blockSum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = bsum;
}

// Single block: out[k] (+)= sum over i of partials[i*stride + k], fixed order.
__global__ void __launch_bounds__(kRedThreads) finish_kernel(const double *__restrict__ partials, int n, int stride,
                                                            int k, double *__restrict__ out, bool add) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partials[(int64_t)i * stride + k];
  const double b = blockSum(acc);
  if (threadIdx.x == 0) out[0] = add ? out[0] + b : b;
}
// one block per problem: the finish_kernel sum of that problem's partials
__global__ void __launch_bounds__(kRedThreads) batch_pop_finish_kernel(const double *const *__restrict__ slots,
                                                                      const int64_t *__restrict__ n,
                                                                      double *__restrict__ out) {
  const double *p = slots[blockIdx.x];
  const int nn = (int)n[blockIdx.x];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) acc += p[i];
  const double b = blockSum(acc);
  if (threadIdx.x == 0) out[blockIdx.x] = b;
}
}  // namespace

template <typename T>
void launch_population(const T *psi, const double *w, const double *vol, int64_t rows, int G, int D, double *partials,
                       int nblocks, double *out, cudaStream_t s) {
  population_kernel<T><<<nblocks, kRedThreads, 0, s>>>(psi, w, vol, rows, G, D, partials);
  finish_kernel<<<1, kRedThreads, 0, s>>>(partials, nblocks, 1, 0, out, false);
}

template <typename T>
void launch_population_moments(const T *phi, int M, const double *vol, int64_t rows, int G, double scale,
                               double *partials, int nblocks, double *out, cudaStream_t s) {
  moment_population_kernel<T><<<nblocks, kRedThreads, 0, s>>>(phi, M, vol, rows, G, scale, partials);
  finish_kernel<<<1, kRedThreads, 0, s>>>(partials, nblocks, 1, 0, out, false);
}

template <typename T>
void launch_balance_terms(const T *psi, const T *rhs, const T *sigt, const double *w, const double *vol, int64_t rows,
                          int G, int D, double *partials, int nblocks, double *out2, cudaStream_t s) {
  balance_kernel<T><<<nblocks, kRedThreads, 0, s>>>(psi, rhs, sigt, w, vol, rows, G, D, partials);
  finish_kernel<<<1, kRedThreads, 0, s>>>(partials, nblocks, 2, 0, out2, false);
  finish_kernel<<<1, kRedThreads, 0, s>>>(partials, nblocks, 2, 1, out2 + 1, false);
}

template <typename T>
void launch_leakage(const T *plane, int64_t nelem, int Gs, int Ds, int dlo, int na, const double *w, const double *cosv,
                    const double *wa, const double *wb, double *partials, int nblocks, double *out, cudaStream_t s) {
  leakage_kernel<T><<<nblocks, kRedThreads, 0, s>>>(plane, nelem, Gs, Ds, dlo, na, w, cosv, wa, wb, partials);
  finish_kernel<<<1, kRedThreads, 0, s>>>(partials, nblocks, 1, 0, out, true);
}

void launch_batch_pop_finish(const double *const *slots, const int64_t *n, int ninst, double *out, cudaStream_t s) {
  if (ninst > 0) batch_pop_finish_kernel<<<ninst, kRedThreads, 0, s>>>(slots, n, out);
}

void launch_sum_partials(const double *partials, int64_t n, double *out, cudaStream_t s) {
  finish_kernel<<<1, kRedThreads, 0, s>>>(partials, (int)n, 1, 0, out, false);
}

template void launch_population<double>(const double *, const double *, const double *, int64_t, int, int, double *, int, double *, cudaStream_t);
template void launch_population<float>(const float *, const double *, const double *, int64_t, int, int, double *, int, double *, cudaStream_t);
template void launch_population_moments<double>(const double *, int, const double *, int64_t, int, double, double *,
                                                int, double *, cudaStream_t);
template void launch_population_moments<float>(const float *, int, const double *, int64_t, int, double, double *,
                                               int, double *, cudaStream_t);
template void launch_balance_terms<double>(const double *, const double *, const double *, const double *, const double *, int64_t, int, int, double *, int, double *, cudaStream_t);
template void launch_balance_terms<float>(const float *, const float *, const float *, const double *, const double *, int64_t, int, int, double *, int, double *, cudaStream_t);
template void launch_leakage<double>(const double *, int64_t, int, int, int, int, const double *, const double *, const double *, const double *, double *, int, double *, cudaStream_t);
template void launch_leakage<float>(const float *, int64_t, int, int, int, int, const double *, const double *, const double *, const double *, double *, int, double *, cudaStream_t);

}  // namespace kgb
