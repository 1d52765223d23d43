// scatter.cu -- group-to-group scattering and the isotropic source on GB300.
//
// Replaces Kernel::scattering (src/Kripke/Kernel/Scattering.cpp:59-100,
// 137-145) and Kernel::source (src/Kripke/Kernel/Source.cpp:57-76).
//   phi_out(nm,g,z) += sum_g' [sum_mix f * sigs(mat, l(nm), g, g')] * phi(nm,g',z)
// One thread owns a (zone, destination group) row and keeps all (L+1)^2 moment
// sums in registers; for each source group it forms the L+1 coefficients
// (one per Legendre order, shared by the 2l+1 moments of that order) exactly
// as the reference does -- the sum over the zone's mix elements of
// sigs*fraction, from 0 -- and applies them.  Source groups are visited in
// ascending order and only over the range where any material's matrix row is
// nonzero (adding an exact zero term leaves the sum unchanged).
// sigs is stored transposed, [mat][l][g'][g], so a warp's coefficient loads
// are contiguous.
#include "kgb_internal.h"

namespace kgb {

namespace {
constexpr int kScatThreads = 128;

__host__ __device__ constexpr int legendreOf(int m) {
  int l = 0;
  while ((l + 1) * (l + 1) <= m) ++l;
  return l;
}

// One (zone, destination group) row of phi_out; with SRC the isotropic source
// of material 0 is added to moment 0 afterwards, as Kernel::source does.
template <typename T, int LMAX, bool SRC>
__device__ __forceinline__ void scatterRow(const T *__restrict__ phi, T *__restrict__ phi_out,
                                           const T *__restrict__ sigsT, const ScatterArgsBase &a, int64_t r,
                                           bool accumulate, double q) {
  constexpr int MM = (LMAX + 1) * (LMAX + 1);
  const int Gd = a.dst_ghi - a.dst_glo;
  const int64_t zi = r / Gd;
  const int64_t z = a.zlist ? (int64_t)a.zlist[zi] : zi;
  const int g = a.dst_glo + (int)(r - zi * Gd);
  const int ms = a.zmix_start[z], mcnt = a.zmix_count[z];
  // a single-material zone has fraction exactly 1, where the reference's
  // 0 + sigs*fraction is sigs itself
  const bool pure = mcnt == 1 && a.mix_frac[ms] == 1.0;
  const int mat0 = a.mix_mat[ms];
  const int lo = max(a.gp_lo[g], a.src_glo);
  const int hi = min(a.gp_hi[g] + 1, a.src_ghi);
  T acc[MM];
#pragma unroll
  for (int m = 0; m < MM; ++m) acc[m] = T(0);
  for (int gp = lo; gp < hi; ++gp) {
    T sl[LMAX + 1];
    if (pure) {
#pragma unroll
      for (int l = 0; l <= LMAX; ++l) sl[l] = sigsT[(((int64_t)mat0 * (LMAX + 1) + l) * a.G + gp) * a.G + g];
    } else {
#pragma unroll
      for (int l = 0; l <= LMAX; ++l) sl[l] = T(0);
      for (int x = 0; x < mcnt; ++x) {
        const int mat = a.mix_mat[ms + x];
        const T f = (T)a.mix_frac[ms + x];
#pragma unroll
        for (int l = 0; l <= LMAX; ++l) sl[l] += sigsT[(((int64_t)mat * (LMAX + 1) + l) * a.G + gp) * a.G + g] * f;
      }
    }
    const T *ph = phi + (z * a.G + gp) * MM;
#pragma unroll
    for (int m = 0; m < MM; ++m) acc[m] += sl[legendreOf(m)] * ph[m];
  }
  T *o = phi_out + (z * a.G + g) * MM;
#pragma unroll
  for (int m = 0; m < MM; ++m) o[m] = accumulate ? o[m] + acc[m] : acc[m];
  if (SRC)
    for (int x = 0; x < mcnt; ++x)
      if (a.mix_mat[ms + x] == 0) o[0] += (T)(q * a.mix_frac[ms + x]);
}

template <typename T, int LMAX>
__global__ void __launch_bounds__(kScatThreads) scattering_kernel(const T *__restrict__ phi, T *__restrict__ phi_out,
                                                                 const T *__restrict__ sigsT, const ScatterArgsBase a,
                                                                 bool accumulate) {
  const int64_t rows = a.Z * (a.dst_ghi - a.dst_glo);
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
    scatterRow<T, LMAX, false>(phi, phi_out, sigsT, a, r, accumulate, 0.0);
}

// Batched scattering with the source fused: work items are row ranges of one
// problem each.
template <typename T, int LMAX>
__global__ void __launch_bounds__(kScatThreads) batch_scattering_kernel(const BatchScat<T> *__restrict__ inst,
                                                                       const BatchRows *__restrict__ items,
                                                                       int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const BatchRows w = items[it];
    const BatchScat<T> &b = inst[w.inst];
    for (int64_t r = w.r0 + threadIdx.x; r < w.r1; r += blockDim.x)
      scatterRow<T, LMAX, true>(b.phi, b.phi_out, b.sigsT, b.a, r, false, b.q);
  }
}

template <typename T>
__global__ void source_kernel(T *__restrict__ phi_out, int64_t nmix, const int *__restrict__ mix_zone,
                              const int *__restrict__ mix_mat, const double *__restrict__ mix_frac, int G, int M,
                              double strength) {
  const int64_t n = nmix * G;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t mix = t / G;
    const int g = (int)(t - mix * G);
    if (mix_mat[mix] == 0) {
      T *o = phi_out + ((int64_t)mix_zone[mix] * G + g) * M;  // moment 0
      *o += (T)(strength * mix_frac[mix]);
    }
  }
}

int gridFor(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = 152 * 16;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}
}  // namespace

template <typename T>
void launch_scattering(const T *phi, T *phi_out, const T *sigsT, const ScatterArgsBase &a, bool accumulate,
                       cudaStream_t s) {
  const int64_t rows = a.Z * (a.dst_ghi - a.dst_glo);
  const int grid = gridFor(rows, kScatThreads);
  switch (a.L) {
    case 0: scattering_kernel<T, 0><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
    case 1: scattering_kernel<T, 1><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
    case 2: scattering_kernel<T, 2><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
    case 3: scattering_kernel<T, 3><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
    case 4: scattering_kernel<T, 4><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
    case 5: scattering_kernel<T, 5><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
    case 6: scattering_kernel<T, 6><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
    default: scattering_kernel<T, 7><<<grid, kScatThreads, 0, s>>>(phi, phi_out, sigsT, a, accumulate); break;
  }
}

template <typename T>
void launch_source(T *phi_out, int64_t nmix, const int *mix_zone, const int *mix_mat, const double *mix_frac, int G,
                   int M, double strength, cudaStream_t s) {
  const int64_t n = nmix * G;
  if (n == 0) return;
  source_kernel<T><<<gridFor(n, 256), 256, 0, s>>>(phi_out, nmix, mix_zone, mix_mat, mix_frac, G, M, strength);
}

template <typename T>
void launch_batch_scattering(const BatchScat<T> *inst, const BatchRows *items, int nitems, int L, int grid,
                             cudaStream_t s) {
  if (nitems <= 0) return;
  switch (L) {
    case 0: batch_scattering_kernel<T, 0><<<grid, kScatThreads, 0, s>>>(inst, items, nitems); break;
    case 1: batch_scattering_kernel<T, 1><<<grid, kScatThreads, 0, s>>>(inst, items, nitems); break;
    case 2: batch_scattering_kernel<T, 2><<<grid, kScatThreads, 0, s>>>(inst, items, nitems); break;
    case 3: batch_scattering_kernel<T, 3><<<grid, kScatThreads, 0, s>>>(inst, items, nitems); break;
    default: batch_scattering_kernel<T, 4><<<grid, kScatThreads, 0, s>>>(inst, items, nitems); break;
  }
}

template void launch_batch_scattering<double>(const BatchScat<double> *, const BatchRows *, int, int, int,
                                              cudaStream_t);
template void launch_batch_scattering<float>(const BatchScat<float> *, const BatchRows *, int, int, int,
                                             cudaStream_t);
template void launch_scattering<double>(const double *, double *, const double *, const ScatterArgsBase &, bool, cudaStream_t);
template void launch_scattering<float>(const float *, float *, const float *, const ScatterArgsBase &, bool, cudaStream_t);
template void launch_source<double>(double *, int64_t, const int *, const int *, const double *, int, int, double, cudaStream_t);
template void launch_source<float>(float *, int64_t, const int *, const int *, const double *, int, int, double, cudaStream_t);

}  // namespace kgb
