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
#include <algorithm>

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

// Zone-blocked scattering of single-material zones (mixed form; groups <= 64,
// Legendre order <= 4).  Work items are runs of a material's zone list; a CTA
// keeps the material's transfer matrices ([l][g'][g], from sigsT) in shared
// memory and stages its zones' phi blocks ([g'][m] rows padded to a multiple
// of 4 floats, so the moment loads are 16-byte vectors).  A warp covers up to
// 32 destination groups of one zone (groups < 32: several zones, one per run of
// G lanes): each lane keeps all (L+1)^2 moment sums of its (zone, group) and
// walks the source groups over the warp's nonzero range; the matrix entries
// of a warp are contiguous and the phi entries of one zone are broadcast.
// Every lane sums the same terms in the same order as scattering_kernel (source
// groups ascending from 0; beyond its own nonzero range the coefficients are
// exact zeros), so the outputs are bit for bit that kernel's.  The outputs go
// back through the staging buffer as contiguous zone blocks.
constexpr int kBlkThreads = 256;

template <int LMAX>
__global__ void __launch_bounds__(kBlkThreads, 2)
    scatter_block_kernel(const float *__restrict__ phi, float *__restrict__ phi_out, const float *__restrict__ sigsT,
                         const int *__restrict__ zl, const __grid_constant__ ScatterBlockPlan pl, bool accumulate) {
  constexpr int MM = (LMAX + 1) * (LMAX + 1);
  constexpr int MP = (MM + 3) / 4 * 4;  // padded row of the staged blocks
  extern __shared__ __align__(16) float blk_smem[];
  const int G = pl.G, L1 = LMAX + 1;
  float *sS = blk_smem;                       // [L1][G][G]: S(l)[g' -> g] at (l * G + g') * G + g
  float *sB = blk_smem + (size_t)L1 * G * G;  // [zpc][G][MP]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Gw = G < 32 ? G : 32, zpw = 32 / Gw, gblocks = (G + 31) / 32;
  const int gb = warp % gblocks, zsub = lane / Gw;
  const int zc = (warp / gblocks) * zpw + zsub;  // zone of the chunk this lane serves
  const int g = gb * 32 + lane % Gw;
  const bool lane_ok = zsub < zpw && g < G;
  int lo = lane_ok ? pl.gp_lo[g] : G, hi = lane_ok ? pl.gp_hi[g] : -1;
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  int cur = -1;
  for (int64_t it = blockIdx.x; it < pl.items; it += gridDim.x) {
    // item -> (material, run of zones)
    int m = 0;
    int64_t first = it;
    while (m < 2 && first >= pl.nitems[m]) first -= pl.nitems[m++];
    const int64_t z0 = pl.off[m] + first * pl.zpc;
    const int nz = (int)min((int64_t)pl.zpc, pl.off[m + 1] - z0);
    if (m != cur) {  // this material's matrices
      __syncthreads();
      const float *src = sigsT + (size_t)m * L1 * G * G;
      for (int i = threadIdx.x; i < L1 * G * G; i += kBlkThreads) sS[i] = src[i];
      cur = m;
    }
    // the zones' phi blocks, contiguous [G][MM] in global memory, into padded rows
    const int n = G * MM;
    for (int c = 0; c < nz; ++c) {
      const float *src = phi + (int64_t)zl[z0 + c] * n;
      float *dst = sB + (size_t)c * G * MP;
      for (int e = threadIdx.x; e < n; e += kBlkThreads) {
        const int gp = e / MM;
        dst[gp * MP + (e - gp * MM)] = src[e];
      }
    }
    __syncthreads();
    float acc[MM];
#pragma unroll
    for (int k = 0; k < MM; ++k) acc[k] = 0.0f;
    if (lane_ok && zc < nz) {
      const float *pb = sB + (size_t)zc * G * MP;
      for (int gp = lo; gp <= hi; ++gp) {
        float sl[LMAX + 1];
#pragma unroll
        for (int l = 0; l <= LMAX; ++l) sl[l] = sS[(l * G + gp) * G + g];
        const float4 *pr = reinterpret_cast<const float4 *>(pb + gp * MP);
#pragma unroll
        for (int q = 0; q < MP / 4; ++q) {
          const float4 v = pr[q];
          const float pv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int k = 4 * q + u;
            if (k < MM) acc[k] += sl[legendreOf(k)] * pv[u];
          }
        }
      }
    }
    __syncthreads();  // every lane has read the staged blocks
    if (lane_ok && zc < nz) {
      float *ob = sB + ((size_t)zc * G + g) * MP;
#pragma unroll
      for (int k = 0; k < MM; ++k) ob[k] = acc[k];
    }
    __syncthreads();
    for (int c = 0; c < nz; ++c) {
      float *dst = phi_out + (int64_t)zl[z0 + c] * n;
      const float *src = sB + (size_t)c * G * MP;
      for (int e = threadIdx.x; e < n; e += kBlkThreads) {
        const int gp = e / MM;
        const float v = src[gp * MP + (e - gp * MM)];
        dst[e] = accumulate ? dst[e] + v : v;
      }
    }
    __syncthreads();  // the buffer is refilled by the next item
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

bool scatter_block_applies(int G, int L) { return G >= 1 && G <= 64 && L <= 4; }

size_t scatter_block_smem(int G, int L) {
  const int MM = (L + 1) * (L + 1), MP = (MM + 3) / 4 * 4;
  const int Gw = G < 32 ? G : 32, zpc = (kBlkThreads / 32) * (32 / Gw) / ((G + 31) / 32);
  return sizeof(float) * ((size_t)(L + 1) * G * G + (size_t)zpc * G * MP);
}

void launch_scatter_block(const float *phi, float *phi_out, const float *sigsT, const int *zl, const int64_t off[4],
                          int G, int L, const int *gp_lo, const int *gp_hi, bool accumulate, int nsm,
                          cudaStream_t s) {
  ScatterBlockPlan pl{};
  pl.G = G;
  const int Gw = G < 32 ? G : 32;
  pl.zpc = (kBlkThreads / 32) * (32 / Gw) / ((G + 31) / 32);
  pl.items = 0;
  for (int m = 0; m < 3; ++m) {
    pl.off[m] = off[m];
    pl.nitems[m] = (off[m + 1] - off[m] + pl.zpc - 1) / pl.zpc;
    pl.items += pl.nitems[m];
  }
  pl.off[3] = off[3];
  pl.gp_lo = gp_lo;
  pl.gp_hi = gp_hi;
  if (pl.items == 0) return;
  const size_t smem = scatter_block_smem(G, L);
  const int grid = (int)std::min<int64_t>(pl.items, (int64_t)2 * nsm);
  auto go = [&](auto kernel) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kernel<<<grid, kBlkThreads, smem, s>>>(phi, phi_out, sigsT, zl, pl, accumulate);
  };
  switch (L) {
    case 0: go(scatter_block_kernel<0>); break;
    case 1: go(scatter_block_kernel<1>); break;
    case 2: go(scatter_block_kernel<2>); break;
    case 3: go(scatter_block_kernel<3>); break;
    default: go(scatter_block_kernel<4>); break;
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
