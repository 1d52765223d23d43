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

#include "fp32_pair.h"
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
  float *sS = blk_smem;  // [L1][G][G]: S(l)[g' -> g] at (l * G + g') * G + g
  // [zpc][G][MP], after the matrices rounded up to whole float4s (the rows are read as float4)
  float *sB = blk_smem + ((size_t)L1 * G * G + 3) / 4 * 4;
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

// Staged zone-blocked scattering (groups a multiple of 4, at most 64; Legendre
// order <= 4).  A CTA holds one material's transfer matrices ([l][g'][g]) and
// runs kZoneGroups independent groups of kZoneGroup threads (each single-
// buffered: while one waits for its copy the others compute).  A group's item is a run of zpi zones
// of that material: one elected thread brings each zone's contiguous [G][MM]
// phi block into the group's buffer with one bulk copy (an mbarrier counts the
// bytes); a thread then owns 4 destination groups x MM moments of one zone in
// registers.  A warp covers at most 8 group quads of each of its zw zones (with
// 64 groups, two warps split a zone's quads), so its source-group range is that
// of its own destination groups -- with downscatter the low groups' warps stop
// early -- and its matrix loads are one 128-byte row.  It walks the source
// groups g' over its warp's nonzero range, in
// steps of 4 so that the offset of row g' within its 16-byte word is a
// compile-time constant (rows are MM floats; (MM g') mod 4 depends on g' mod 4
// only): a row is read as 16-byte broadcasts, a matrix row as one 16-byte load
// per Legendre order.  Each output keeps scattering_kernel's sum -- source
// groups ascending from 0, exact zeros outside a row's nonzero range -- so the
// results are bit for bit that kernel's.  The group's 4 x MM outputs of a
// thread are contiguous in phi_out and 16-byte aligned, stored (or added to,
// one FP32 add per element) as 16-byte words, while the next item's copies are
// in flight.
constexpr int kZoneThreads = 256;
constexpr int kZoneGroup = 64;                         // threads of one group
constexpr int kZoneGroups = kZoneThreads / kZoneGroup;  // independent groups per CTA
constexpr uint64_t kZoneWaitNs = 200000000ull;  // 0.2 s

__device__ __forceinline__ uint64_t zoneNowNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool zoneTestWait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// bounded wait for the phase with the given parity (false: gave up after kZoneWaitNs)
__device__ __forceinline__ bool zoneWait(uint32_t bar, uint32_t parity) {
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 15u) == 15u) {
      const uint64_t t = zoneNowNs();
      if (t0 == 0) t0 = t;
      else if (t - t0 > kZoneWaitNs) return false;
    }
  }
}

template <int LMAX>
__global__ void __launch_bounds__(kZoneThreads, 1)
    scatter_zone_kernel(const float *__restrict__ phi, float *__restrict__ phi_out, const float *__restrict__ sigsT,
                        const int *__restrict__ zl, const __grid_constant__ ScatterZonePlan pl, bool accumulate) {
  constexpr int MM = (LMAX + 1) * (LMAX + 1), L1 = LMAX + 1;
  extern __shared__ __align__(16) float zone_smem[];
  __shared__ __align__(8) uint64_t full[kZoneGroups];
  __shared__ int bad[kZoneGroups];
  const int G = pl.G, GQ = G / 4, zpi = pl.zpi;
  float *sS = zone_smem;  // [L1][G][G]
  const int tid = threadIdx.x, gi = tid / kZoneGroup, gt = tid % kZoneGroup;
  float *buf = zone_smem + (size_t)L1 * G * G + (size_t)gi * zpi * pl.slot;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&full[gi]);
  // warp -> (row of zw zones, part h of the quads); lane -> (zone of the row, quad of the part)
  const int gw = gt / 32, ln = gt % 32, h = gw % pl.nh, lz = ln / pl.qw;
  const int c = (gw / pl.nh) * pl.zw + lz, q = h * pl.qw + ln % pl.qw;  // zone slot, group quad
  const bool lane_ok = lz < pl.zw && q < GQ && c < zpi;
  const int qr = q < GQ ? q : GQ - 1;  // quad read by idle lanes (results unused)
  const int cr = lane_ok ? c : zpi - 1;  // slot read by idle lanes (results unused)
  // this warp's source-group range, rounded out to whole steps of 4
  int lo = G, hi = -1;
  if (lane_ok)
    for (int i = 0; i < 4; ++i) {
      lo = min(lo, pl.gp_lo[4 * qr + i]);
      hi = max(hi, pl.gp_hi[4 * qr + i]);
    }
  lo = __reduce_min_sync(0xffffffffu, lo) & ~3;
  hi = (__reduce_max_sync(0xffffffffu, hi) + 4) & ~3;
  if (tid == 0) {
    for (int i = 0; i < kZoneGroups; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&full[i])));
      bad[i] = 0;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int stride = kZoneGroups * gridDim.x, first = kZoneGroups * blockIdx.x + gi;
  const uint32_t zbytes = (uint32_t)G * MM * 4;
  uint32_t ph = 0;
  bool pending = false;  // a copy issued by this group and not yet waited for (elected thread)
  for (int m = 0; m < 3; ++m) {
    const int64_t n = pl.off[m + 1] - pl.off[m];
    if (n == 0) continue;
    __syncthreads();  // both groups are done with the previous material's matrices
    {
      const float4 *src = reinterpret_cast<const float4 *>(sigsT + (size_t)m * L1 * G * G);
      float4 *dst = reinterpret_cast<float4 *>(sS);
      for (int i = tid; i < L1 * G * G / 4; i += kZoneThreads) dst[i] = src[i];
    }
    __syncthreads();
    const int64_t nitems = (n + zpi - 1) / zpi;
    auto issue = [&](int64_t it) {
      const int64_t z0 = pl.off[m] + it * zpi;
      const int nz = (int)min((int64_t)zpi, pl.off[m + 1] - z0);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the buffer's last generic reads
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"((uint32_t)nz * zbytes)
                   : "memory");
      for (int k = 0; k < nz; ++k)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(buf + (size_t)k * pl.slot)),
                     "l"(phi + (int64_t)zl[z0 + k] * G * MM), "r"(zbytes), "r"(bar)
                     : "memory");
      pending = true;
    };
    int64_t it = first;
    if (it < nitems && gt == 0 && !bad[gi]) issue(it);
    while (it < nitems) {
      // one elected thread waits (bounded), the group learns the outcome at its barrier
      if (gt == 0) {
        if (!bad[gi] && !zoneWait(bar, ph)) {
          bad[gi] = 1;
          atomicExch(pl.err, 1);
        } else if (!bad[gi]) {
          pending = false;
        }
      }
      asm volatile("bar.sync %0, %1;" ::"r"(1 + gi), "r"(kZoneGroup) : "memory");
      if (bad[gi]) break;
      zoneTestWait(bar, ph);  // completed phase: this thread's own acquire of the copied bytes
      ph ^= 1u;
      const int64_t z0 = pl.off[m] + it * zpi;
      const int nz = (int)min((int64_t)zpi, pl.off[m + 1] - z0);
      float acc[4][MM];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < MM; ++k) acc[i][k] = 0.0f;
      const float *zb = buf + (size_t)cr * pl.slot;
      for (int gb = lo; gb < hi; gb += 4) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int gp = gb + r;
          constexpr int kAlignMul = MM & 3;  // (MM gp) mod 4 = (MM mod 4)(gp mod 4) mod 4
          const int R = (kAlignMul * r) & 3;
          const float4 *pr = reinterpret_cast<const float4 *>(zb + MM * gp - R);
          float v[MM + 3 + 4];
#pragma unroll
          for (int j = 0; j < (MM + 3 + 3) / 4; ++j) {
            if (4 * j < R + MM) {
              const float4 w = pr[j];
              v[4 * j] = w.x;
              v[4 * j + 1] = w.y;
              v[4 * j + 2] = w.z;
              v[4 * j + 3] = w.w;
            }
          }
          float4 sl[L1];
#pragma unroll
          for (int l = 0; l < L1; ++l) sl[l] = *reinterpret_cast<const float4 *>(sS + ((size_t)l * G + gp) * G + 4 * qr);
#pragma unroll
          for (int k = 0; k < MM; ++k) {
            const float p = v[R + k];
            const float4 s4 = sl[legendreOf(k)];
            fma2Rn(acc[0][k], acc[1][k], s4.x, s4.y, p);  // acc += s * p, each rounded once
            fma2Rn(acc[2][k], acc[3][k], s4.z, s4.w, p);
          }
        }
      }
      asm volatile("bar.sync %0, %1;" ::"r"(1 + gi), "r"(kZoneGroup) : "memory");  // the buffer is read
      const int64_t next = it + stride;
      if (next < nitems && gt == 0) issue(next);
      if (lane_ok && c < nz) {
        float4 *o = reinterpret_cast<float4 *>(phi_out + ((int64_t)zl[z0 + c] * G + 4 * q) * MM);
#pragma unroll
        for (int j = 0; j < MM; ++j) {  // the thread's 4 x MM outputs, row-major, as MM 16-byte words
          float4 w = make_float4(acc[(4 * j) / MM][(4 * j) % MM], acc[(4 * j + 1) / MM][(4 * j + 1) % MM],
                                 acc[(4 * j + 2) / MM][(4 * j + 2) % MM], acc[(4 * j + 3) / MM][(4 * j + 3) % MM]);
          if (accumulate) {
            const float4 old = o[j];
            w.x = old.x + w.x;
            w.y = old.y + w.y;
            w.z = old.z + w.z;
            w.w = old.w + w.w;
          }
          o[j] = w;
        }
      }
      it = next;
    }
  }
  // a copy still in flight (only after a wait that gave up) must land before the CTA's memory goes away
  if (gt == 0 && pending) zoneWait(bar, ph);
  __syncthreads();
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

namespace {
// staged form: floats between zone blocks (16-byte multiple; an odd number of
// 16-byte words, so the zones that share a warp read distinct banks)
uint32_t zoneSlot(int G, int L) {
  const uint32_t mm = (uint32_t)(L + 1) * (L + 1);
  uint32_t slot = ((uint32_t)G * mm + 3u) & ~3u;
  if ((slot / 4) % 2 == 0) slot += 4;
  return slot;
}
// a zone's G/4 quads in nh parts of qw <= 8 (one warp each), zw = 32 / qw zones per warp
void zoneLanes(int G, int &nh, int &qw, int &zw) {
  const int gq = G / 4;
  nh = (gq + 7) / 8;
  qw = (gq + nh - 1) / nh;
  zw = 32 / qw;
}
int zoneItemZones(int G) {
  int nh, qw, zw;
  zoneLanes(G, nh, qw, zw);
  return (kZoneGroup / 32 / nh) * zw;
}
}  // namespace

size_t scatter_block_smem(int G, int L) {
  const int MM = (L + 1) * (L + 1), MP = (MM + 3) / 4 * 4;
  if (G % 4 == 0)  // staged form: the matrices and every group's zone buffer
    return sizeof(float) * ((size_t)(L + 1) * G * G + (size_t)kZoneGroups * zoneItemZones(G) * zoneSlot(G, L));
  const int Gw = G < 32 ? G : 32, zpc = (kBlkThreads / 32) * (32 / Gw) / ((G + 31) / 32);
  return sizeof(float) * (((size_t)(L + 1) * G * G + 3) / 4 * 4 + (size_t)zpc * G * MP);
}


void launch_scatter_block(const float *phi, float *phi_out, const float *sigsT, const int *zl, const int64_t off[4],
                          int G, int L, const int *gp_lo, const int *gp_hi, bool accumulate, int *err, int nsm,
                          cudaStream_t s) {
  if (G % 4 == 0) {
    ScatterZonePlan pl{};
    pl.G = G;
    pl.zpi = zoneItemZones(G);
    zoneLanes(G, pl.nh, pl.qw, pl.zw);
    pl.slot = zoneSlot(G, L);
    pl.gp_lo = gp_lo;
    pl.gp_hi = gp_hi;
    pl.err = err;
    int64_t most = 0;
    for (int m = 0; m < 4; ++m) pl.off[m] = off[m];
    for (int m = 0; m < 3; ++m) most = std::max(most, (off[m + 1] - off[m] + pl.zpi - 1) / pl.zpi);
    if (most == 0) return;
    const size_t smem = scatter_block_smem(G, L);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((most + kZoneGroups - 1) / kZoneGroups, nsm));
    auto go = [&](auto kernel) {
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kernel<<<grid, kZoneThreads, smem, s>>>(phi, phi_out, sigsT, zl, pl, accumulate);
    };
    switch (L) {
      case 0: go(scatter_zone_kernel<0>); break;
      case 1: go(scatter_zone_kernel<1>); break;
      case 2: go(scatter_zone_kernel<2>); break;
      case 3: go(scatter_zone_kernel<3>); break;
      default: go(scatter_zone_kernel<4>); break;
    }
    return;
  }
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
