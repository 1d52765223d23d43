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
#include "fp32_pair.h"
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

// Rows of the two transforms, shared by the per-call kernels and the batched
// kernels (one launch over many problems).  VEC: every psi / rhs row starts on
// a 16-byte boundary (D*sizeof(T) % 16 == 0).

// L rows [d][MB] (moments m0 .. m0+mc-1, zero padded) into shared memory
template <typename T, int MB>
__device__ __forceinline__ void loadRows(T *sm, const T *__restrict__ mat_dm, int D, int M, int m0, int mc) {
  for (int i = threadIdx.x; i < D * MB; i += blockDim.x) {
    const int d = i / MB, m = i - d * MB;
    sm[i] = (m < mc) ? mat_dm[(int64_t)d * M + m0 + m] : T(0);
  }
}

// phi(m0 .. m0+mc-1) of one (zone, group) row: sum over directions, ascending
template <typename T, int MB, bool VEC>
__device__ __forceinline__ void ltimesRow(const T *__restrict__ p, const T *sell, int D, T *o, int mc,
                                          bool accumulate) {
  constexpr int V = Vec16<T>::n;
  T acc[MB];
#pragma unroll
  for (int m = 0; m < MB; ++m) acc[m] = T(0);
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
#pragma unroll
  for (int m = 0; m < MB; ++m)
    if (m < mc) o[m] = accumulate ? o[m] + acc[m] : acc[m];
}

// rhs(d) of one (zone, group) row: sum over moments, ascending
template <typename T, int MB, bool VEC>
__device__ __forceinline__ void lplusRow(const T *__restrict__ src, const T *sel, int D, int M, T *o,
                                         bool accumulate) {
  constexpr int V = Vec16<T>::n;
  T po[MB];
#pragma unroll
  for (int m = 0; m < MB; ++m) po[m] = (m < M) ? src[m] : T(0);
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

// LTimes, two rows per thread (FP32, whole 16-byte vectors, up to 28 moments):
// every L vector read from shared memory feeds both rows, halving the
// shared-memory traffic per multiply-add; each row's sums run in the same order
// as above.  (LPlusTimes measured slower both paired and with 8 threads per
// row: 6.0 -> 7.2 / 7.4 ms at 64^3.)
template <typename T, int MB>
__device__ __forceinline__ void ltimesRow2(const T *__restrict__ p0, const T *__restrict__ p1, const T *sell, int D,
                                           T *o0, T *o1, int mc, bool accumulate) {
  constexpr int V = Vec16<T>::n;
  T a0[MB], a1[MB];
#pragma unroll
  for (int m = 0; m < MB; ++m) a0[m] = a1[m] = T(0);
  for (int d0 = 0; d0 < D; d0 += V) {
    T pv0[V], pv1[V];
    load16(pv0, p0 + d0);
    load16(pv1, p1 + d0);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const T *e = sell + (d0 + v) * MB;
#pragma unroll
      for (int m = 0; m < MB; m += V) {
        T ev[V];
        load16(ev, e + m);
#pragma unroll
        for (int u = 0; u < V; ++u) {
          a0[m + u] += ev[u] * pv0[v];
          a1[m + u] += ev[u] * pv1[v];
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < MB; ++m)
    if (m < mc) {
      o0[m] = accumulate ? o0[m] + a0[m] : a0[m];
      o1[m] = accumulate ? o1[m] + a1[m] : a1[m];
    }
}

template <typename T, int MB, bool VEC>
constexpr bool pairRows() {
  return sizeof(T) == 4 && VEC && MB <= 28;
}

template <typename T, int MB, bool VEC>
__global__ void __launch_bounds__(kMomThreads) ltimes_kernel(const T *__restrict__ psi, T *__restrict__ phi,
                                                            const T *__restrict__ ell_dm, int64_t rows, int D,
                                                            int M, int m0, int mc, bool accumulate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sell = reinterpret_cast<T *>(smem_raw);  // [D][MB]
  loadRows<T, MB>(sell, ell_dm, D, M, m0, mc);
  __syncthreads();
  if constexpr (pairRows<T, MB, VEC>()) {
    for (int64_t r = 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); r < rows;
         r += 2 * (int64_t)gridDim.x * blockDim.x) {
      if (r + 1 < rows)
        ltimesRow2<T, MB>(psi + r * D, psi + (r + 1) * D, sell, D, phi + r * M + m0, phi + (r + 1) * M + m0, mc,
                          accumulate);
      else
        ltimesRow<T, MB, VEC>(psi + r * D, sell, D, phi + r * M + m0, mc, accumulate);
    }
  } else {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
      ltimesRow<T, MB, VEC>(psi + r * D, sell, D, phi + r * M + m0, mc, accumulate);
  }
}

template <typename T, int MB, bool VEC>
__global__ void __launch_bounds__(kMomThreads) lplustimes_kernel(const T *__restrict__ phi_out, T *__restrict__ rhs,
                                                                const T *__restrict__ ellp_dm, int64_t rows, int D,
                                                                int M, bool accumulate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sel = reinterpret_cast<T *>(smem_raw);  // [D][MB]
  loadRows<T, MB>(sel, ellp_dm, D, M, 0, M);
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
    lplusRow<T, MB, VEC>(phi_out + r * M, sel, D, M, rhs + r * D, accumulate);
}

// Batched transforms: work items are row ranges of one problem each; a block
// reloads the L / L+ rows when its next item belongs to another problem.
template <typename T, int MB, bool VEC, bool PLUS>
__global__ void __launch_bounds__(kMomThreads) batch_moments_kernel(const BatchMom<T> *__restrict__ inst,
                                                                   const BatchRows *__restrict__ items, int nitems) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sm = reinterpret_cast<T *>(smem_raw);  // [D][MB]
  int cur = -1;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const BatchRows w = items[it];
    const BatchMom<T> b = inst[w.inst];
    if (w.inst != cur) {
      __syncthreads();
      loadRows<T, MB>(sm, b.mat, b.D, b.M, 0, b.M);
      __syncthreads();
      cur = w.inst;
    }
    for (int64_t r = w.r0 + threadIdx.x; r < w.r1; r += blockDim.x) {
      if (PLUS) lplusRow<T, MB, VEC>(b.src + r * b.M, sm, b.D, b.M, b.dst + r * b.D, false);
      else ltimesRow<T, MB, VEC>(b.src + r * b.D, sm, b.D, b.dst + r * b.M, b.M, false);
    }
  }
}

// LTimes, FP32, register-tiled (directions a multiple of 32, M <= 32): a block
// takes 128-row tiles of psi, copies each 32-direction chunk into shared
// memory with cp.async (two buffers: the next chunk, or the next tile's first,
// streams in while one is multiplied) and each thread accumulates 4 rows x MB
// moments (rows lane + 32 i, moments MB*warp ...) in registers.  Per direction
// a thread reads its 4 rows' values 16 bytes at a time (4 directions per read)
// and the warp's MB moments of L as one or two 16-byte broadcasts: 4*MB
// multiply-adds per 1 + MB/4 shared-memory reads, against MB per one for the
// row-per-thread kernel.  Each output is one FMA chain over ascending
// directions, as in ltimesRow, so the results are the same bit for bit.
constexpr int kTileRows = 128;     // rows per tile (4 per thread)
constexpr int kTileK = 32;         // directions per shared-memory chunk
constexpr int kTilePitch = kTileK + 4;  // row pitch: the 8 lanes of a quarter-warp hit distinct banks

template <int MB>
__global__ void __launch_bounds__(kMomThreads) ltimes_tile_kernel(const float *__restrict__ psi,
                                                                 float *__restrict__ phi,
                                                                 const float *__restrict__ ell_dm, int64_t rows,
                                                                 int D, int M, bool accumulate, int *outexp,
                                                                 int rexp_w, int G) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *ls = reinterpret_cast<float *>(smem_raw);  // [D][32]: warp w's moments at 8w .. 8w+MB-1
  float *as = ls + (size_t)D * 32;                   // [2][kTileRows][kTilePitch]
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int i = tid; i < D * 32; i += blockDim.x) {
    const int d = i >> 5, c = i & 31, g = c >> 3, j = c & 7, m = MB * g + j;
    ls[i] = (j < MB && m < M) ? ell_dm[(int64_t)d * M + m] : 0.f;
  }
  const int64_t ntiles = (rows + kTileRows - 1) / kTileRows;
  const int nk = D / kTileK;
  // chunk q of this block: tile blockIdx.x + (q / nk) * gridDim.x, directions (q % nk) * 32
  const int64_t nq = ntiles > blockIdx.x ? ((ntiles - 1 - blockIdx.x) / gridDim.x + 1) * nk : 0;
  auto issue = [&](int64_t q) {
    const int64_t tile = blockIdx.x + (q / nk) * gridDim.x;
    const int k0 = (int)(q % nk) * kTileK;
    float *buf = as + (q & 1) * (kTileRows * kTilePitch);
#pragma unroll
    for (int i = 0; i < kTileRows * kTileK / 4 / kMomThreads; ++i) {
      const int idx = tid + i * kMomThreads, r = idx >> 3, c4 = idx & 7;
      const int64_t row = tile * kTileRows + r;
      if (row < rows) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(buf + r * kTilePitch + 4 * c4);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(psi + row * D + k0 + 4 * c4)
                     : "memory");
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  if (nq > 0) issue(0);
  __syncthreads();  // L in shared memory
  float acc[4][MB];
  for (int64_t q = 0; q < nq; ++q) {
    if (q % nk == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int m = 0; m < MB; ++m) acc[i][m] = 0.f;
    }
    if (q + 1 < nq) {
      issue(q + 1);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const float *buf = as + (q & 1) * (kTileRows * kTilePitch);
    const float *lk = ls + (size_t)(q % nk) * kTileK * 32 + 8 * w;
#pragma unroll 2
    for (int k4 = 0; k4 < kTileK / 4; ++k4) {
      float4 a[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = *reinterpret_cast<const float4 *>(buf + (lane + 32 * i) * kTilePitch + 4 * k4);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        float l[8];
        *reinterpret_cast<float4 *>(l) = *reinterpret_cast<const float4 *>(lk + (4 * k4 + kk) * 32);
        if (MB > 4) *reinterpret_cast<float4 *>(l + 4) = *reinterpret_cast<const float4 *>(lk + (4 * k4 + kk) * 32 + 4);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float x = kk == 0 ? a[i].x : kk == 1 ? a[i].y : kk == 2 ? a[i].z : a[i].w;
#pragma unroll
          for (int m = 0; m + 1 < MB; m += 2) fma2Rn(acc[i][m], acc[i][m + 1], l[m], l[m + 1], x);
          if (MB & 1) acc[i][MB - 1] = __fmaf_rn(l[MB - 1], x, acc[i][MB - 1]);
        }
      }
    }
    __syncthreads();  // the buffer is refilled two chunks later
    if (q % nk == nk - 1) {
      const int64_t tile = blockIdx.x + (q / nk) * gridDim.x;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t row = tile * kTileRows + lane + 32 * i;
        const bool valid = row < rows;
        if (outexp) {
          // phi's exponent record for the gathered scattering (not accumulated): the
          // 32 lanes hold consecutive (zone, group) rows, one warp reduction per moment
          // over each run of rows of one zone, one atomic per run
          const unsigned live = __ballot_sync(0xffffffffu, valid);
          const unsigned rw = (unsigned)rexp_w;
          const unsigned run = (rw >= 32u ? 0xffffffffu : (((1u << rw) - 1u) << (lane & ~(rw - 1u)))) & live;
          if (valid) {
            const int64_t zb = (row / G) * M;
#pragma unroll
            for (int m = 0; m < MB; ++m) {
              if (MB * w + m < M) {
                const unsigned ex = (__float_as_uint(acc[i][m]) >> 23) & 0xFFu;
                const unsigned mx = __reduce_max_sync(run, ex);
                if ((lane & (rw - 1u)) == 0) atomicMax(outexp + zb + MB * w + m, (int)mx);
              }
            }
          }
        }
        if (!valid) continue;
        float *o = phi + row * M + MB * w;
#pragma unroll
        for (int m = 0; m < MB; ++m)
          if (MB * w + m < M) o[m] = accumulate ? o[m] + acc[i][m] : acc[i][m];
      }
    }
  }
}

// LPlusTimes, FP32, register-tiled (M <= 32, directions a multiple of 4): a
// block takes 32-row tiles of phi_out (staged in shared memory, the next tile's
// values loaded into registers while this one is multiplied) and sweeps the
// directions 128 at a time; warp w accumulates rows 8w .. 8w+7, lane l the
// directions 4l .. 4l+3 of the block.  Per 4 moments a thread reads its rows'
// moments as 8 broadcasts and L+ as 4 contiguous 16-byte reads (128
// multiply-adds per 12 reads), and each warp stores 512 contiguous bytes of a
// row.  Every output is the FMA chain of lplusRow (ascending moments, then the
// zero padding up to the moment class MB), so the results are the same bit
// for bit -- also those of the fused sweep's prologue.
constexpr int kPlusRows = 32;

template <int MB>
__global__ void __launch_bounds__(kMomThreads) lplus_tile_kernel(const float *__restrict__ phi_out,
                                                                float *__restrict__ rhs,
                                                                const float *__restrict__ ellp_dm, int64_t rows,
                                                                int D, int M, bool accumulate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *lp = reinterpret_cast<float *>(smem_raw);  // [MB][D]: L+ transposed, zero rows beyond M
  float *po = lp + (size_t)MB * D;                   // [2][kPlusRows][MB]
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int i = tid; i < MB * D; i += blockDim.x) {
    const int m = i / D, d = i - m * D;
    lp[i] = m < M ? ellp_dm[(int64_t)d * M + m] : 0.f;
  }
  constexpr int kPer = (kPlusRows * 32 + kMomThreads - 1) / kMomThreads;  // staged values per thread (M <= 32)
  const int64_t ntiles = (rows + kPlusRows - 1) / kPlusRows;
  float nxt[kPer];
  auto fetch = [&](int64_t tile) {  // the tile's phi_out block is contiguous: rows * M values
    const int64_t base = tile * kPlusRows * M;
    const int64_t n = (tile * kPlusRows + kPlusRows <= rows ? kPlusRows : rows - tile * kPlusRows) * M;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int idx = tid + i * kMomThreads;
      nxt[i] = (idx < kPlusRows * M && idx < n) ? phi_out[base + idx] : 0.f;
    }
  };
  auto stage = [&](float *buf) {
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int idx = tid + i * kMomThreads;
      if (idx < kPlusRows * M) {
        const int r = idx / M;
        buf[r * MB + (idx - r * M)] = nxt[i];
      }
    }
    for (int i = tid; i < kPlusRows * (MB - M); i += kMomThreads) {  // zero padding
      const int r = i / (MB - M);
      buf[r * MB + M + (i - r * (MB - M))] = 0.f;
    }
  };
  int64_t tile = blockIdx.x;
  if (tile < ntiles) fetch(tile);
  for (int b = 0; tile < ntiles; tile += gridDim.x, b ^= 1) {
    float *buf = po + b * (kPlusRows * MB);
    stage(buf);
    __syncthreads();  // L+ (first pass) and this tile's moments in shared memory
    if (tile + gridDim.x < ntiles) fetch(tile + gridDim.x);
    for (int d0 = 0; d0 < D; d0 += 128) {
      const int d = d0 + 4 * lane;
      if (d >= D) continue;
      float acc[8][4];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[i][u] = 0.f;
#pragma unroll
      for (int m4 = 0; m4 < MB; m4 += 4) {
        float4 e[4];
#pragma unroll
        for (int mm = 0; mm < 4; ++mm) e[mm] = *reinterpret_cast<const float4 *>(lp + (size_t)(m4 + mm) * D + d);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float4 x = *reinterpret_cast<const float4 *>(buf + (8 * w + i) * MB + m4);
          const float xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
          for (int mm = 0; mm < 4; ++mm) {
            acc[i][0] = __fmaf_rn(e[mm].x, xv[mm], acc[i][0]);
            acc[i][1] = __fmaf_rn(e[mm].y, xv[mm], acc[i][1]);
            acc[i][2] = __fmaf_rn(e[mm].z, xv[mm], acc[i][2]);
            acc[i][3] = __fmaf_rn(e[mm].w, xv[mm], acc[i][3]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int64_t row = tile * kPlusRows + 8 * w + i;
        if (row >= rows) continue;
        float4 *o = reinterpret_cast<float4 *>(rhs + row * D + d);
        float4 v = make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
        if (accumulate) {
          const float4 old = *o;
          v = make_float4(old.x + v.x, old.y + v.y, old.z + v.z, old.w + v.w);
        }
        *o = v;
      }
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
      const int64_t units = pairRows<T, MB, true>() ? (rows + 1) / 2 : rows;
      ltimes_kernel<T, MB, true><<<gridFor(units), kMomThreads, smem, s>>>(psi, phi, ell, rows, D, M, 0, M, acc);
    } else {
      setSmem(ltimes_kernel<T, MB, false>, smem);
      ltimes_kernel<T, MB, false><<<gridFor(rows), kMomThreads, smem, s>>>(psi, phi, ell, rows, D, M, 0, M, acc);
    }
  }
};

template <int MB>
void launchLTimesTile(const float *psi, float *phi, const float *ell_dm, int64_t rows, int D, int M, bool acc,
                      cudaStream_t s, int *outexp = nullptr, int rexp_w = 32, int G = 1) {
  const size_t smem = sizeof(float) * ((size_t)D * 32 + 2 * kTileRows * kTilePitch);
  setSmem(ltimes_tile_kernel<MB>, smem);
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ltimes_tile_kernel<MB>, kMomThreads, smem);
  const int64_t ntiles = (rows + kTileRows - 1) / kTileRows;
  const int64_t cap = (int64_t)nsm * (per > 0 ? per : 1);
  const int grid = (int)(ntiles < cap ? (ntiles > 0 ? ntiles : 1) : cap);
  ltimes_tile_kernel<MB><<<grid, kMomThreads, smem, s>>>(psi, phi, ell_dm, rows, D, M, acc, outexp, rexp_w, G);
}

bool ltimes_tiled_applies(int D, int M) { return D % kTileK == 0 && D <= 1024 && M <= 32 && M >= 13; }

// The register-tiled FP32 kernel when it applies (returns false otherwise).
bool launchLTimesTiled(const float *psi, float *phi, const float *ell_dm, int64_t rows, int D, int M, bool acc,
                       cudaStream_t s, int *outexp = nullptr, int rexp_w = 32, int G = 1) {
  if (!ltimes_tiled_applies(D, M)) return false;
  const int mb = (M + 3) / 4;
  if (mb == 4) launchLTimesTile<4>(psi, phi, ell_dm, rows, D, M, acc, s, outexp, rexp_w, G);
  else if (mb == 5) launchLTimesTile<5>(psi, phi, ell_dm, rows, D, M, acc, s, outexp, rexp_w, G);
  else if (mb == 6) launchLTimesTile<6>(psi, phi, ell_dm, rows, D, M, acc, s, outexp, rexp_w, G);
  else if (mb == 7) launchLTimesTile<7>(psi, phi, ell_dm, rows, D, M, acc, s, outexp, rexp_w, G);
  else launchLTimesTile<8>(psi, phi, ell_dm, rows, D, M, acc, s, outexp, rexp_w, G);
  return true;
}
bool launchLTimesTiled(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t) {
  return false;
}

bool launch_ltimes_record(const float *psi, float *phi, const float *ell_dm, int64_t rows, int D, int M,
                          int *outexp, int rexp_w, int G, cudaStream_t s) {
  return launchLTimesTiled(psi, phi, ell_dm, rows, D, M, false, s, outexp, rexp_w, G);
}

template <typename T>
void launch_ltimes(const T *psi, T *phi, const T *ell_dm, int64_t rows, int D, int M, bool accumulate, cudaStream_t s) {
  if (launchLTimesTiled(psi, phi, ell_dm, rows, D, M, accumulate, s)) return;
#define KGB_L(MBV) LTimesLaunch<T, MBV>{psi, phi, ell_dm, rows, D, M, accumulate, s}
  byMoments<T, LTimesLaunch>(M, KGB_L(4), KGB_L(12), KGB_L(16), KGB_L(28), KGB_L(36), KGB_L(52), KGB_L(64));
#undef KGB_L
}

template <int MB>
void launchLPlusTile(const float *phi_out, float *rhs, const float *ellp_dm, int64_t rows, int D, int M, bool acc,
                     cudaStream_t s) {
  const size_t smem = sizeof(float) * ((size_t)MB * D + 2 * kPlusRows * MB);
  setSmem(lplus_tile_kernel<MB>, smem);
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lplus_tile_kernel<MB>, kMomThreads, smem);
  const int64_t ntiles = (rows + kPlusRows - 1) / kPlusRows;
  const int64_t cap = (int64_t)nsm * (per > 0 ? per : 1);
  const int grid = (int)(ntiles < cap ? (ntiles > 0 ? ntiles : 1) : cap);
  lplus_tile_kernel<MB><<<grid, kMomThreads, smem, s>>>(phi_out, rhs, ellp_dm, rows, D, M, acc);
}

// The register-tiled FP32 kernel when it applies (returns false otherwise).  MB
// is the moment class of lplusRow, so both add the same zero padding.
bool launchLPlusTiled(const float *phi_out, float *rhs, const float *ellp_dm, int64_t rows, int D, int M, bool acc,
                      cudaStream_t s) {
  if (D % 4 != 0 || M > 28) return false;
  const int mb = moment_class(M);
  // L+ stays in shared memory: at most 200 KB with the two moment tiles
  if (sizeof(float) * ((size_t)mb * D + 2 * kPlusRows * mb) > 200 * 1024) return false;
  if (mb == 4) launchLPlusTile<4>(phi_out, rhs, ellp_dm, rows, D, M, acc, s);
  else if (mb == 12) launchLPlusTile<12>(phi_out, rhs, ellp_dm, rows, D, M, acc, s);
  else if (mb == 16) launchLPlusTile<16>(phi_out, rhs, ellp_dm, rows, D, M, acc, s);
  else launchLPlusTile<28>(phi_out, rhs, ellp_dm, rows, D, M, acc, s);
  return true;
}
bool launchLPlusTiled(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t) {
  return false;
}

template <typename T>
void launch_lplustimes(const T *phi_out, T *rhs, const T *ellp_dm, int64_t rows, int D, int M, bool accumulate,
                       cudaStream_t s) {
  if (launchLPlusTiled(phi_out, rhs, ellp_dm, rows, D, M, accumulate, s)) return;
#define KGB_L(MBV) LPlusLaunch<T, MBV>{phi_out, rhs, ellp_dm, rows, D, M, accumulate, s}
  byMoments<T, LPlusLaunch>(M, KGB_L(4), KGB_L(12), KGB_L(16), KGB_L(28), KGB_L(36), KGB_L(52), KGB_L(64));
#undef KGB_L
}

// Batched launches: MB is the moment class of every problem in the items (all
// share one vector width); FP64 LPlusTimes runs scalar like the per-call path.
template <typename T, int MB>
struct BatchMomLaunch {
  const BatchMom<T> *inst; const BatchRows *items; int nitems, Dmax; bool plus, vec; int grid; cudaStream_t s;
  void operator()() const {
    const size_t smem = sizeof(T) * (size_t)Dmax * MB;
    auto go = [&](auto kernel) {
      setSmem(kernel, smem);
      kernel<<<grid, kMomThreads, smem, s>>>(inst, items, nitems);
    };
    if (plus) {
      if (vec) go(batch_moments_kernel<T, MB, true, true>);
      else go(batch_moments_kernel<T, MB, false, true>);
    } else {
      if (vec) go(batch_moments_kernel<T, MB, true, false>);
      else go(batch_moments_kernel<T, MB, false, false>);
    }
  }
};

template <typename T>
void launch_batch_moments(const BatchMom<T> *inst, const BatchRows *items, int nitems, int M, int Dmax, bool plus,
                          bool vec, int grid, cudaStream_t s) {
  if (nitems <= 0) return;
#define KGB_L(MBV) BatchMomLaunch<T, MBV>{inst, items, nitems, Dmax, plus, vec, grid, s}
  byMoments<T, BatchMomLaunch>(M, KGB_L(4), KGB_L(12), KGB_L(16), KGB_L(28), KGB_L(36), KGB_L(52), KGB_L(64));
#undef KGB_L
}

int moment_class(int M) {
  return M <= 4 ? 4 : M <= 12 ? 12 : M <= 16 ? 16 : M <= 28 ? 28 : M <= 36 ? 36 : M <= 52 ? 52 : 64;
}

template void launch_batch_moments<double>(const BatchMom<double> *, const BatchRows *, int, int, int, bool, bool, int,
                                           cudaStream_t);
template void launch_batch_moments<float>(const BatchMom<float> *, const BatchRows *, int, int, int, bool, bool, int,
                                          cudaStream_t);

template void launch_ltimes<double>(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t);
template void launch_ltimes<float>(const float *, float *, const float *, int64_t, int, int, bool, cudaStream_t);
template void launch_lplustimes<double>(const double *, double *, const double *, int64_t, int, int, bool, cudaStream_t);
template void launch_lplustimes<float>(const float *, float *, const float *, int64_t, int, int, bool, cudaStream_t);

}  // namespace kgb
