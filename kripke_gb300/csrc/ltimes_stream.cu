// ltimes_stream.cu -- the mixed form's LTimes (FP32 SIMT) fed by the Tensor
// Memory Accelerator.
//
// Kernel::LTimes (src/Kripke/Kernel/LTimes.cpp:54-65): phi(z,g,m) =
// sum_d ell(m,d) psi(z,g,d) over the (zone, group) rows of the device nesting.
// The arithmetic is the register-tiled kernel's of moments.cu: a block takes
// 128-row tiles, each thread keeps MB = ceil(M/4) moments of four rows in
// registers and walks the directions in ascending order with paired FP32
// multiply-adds, so every output is the same FMA chain -- bit for bit the
// register-tiled and row-per-thread kernels.  Each compute warp takes 32 rows
// of the tile for all moments (its four lane groups a quarter of the moments
// each; the last group carries three zero moments when M = 25).  The block is
// held to 96 registers a thread so that four fit on an SM: 2.73 ms at 64^3
// zones x 64 groups x 128 directions, P4, against 2.86 ms at three blocks per
// SM, and 2.74 ms with each warp on all 128 rows for a quarter of the moments
// at four blocks (fewer shared-memory wavefronts, 70.6 against 86.7 M at 32^3,
// but an extra loop for the short last quarter).  What differs from the
// register-tiled kernel is the operand path.  There every thread copied its
// share of each 32-direction chunk with cp.async and the block synchronised
// twice a chunk; here a fifth warp issues one TMA copy per chunk (a {32
// directions, 128 rows} box, 128-byte swizzled so a quarter-warp's 16-byte
// reads of eight rows fall in distinct banks) into a ring of shared-memory
// stages, the compute warps wait on the stage's mbarrier and release it by one
// arrival each on a second mbarrier, and no block-wide barrier remains in the
// loop.  Rows past the end read zeros (the box's fill) and are not stored.
// Every wait is bounded (0.2 s of globaltimer); one that gives up sets *err,
// the block stops issuing and finishes the copies it started, and the host
// reports KGB_ERR_TIMEOUT.
//
// The octant-pair form (SYM, the table of ltimes_sym.h) sums each chunk as
// L(m, b) (psi(b) +- psi(b')) over the chunk's first 16 directions and their
// mirror images: half the multiply-adds, which bounded the kernel (2.64 ->
// 2.16 ms at 64^3 x 64 groups x 128 directions, P4), in another order than
// the reference's ascending sum, so it is held to FP32 rounding of it.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "fp32_pair.h"
#include "ltimes_sym.h"
#include "kgb_internal.h"

namespace kgb {

namespace {

constexpr int kLsRows = 128;              // rows per tile
constexpr int kLsK = 32;                  // directions per stage (one 128-byte row)
constexpr int kLsCompute = 4;             // compute warps
constexpr int kLsThreads = (kLsCompute + 1) * 32;
constexpr int kLsMaxStages = 4;
constexpr uint32_t kLsStageBytes = kLsRows * kLsK * 4;  // 16 KB
constexpr uint64_t kLsWaitNs = 200000000ull;

__device__ __forceinline__ uint32_t sAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gNow() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool waitPar(uint64_t *bar, uint32_t parity, volatile int *abort) {
  uint32_t done = 0;
  uint64_t t0 = 0;
  for (uint32_t it = 0; !done; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(sAddr(bar)), "r"(parity)
        : "memory");
    if (!done && (it & 63u) == 63u) {
      if (*abort) return false;
      const uint64_t t = gNow();
      if (t0 == 0) t0 = t;
      else if (t - t0 > kLsWaitNs) break;
    }
  }
  if (!done) *abort = 1;
  return done != 0;
}

// SYM: the octant-pair form (MB = 8).  sym holds, per 32-direction chunk, the partner
// column (16..31) of each of the chunk's first 16 directions, then the moment of each of
// the 32 slots (-1: empty); lane groups 0 and 1 hold the moments whose L columns repeat
// with sign +1 on the partners, groups 2 and 3 those with sign -1.
template <int MB, bool SYM>
__global__ void __launch_bounds__(kLsThreads, 4) ltimes_stream_kernel(const __grid_constant__ CUtensorMap pmap,
                                                                   float *__restrict__ phi,
                                                                   const float *__restrict__ ell_dm, int64_t rows,
                                                                   int D, int M, int ns, const int *__restrict__ sym,
                                                                   int *err) {
  extern __shared__ __align__(1024) unsigned char sraw[];
  __shared__ __align__(8) uint64_t full[kLsMaxStages], empty[kLsMaxStages];
  __shared__ int abort_flag;
  volatile int *abort = &abort_flag;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const uint32_t base = sAddr(sraw);
  unsigned char *const al = sraw + (((base + 1023u) & ~1023u) - base);  // stages: 1024-byte aligned (swizzle)
  float *const ls = reinterpret_cast<float *>(al + (size_t)ns * kLsStageBytes);  // [D][32] (SYM: [D/2][32])
  int *const pcol = reinterpret_cast<int *>(ls + (size_t)(SYM ? D / 2 : D) * 32);  // SYM: [D/32][16], slots [32]
  int *const slotm = pcol + (SYM ? D / 2 : 0);
  if constexpr (SYM) {
    for (int i = tid; i < D / 2 + 32; i += blockDim.x) pcol[i] = sym[i];
    for (int i = tid; i < D / 2 * 32; i += blockDim.x) {
      const int c = i >> 9, b = (i >> 5) & 15, m = sym[D / 2 + (i & 31)];
      ls[i] = m >= 0 ? ell_dm[(int64_t)(32 * c + b) * M + m] : 0.f;
    }
  } else {
    for (int i = tid; i < D * 32; i += blockDim.x) {
      const int d = i >> 5, c = i & 31, g = c >> 3, j = c & 7, m = MB * g + j;
      ls[i] = (j < MB && m < M) ? ell_dm[(int64_t)d * M + m] : 0.f;
    }
  }
  if (tid == 0) {
    for (int s = 0; s < ns; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sAddr(&full[s])), "r"(1));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sAddr(&empty[s])), "r"(kLsCompute));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  __syncthreads();
  const int64_t ntiles = (rows + kLsRows - 1) / kLsRows;
  const int nk = D / kLsK;
  // chunk q of this block: tile blockIdx.x + (q / nk) * gridDim.x, directions (q % nk) * 32
  const int64_t nq = ntiles > blockIdx.x ? ((ntiles - 1 - blockIdx.x) / gridDim.x + 1) * nk : 0;

  if (w == kLsCompute) {
    // producer: one TMA copy per chunk, into the stage the compute warps released
    if (lane == 0) {
      int64_t q = 0;
      for (; q < nq; ++q) {
        const int s = (int)(q % ns);
        const int64_t n = q / ns;
        if (n > 0 && !waitPar(&empty[s], (uint32_t)(n - 1) & 1u, abort)) break;
        const int64_t tile = blockIdx.x + (q / nk) * gridDim.x;
        const int k0 = (int)(q % nk) * kLsK;
        const uint32_t bar = sAddr(&full[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kLsStageBytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
            "[%4];" ::"r"(sAddr(al + (size_t)s * kLsStageBytes)),
            "l"(&pmap), "r"(k0), "r"((int)(tile * kLsRows)), "r"(bar)
            : "memory");
      }
      // a give-up: the copies already issued still land in the stages; wait for them (bounded)
      // before the block's shared memory is released
      if (q < nq)
        for (int64_t r = q - ns < 0 ? 0 : q - ns; r < q; ++r) {
          volatile int dummy = 0;
          waitPar(&full[r % ns], (uint32_t)(r / ns) & 1u, &dummy);
        }
    }
    return;
  }

  float acc[4][MB];
  // warp w holds the tile's rows 32 w .. 32 w + 31: lane group mg = lane % 4 the moments
  // MB mg .. MB mg + MB - 1 of the rows 32 w + rg + 8 i (rg = lane / 4, i = 0..3)
  const int mg = lane & 3;
  const int rbase = 32 * w + (lane >> 2);
  const int swz = rbase & 7;  // the thread's rows share their low three bits
  for (int64_t q = 0; q < nq; ++q) {
    if (q % nk == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int m = 0; m < MB; ++m) acc[i][m] = 0.f;
    }
    const int s = (int)(q % ns);
    const bool ok = __all_sync(0xffffffffu, waitPar(&full[s], (uint32_t)(q / ns) & 1u, abort));
    if (!ok) break;
    const unsigned char *buf = al + (size_t)s * kLsStageBytes;
    auto ldA = [&](int k4, float4 (&a)[4]) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
        a[i] = *reinterpret_cast<const float4 *>(buf + (rbase + 8 * i) * 128 + ((k4 ^ swz) << 4));
    };
    if constexpr (SYM) {
      // the chunk's two mirrored octants: for each of the first octant's 16 directions b and
      // its partner b', x = psi(b) + psi(b') (groups 0, 1) or psi(b) - psi(b') (groups 2, 3),
      // one rounding, then the slot moments' multiply-adds with L(m, b)
      const float sg = (mg >> 1) ? -1.f : 1.f;
      const int c = (int)(q % nk);
      const float *lk = ls + (size_t)c * 16 * 32 + 8 * mg;
      const int *pc = pcol + c * 16;
      auto body = [&](int b4, const float4 (&a)[4]) {
#pragma unroll
        for (int bb = 0; bb < 4; ++bb) {
          const int b = 4 * b4 + bb;
          float l[8];
          *reinterpret_cast<float4 *>(l) = *reinterpret_cast<const float4 *>(lk + b * 32);
          *reinterpret_cast<float4 *>(l + 4) = *reinterpret_cast<const float4 *>(lk + b * 32 + 4);
          const int col = pc[b];
          const int voff = (((col >> 2) ^ swz) << 4) + ((col & 3) << 2);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float u = bb == 0 ? a[i].x : bb == 1 ? a[i].y : bb == 2 ? a[i].z : a[i].w;
            const float v = *reinterpret_cast<const float *>(buf + (rbase + 8 * i) * 128 + voff);
            const float x = __fmaf_rn(sg, v, u);
#pragma unroll
            for (int m = 0; m < MB; m += 2) fma2Rn(acc[i][m], acc[i][m + 1], l[m], l[m + 1], x);
          }
        }
      };
      float4 a[4], b[4];
      ldA(0, a);
#pragma unroll
      for (int b4 = 0; b4 < 4; b4 += 2) {
        ldA(b4 + 1, b);
        body(b4, a);
        if (b4 + 2 < 4) ldA(b4 + 2, a);
        body(b4 + 1, b);
      }
    } else {
      const float *lk = ls + (size_t)(q % nk) * kLsK * 32 + 8 * mg;
      // the chunk's 32 directions into the thread's MB moments of its four rows
      auto body = [&](int k4, const float4 (&a)[4]) {
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
      };
      // the next direction quad's psi is read before this one's multiply-adds (2.74 -> 2.64 ms
      // at 64^3 zones x 64 groups x 128 directions, P4; unrolling alone: 2.67)
      float4 a[4], b[4];
      ldA(0, a);
#pragma unroll
      for (int k4 = 0; k4 < kLsK / 4; k4 += 2) {
        ldA(k4 + 1, b);
        body(k4, a);
        if (k4 + 2 < kLsK / 4) ldA(k4 + 2, a);
        body(k4 + 1, b);
      }
    }
    __syncwarp();
    if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sAddr(&empty[s])) : "memory");
    if (q % nk == nk - 1) {
      const int64_t tile = blockIdx.x + (q / nk) * gridDim.x;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t row = tile * kLsRows + rbase + 8 * i;
        if (row >= rows) continue;
        if constexpr (SYM) {
          float *o = phi + row * M;
#pragma unroll
          for (int m = 0; m < MB; ++m) {
            const int mo = slotm[MB * mg + m];
            if (mo >= 0) o[mo] = acc[i][m];
          }
        } else {
          float *o = phi + row * M + MB * mg;
#pragma unroll
          for (int m = 0; m < MB; ++m)
            if (MB * mg + m < M) o[m] = acc[i][m];
        }
      }
    }
  }
  if (*abort && err && lane == 0) atomicExch(err, 1);
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

template <int MB, bool SYM>
int launchAs(const CUtensorMap &m, float *phi, const float *ell_dm, int64_t rows, int D, int M, int ns,
             const int *sym, int *err, int nsm, cudaStream_t s) {
  // stages, the L table ([D][32], SYM: [D/2][32] and the partner / slot table) and the alignment slack
  const size_t smem = (size_t)ns * kLsStageBytes + (SYM ? (size_t)D / 2 * 32 * 4 + (size_t)(D / 2 + 32) * 4
                                                         : (size_t)D * 32 * 4) + 1024;
  if (cudaFuncSetAttribute(ltimes_stream_kernel<MB, SYM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 1;
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ltimes_stream_kernel<MB, SYM>, kLsThreads, smem);
  if (per < 1) return 1;
  const int64_t ntiles = (rows + kLsRows - 1) / kLsRows;
  const int64_t cap = (int64_t)nsm * per;
  const int grid = (int)(ntiles < cap ? (ntiles > 0 ? ntiles : 1) : cap);
  ltimes_stream_kernel<MB, SYM><<<grid, kLsThreads, smem, s>>>(m, phi, ell_dm, rows, D, M, ns, sym, err);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace

bool ltimes_stream_applies(int D, int M) { return ltimesStreamShape(D, M); }

bool ltimes_sym_table(const double *L, int D, int M, std::vector<int> &table) {
  return ltimesSymTable(L, D, M, table);
}

int launch_ltimes_stream(const float *psi, float *phi, const float *ell_dm, int64_t rows, int D, int M, int ns,
                         const int *sym, int *err, int nsm, cudaStream_t s) {
  if (!ltimes_stream_applies(D, M) || ns < 2 || ns > kLsMaxStages || ((uintptr_t)psi & 15u) != 0) return 1;
  PFN_cuTensorMapEncodeTiled_v12000 fn = encoder();
  if (!fn) return 1;
  CUtensorMap m;
  const cuuint64_t dims[2] = {(cuuint64_t)D, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)D * 4};
  const cuuint32_t box[2] = {kLsK, kLsRows};
  const cuuint32_t estr[2] = {1, 1};
  if (fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(psi), dims, strides, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return 1;
  if (sym) return launchAs<8, true>(m, phi, ell_dm, rows, D, M, ns, sym, err, nsm, s);
  const int mb = (M + 3) / 4;
  if (mb == 4) return launchAs<4, false>(m, phi, ell_dm, rows, D, M, ns, nullptr, err, nsm, s);
  if (mb == 5) return launchAs<5, false>(m, phi, ell_dm, rows, D, M, ns, nullptr, err, nsm, s);
  if (mb == 6) return launchAs<6, false>(m, phi, ell_dm, rows, D, M, ns, nullptr, err, nsm, s);
  if (mb == 7) return launchAs<7, false>(m, phi, ell_dm, rows, D, M, ns, nullptr, err, nsm, s);
  return launchAs<8, false>(m, phi, ell_dm, rows, D, M, ns, nullptr, err, nsm, s);
}

}  // namespace kgb
