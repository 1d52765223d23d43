// tf32_moments.cu -- the mixed form's LTimes and LPlusTimes as tensor-core GEMMs
// in split TF32 (three products, FP32 accumulation in tensor memory).
//
// Both transforms are row products C[r][n] = sum_k A[r][k] B[k][n] over the
// (zone, group) rows of the device nesting ([zone][group][direction] for psi
// and rhs, [zone][group][moment] for phi and phi_out):
//   LTimes      A = psi (K = directions), B[d][m] = ell(m,d),      C = phi
//   LPlusTimes  A = phi_out (K = moments), B[m][d] = ell_plus(d,m), C = rhs
// replacing Kernel::LTimes (src/Kripke/Kernel/LTimes.cpp:54-65) and
// Kernel::LPlusTimes (src/Kripke/Kernel/LPlusTimes.cpp:49-60) in the mixed form,
// overwriting phi (rhs) in the solver loop, accumulating into it through the
// kernel entry points (C += A B by bulk reduce-adds: one FP32 add per element).
//
// Split TF32: every FP32 operand x is written exactly as hi + mid + lo, three
// TF32 numbers.  The kernels truncate A: hi = x with its 13 low fraction bits
// cleared (10 fraction bits kept), r = x - hi (exact, at most 13 significant
// bits, |r| < 2^-10 |x|), mid = r truncated likewise, lo = r - mid (exact, at
// most 2 significant bits); B is rounded to nearest on the host (|r| <= 2^-11 |x|).
// Both are exact splits; truncation is two logic operations per element where
// rounding took two conversions (LTimes 3.91 -> 3.75 ms, LPlusTimes 1.83 ->
// 1.75 ms at 64^3 zones x 64 groups x 128 directions x P4).
// The product a b is taken as the six terms of order up to 2^-20:
//   hi hi + hi mid + mid hi + mid mid + hi lo + lo hi
// (six kind::tf32 MMAs per K step; TF32 x TF32 products are exact, the sums
// accumulate in FP32 in tensor memory); the dropped mid lo + lo mid + lo lo are
// below 2^-30 |a b|, so what remains is the FP32 accumulation.  The tensor
// core's accumulation is not rounded to nearest at every step, so a chunk's
// MMAs add the small terms of all its K steps first and the four leading
// hi x hi products last, and LTimes accumulates each 32-direction chunk
// separately, the epilogue adding the chunks in FP32, rounded to nearest, in
// K order.  (Two pieces, hi + lo with
// lo rounded to TF32, leave 2^-22 |a b| per product: measured four times the
// SIMT kernel's error on 192-direction rows with cancellation.)  B is split on
// the host once.
//
// Data movement (one persistent CTA per SM, 128-row tiles):
//  - LTimes: A streams through shared memory by 2D TMA (boxes of 128 rows x 32
//    directions, 128-byte swizzle, a ring of stages); phi tiles leave as bulk
//    copies of each warp's 32 rows (contiguous [rows][M], staged in shared memory).
//  - LPlusTimes: phi_out tiles (128 x M floats, contiguous) arrive by one bulk
//    copy each; rhs leaves by 2D TMA stores of 32 rows x 32 directions per warp
//    (128-byte swizzle, staged in shared memory).
//  - The split operands go to tensor memory (A of tcgen05.mma read from tensor
//    memory: one lane per row, one column per element; a 32-element K chunk takes
//    96 columns for its three pieces), B stays in shared memory (no swizzle,
//    K-major core matrices of 8 rows x 16 bytes).
//
// Roles: warps 0-3 are workers (warp w owns tensor-memory lanes 32w..32w+31 =
// tile rows 32w..): they split tile t's A chunks into tensor memory and, after
// that, drain tile t-1's accumulator (read, stage, store).  Warp 4 issues the
// loads, warp 5 the MMAs.  Hand-offs are mbarriers, every wait is bounded
// (0.2 s, globaltimer); a wait that gives up raises the CTA's abort flag, every
// role stops, the CTA waits (bounded) for its copies and MMAs in flight,
// releases tensor memory and reports through the error word.

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "kgb_internal.h"

namespace kgb {

namespace {

constexpr int kRows = 128;                   // tile rows = MMA M
constexpr int kChunk = 32;                   // K elements per chunk (one TMA box, one tensor-memory slot)
constexpr int kWorkers = 4;                  // worker warps
constexpr int kThreads = (kWorkers + 2) * 32;  // + load warp + MMA warp
constexpr int kMaxStages = 8;
constexpr int kMaxSlots = 4;
constexpr int kOutSlots = 4;                 // LPlusTimes: staged 32 x 32 output boxes per warp
constexpr uint32_t kTmemCols = 512;
constexpr int kPieces = 3;                   // hi, mid, lo
constexpr uint32_t kSlotCols = kPieces * kChunk;  // tensor-memory columns of one A chunk
constexpr uint64_t kWaitNs = 200000000ull;   // 0.2 s

__device__ __forceinline__ uint32_t smemAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t nowNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for the completion of the phase with the given parity; gives up
// (and raises the abort flag) after kWaitNs, or returns early once another
// role has given up.
__device__ __forceinline__ bool waitBar(uint64_t *bar, uint32_t parity, volatile int *abort) {
  uint32_t done = 0;
  uint64_t t0 = 0;
  for (uint32_t it = 0; !done; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(parity)
        : "memory");
    if (!done && (it & 63u) == 63u) {
      if (*abort) return false;
      const uint64_t t = nowNs();
      if (t0 == 0) t0 = t;
      else if (t - t0 > kWaitNs) break;
    }
  }
  if (!done) *abort = 1;
  return done != 0;
}

__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar)) : "memory");
}

__device__ __forceinline__ void initBar(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count));
}

// shared-memory matrix descriptor (tcgen05), no swizzle: start, LBO, SBO in 16-byte units
__device__ __forceinline__ uint64_t matDesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; bits 61-63 = 0: no swizzle
  return d;
}

// kind::tf32 instruction descriptor: FP32 accumulate (bits 4-5 = 1), TF32 A and
// B (format 2 at bits 7-9 and 10-12), both K-major, N >> 3 at bit 17, M = 128
__device__ __forceinline__ uint32_t idescTf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kRows >> 4) << 24);
}

// D (tensor memory) += A (tensor memory) x B (shared memory); acc = 0 overwrites D
__device__ __forceinline__ void mmaTf32(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d),
      "r"(a), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar))
               : "memory");
}

__device__ __forceinline__ void tmemSt32(uint32_t taddr, const uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
      "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]), "r"(v[17]),
      "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]),
      "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
      : "memory");
}

__device__ __forceinline__ void tmemLd32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
      "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
}

struct Tf32Args {
  const float *A;      // LPlusTimes: phi_out [rows][K], allocation padded to whole 128-row tiles
  float *C;            // LTimes: phi [rows][ncols], allocation padded likewise
  const float *bimg;   // B in TF32: hi, mid and lo images, each [nk*32/4][N/8][8][4] floats
  int64_t rows;
  int K;               // reduction length (LTimes: directions, LPlusTimes: moments <= 32)
  int nk;              // 32-wide K chunks per tile
  int N;               // MMA width: a multiple of 16, at most 256
  int ncols;           // output columns (LTimes: moments, LPlusTimes: directions)
  int ns, nt, nacc;    // shared-memory A stages, tensor-memory A slots, accumulators
  uint32_t stage_bytes, out_bytes_per_warp;
  uint32_t load_bytes;  // bytes of one A chunk copy (LTimes: the TMA box; LPlusTimes: a whole tile)
  int accumulate;      // 0: C = A B; 1: C += A B (one FP32 add per element, by bulk reductions)
  int *err;
};

// MODE 0: LTimes (A by 2D TMA through `tmap`; narrow outputs by bulk copy).
// MODE 1: LPlusTimes (A by bulk copy; wide outputs by 2D TMA stores through `tmap`).
template <int MODE>
__global__ void __launch_bounds__(kThreads, 1) tf32x3_kernel(const __grid_constant__ CUtensorMap tmap,
                                                             const Tf32Args a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], tready[kMaxSlots], tfree[kMaxSlots];
  __shared__ uint64_t accfull[2], accempty[2], bload, drain;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  volatile int *abort = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int N = a.N, nk = a.nk, NS = a.ns, NT = a.nt, NACC = a.nacc;
  const uint32_t bImgBytes = (uint32_t)nk * kChunk * N * 4;  // one of hi / mid / lo
  const int64_t ntiles = (a.rows + kRows - 1) / kRows;

  const uint32_t base = smemAddr(smem_raw);
  unsigned char *al = smem_raw + (((base + 1023u) & ~1023u) - base);
  unsigned char *sB = al;  // hi, mid, lo images
  unsigned char *sA = sB + ((kPieces * bImgBytes + 1023u) & ~1023u);
  unsigned char *sOut = sA + (uint32_t)NS * a.stage_bytes;
  // LTimes keeps one accumulator per 32-direction chunk (the tensor core accumulates
  // 4 K steps into each; the epilogue adds the chunks in FP32, rounded to nearest)
  const uint32_t accW = (uint32_t)(MODE == 0 ? nk : 1) * N;  // columns of one tile's accumulators
  const uint32_t accCols = (uint32_t)NACC * accW;
  const uint32_t aBase = (accCols + 63u) & ~63u;  // first column of the A slots

  if (tid == 0) {
    for (int i = 0; i < NS; ++i) {
      initBar(&full[i], 1);
      initBar(&empty[i], kWorkers);
    }
    for (int i = 0; i < NT; ++i) {
      initBar(&tready[i], kWorkers);
      initBar(&tfree[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      initBar(&accfull[i], 1);
      initBar(&accempty[i], kWorkers);
    }
    initBar(&bload, 1);
    initBar(&drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;

  if (warp < kWorkers) {
    // ---------------- workers: split tile t into tensor memory, then drain tile t-1 ----------------
    const int r = warp * 32 + lane;                       // tile row = tensor-memory lane
    const uint32_t lanes = (uint32_t)(warp * 32) << 16;  // this warp's lane quarter
    auto wwait = [&](uint64_t *bar, uint32_t parity) -> bool {
      return __all_sync(0xffffffffu, waitBar(bar, parity, abort));
    };
    auto epilogue = [&](int it, int64_t tile) -> bool {
      const int ac = it % NACC;
      if (!wwait(&accfull[ac], (uint32_t)(it / NACC) & 1u)) return false;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t acol = tmem + lanes + (uint32_t)ac * accW;
      if constexpr (MODE == 0) {
        uint32_t v[32];
        tmemLd32(acol, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        for (int c = 1; c < nk; ++c) {  // the chunks' partial sums, in K order
          uint32_t w[32];
          tmemLd32(acol + (uint32_t)(c * N), w);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int k = 0; k < 32; ++k) v[k] = __float_as_uint(__uint_as_float(v[k]) + __uint_as_float(w[k]));
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) arrive(&accempty[ac]);
        // this warp's 32 rows of phi are contiguous: stage them row-major, one bulk copy
        const int M = a.ncols;
        float *stg = reinterpret_cast<float *>(sOut + warp * a.out_bytes_per_warp) + (it & 1) * 32 * M;
        if (lane == 0 && it >= 2) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 32; ++k)
          if (k < M) stg[lane * M + k] = __uint_as_float(v[k]);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          float *dst = a.C + (tile * kRows + warp * 32) * (int64_t)M;
          if (a.accumulate)
            asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f32 [%0], [%1], %2;" ::"l"(dst),
                         "r"(smemAddr(stg)), "r"((uint32_t)(32 * M * 4))
                         : "memory");
          else
            asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                         "r"(smemAddr(stg)), "r"((uint32_t)(32 * M * 4))
                         : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
      } else {
        const int ng = (a.ncols + 31) / 32;
        for (int g = 0; g < ng; ++g) {
          uint32_t v[32];
          tmemLd32(acol + (uint32_t)(32 * g), v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (g == ng - 1) {
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) arrive(&accempty[ac]);
          }
          const int gi = it * ng + g, slot = gi % kOutSlots;
          unsigned char *stg = sOut + warp * a.out_bytes_per_warp + slot * 4096;
          if (lane == 0 && gi >= kOutSlots) asm volatile("cp.async.bulk.wait_group.read 3;" ::: "memory");
          __syncwarp();
          // 32 rows x 128 bytes, 16-byte chunk j of row `lane` at chunk position j ^ (lane & 7)
#pragma unroll
          for (int j = 0; j < 8; ++j)
            *reinterpret_cast<uint4 *>(stg + lane * 128 + ((j ^ (lane & 7)) << 4)) =
                make_uint4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            const int x = 32 * g, y = (int)(tile * kRows + warp * 32);
            if (a.accumulate)
              asm volatile(
                  "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                      &tmap),
                  "r"(x), "r"(y), "r"(smemAddr(stg))
                  : "memory");
            else
              asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                               &tmap),
                           "r"(x), "r"(y), "r"(smemAddr(stg))
                           : "memory");
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          }
        }
      }
      return true;
    };

    int it = 0;
    int64_t prev = -1;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++it) {
      for (int c = 0; c < nk && ok; ++c) {
        const int q = it * nk + c, s = q % NS, u = q % NT;
        if (!wwait(&full[s], (uint32_t)(q / NS) & 1u)) {
          ok = false;
          break;
        }
        float x[32];
        const unsigned char *st = sA + (uint32_t)s * a.stage_bytes;
        if constexpr (MODE == 0) {
          // 128-byte swizzle: 16-byte chunk j of row r sits at chunk position j ^ (r & 7)
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float4 f = *reinterpret_cast<const float4 *>(st + r * 128 + ((j ^ (r & 7)) << 4));
            x[4 * j] = f.x;
            x[4 * j + 1] = f.y;
            x[4 * j + 2] = f.z;
            x[4 * j + 3] = f.w;
          }
        } else {
          const float *row = reinterpret_cast<const float *>(st) + r * a.K;
#pragma unroll
          for (int k = 0; k < 32; ++k) x[k] = k < a.K ? row[k] : 0.0f;
        }
        __syncwarp();
        if (lane == 0) arrive(&empty[s]);  // the stage is in registers
        uint32_t hi[32], mid[32], lo[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) {  // truncating split: x - hi and r - mid are exact
          hi[k] = __float_as_uint(x[k]) & 0xFFFFE000u;
          const float rr = x[k] - __uint_as_float(hi[k]);
          mid[k] = __float_as_uint(rr) & 0xFFFFE000u;
          lo[k] = __float_as_uint(rr - __uint_as_float(mid[k]));
        }
        // the MMAs that last read slot u must be done before it is overwritten
        if (q >= NT && !wwait(&tfree[u], (uint32_t)(q / NT - 1) & 1u)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t sc = tmem + lanes + aBase + (uint32_t)u * kSlotCols;
        tmemSt32(sc, hi);
        tmemSt32(sc + 32, mid);
        tmemSt32(sc + 64, lo);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) arrive(&tready[u]);
      }
      if (!ok) break;
      // Two accumulators: drain tile t-1 now (tile t's MMAs run meanwhile; tile t+1's wait
      // for this drain).  One accumulator: tile t+1's MMAs wait for tile t's drain, and with
      // more K chunks than A slots tile t+1's split waits for its own MMAs, so drain tile t
      // before splitting the next one.
      if (NACC == 1) {
        if (!epilogue(it, tile)) ok = false;
      } else {
        if (prev >= 0 && !epilogue(it - 1, prev)) ok = false;
        prev = tile;
      }
    }
    if (ok && NACC == 2 && prev >= 0) epilogue(it - 1, prev);
    // the bulk stores must have read their staging before the CTA's shared memory goes away
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    __syncwarp();
  } else if (warp == kWorkers && lane == 0) {
    // ---------------- loads: B once, then the A chunks of every tile ----------------
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(&bload)),
                 "r"(kPieces * bImgBytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smemAddr(sB)),
                 "l"(a.bimg), "r"(kPieces * bImgBytes), "r"(smemAddr(&bload))
                 : "memory");
    int it = 0, issued = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles && !*abort; tile += gridDim.x, ++it) {
      for (int c = 0; c < nk; ++c) {
        const int q = it * nk + c, s = q % NS;
        if (q >= NS && !waitBar(&empty[s], (uint32_t)(q / NS - 1) & 1u, abort)) break;
        const uint32_t dst = smemAddr(sA + (uint32_t)s * a.stage_bytes);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(&full[s])),
                     "r"(a.load_bytes)
                     : "memory");
        if constexpr (MODE == 0) {
          asm volatile(
              "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
              "[%4];" ::"r"(dst),
              "l"(&tmap), "r"(c * kChunk), "r"((int)(tile * kRows)), "r"(smemAddr(&full[s]))
              : "memory");
        } else {
          const float *src = a.A + tile * kRows * (int64_t)a.K;
          asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                           dst),
                       "l"(src), "r"(a.load_bytes), "r"(smemAddr(&full[s]))
                       : "memory");
        }
        issued = q + 1;
      }
    }
    // every load issued must have landed before the CTA's shared memory goes away
    volatile int never = 0;  // these waits give up only on their own time limit
    for (int q = max(0, issued - NS); q < issued; ++q) waitBar(&full[q % NS], (uint32_t)(q / NS) & 1u, &never);
    waitBar(&bload, 0, &never);
  } else if (warp == kWorkers + 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = idescTf32(N);
    const uint32_t bHi = smemAddr(sB), bMid = bHi + bImgBytes, bLo = bMid + bImgBytes;
    const uint32_t lbo = 16u * (uint32_t)N;  // core matrices adjacent in K
    bool ok = waitBar(&bload, 0, abort);
    int it = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok && !*abort; tile += gridDim.x, ++it) {
      const int ac = it % NACC;
      if (it >= NACC && !waitBar(&accempty[ac], (uint32_t)(it / NACC - 1) & 1u, abort)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t dtile = tmem + (uint32_t)ac * accW;
      for (int c = 0; c < nk; ++c) {
        const uint32_t dcol = dtile + (MODE == 0 ? (uint32_t)(c * N) : 0u);
        const bool fresh = MODE == 0 || c == 0;  // LTimes: each chunk starts its own sum
        const int q = it * nk + c, u = q % NT;
        if (!waitBar(&tready[u], (uint32_t)(q / NT) & 1u, abort)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t ahi = tmem + aBase + (uint32_t)u * kSlotCols, amid = ahi + 32, alo = ahi + 64;
        // the five small terms of every K step first (their sum stays near 2^-10 of the
        // result, so the accumulator's roundings there are small), then the leading
        // hi x hi products: four large-magnitude accumulations per chunk instead of 24
#pragma unroll
        for (int ks = 0; ks < kChunk / 8; ++ks) {
          const uint32_t boff = (uint32_t)((c * kChunk + ks * 8) / 4) * lbo;
          const uint64_t dh = matDesc(bHi + boff, lbo, 128), dm = matDesc(bMid + boff, lbo, 128),
                         dl = matDesc(bLo + boff, lbo, 128);
          mmaTf32(dcol, alo + ks * 8, dh, idesc, (!fresh || ks > 0) ? 1u : 0u);
          mmaTf32(dcol, ahi + ks * 8, dl, idesc, 1u);
          mmaTf32(dcol, amid + ks * 8, dm, idesc, 1u);
          mmaTf32(dcol, amid + ks * 8, dh, idesc, 1u);
          mmaTf32(dcol, ahi + ks * 8, dm, idesc, 1u);
        }
        // the leading products in descending K order: the accumulator truncates (towards zero)
        // at each step, and in LPlusTimes the first K step holds moment 0, which dominates the
        // sum; added last, only one truncation happens at the sum's full magnitude
#pragma unroll
        for (int ks = kChunk / 8 - 1; ks >= 0; --ks) {
          const uint32_t boff = (uint32_t)((c * kChunk + ks * 8) / 4) * lbo;
          mmaTf32(dcol, ahi + ks * 8, matDesc(bHi + boff, lbo, 128), idesc, 1u);
        }
        commit(&tfree[u]);  // slot u's last reader
      }
      if (!ok) break;
      commit(&accfull[ac]);
    }
    // drain: every MMA issued (also on a failed run) must finish before tensor memory is released
    commit(&drain);
    volatile int never = 0;
    if (!waitBar(&drain, 0, &never)) *abort = 1;
  }
  if (*abort && tid == 0) atomicExch(a.err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encodeFn() {
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

// 2D map over a [rows][cols] FP32 array (row pitch cols * 4 bytes), boxes of
// box_rows x 32 floats with the 128-byte swizzle
bool encodeMap(CUtensorMap *m, const float *base, int64_t rows, int cols, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encodeFn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 4};
  const cuuint32_t box[2] = {32, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t smemBytes(const Tf32Args &a) {
  const size_t b = ((size_t)kPieces * a.nk * kChunk * a.N * 4 + 1023) & ~(size_t)1023;
  return 1024 + b + (size_t)a.ns * a.stage_bytes + (size_t)kWorkers * a.out_bytes_per_warp;
}

constexpr size_t kSmemLimit = 227 * 1024 - 2048;  // dynamic shared memory, less the kernel's static part
// at least this much dynamic shared memory, so no two CTAs share an SM (each takes all of tensor memory)
constexpr size_t kSmemFloor = 116 * 1024;

// tensor-memory plan: accumulators first, then as many A slots (kSlotCols columns each) as fit (at most 4)
bool planTmem(Tf32Args &a, int acc_width) {
  for (int nacc = 2; nacc >= 1; --nacc) {
    const int abase = (nacc * acc_width + 63) / 64 * 64;
    const int nt = std::min(kMaxSlots, ((int)kTmemCols - abase) / (int)kSlotCols);
    if (nt >= 2) {
      a.nacc = nacc;
      a.nt = nt;
      return true;
    }
  }
  return false;
}

template <int MODE>
int launch(const CUtensorMap &m, Tf32Args a, int nsm, cudaStream_t s) {
  const size_t smem = std::max(smemBytes(a), kSmemFloor);
  if (smem > kSmemLimit) return 1;
  if (cudaFuncSetAttribute(tf32x3_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 1;
  const int64_t ntiles = (a.rows + kRows - 1) / kRows;
  const int grid = (int)std::min<int64_t>(ntiles, nsm);
  if (grid <= 0) return 0;
  tf32x3_kernel<MODE><<<grid, kThreads, smem, s>>>(m, a);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace

// the A box (LTimes) and the output box (LPlusTimes) are 32 directions wide: rows at least that long;
// LTimes' per-chunk accumulators and two A slots must fit tensor memory
bool tf32_ltimes_applies(int D, int M) {
  if (!(M >= 1 && M <= 32 && D >= 32 && D % 4 == 0)) return false;
  Tf32Args a{};
  a.N = M <= 16 ? 16 : 32;
  a.nk = (D + kChunk - 1) / kChunk;
  return planTmem(a, a.nk * a.N);
}
bool tf32_lplustimes_applies(int D, int M) { return M >= 1 && M <= 32 && D % 16 == 0 && D >= 32 && D <= 256; }

int64_t tf32_padded_rows(int64_t rows) { return (rows + kRows - 1) / kRows * kRows; }

// B (K x N, row-major, b[k * N + n]) split exactly into TF32 hi, mid and lo (as
// the kernel splits A), as the kernel's shared-memory images: K padded to kpad,
// N to npad, each image [kpad/4][npad/8][8][4] floats (core matrices of 8 rows
// of N x 4 K elements).
void tf32_build_b(const float *b, int K, int N, int kpad, int npad, std::vector<float> &img) {
  img.assign((size_t)kPieces * kpad * npad, 0.0f);
  auto rna = [](float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7F800000u) != 0x7F800000u) u = (u + 0x1000u) & 0xFFFFE000u;  // round the magnitude, ties away
    float r;
    std::memcpy(&r, &u, 4);
    return r;
  };
  for (int k = 0; k < K; ++k)
    for (int n = 0; n < N; ++n) {
      const float x = b[(size_t)k * N + n];
      const float h = rna(x), r = x - h, m = rna(r), l = r - m;
      const size_t off = ((size_t)(k / 4) * (npad / 8) + n / 8) * 32 + (n % 8) * 4 + (k % 4);
      img[off] = h;
      img[(size_t)kpad * npad + off] = m;
      img[(size_t)2 * kpad * npad + off] = l;
    }
}

int launch_tf32_ltimes(const float *psi, float *phi, int64_t rows, int D, int M, const float *bimg, bool accumulate,
                       int *err, int nsm, cudaStream_t s) {
  if (!tf32_ltimes_applies(D, M)) return 1;
  Tf32Args a{};
  a.C = phi;
  a.bimg = bimg;
  a.rows = rows;
  a.K = D;
  a.nk = (D + kChunk - 1) / kChunk;
  a.N = M <= 16 ? 16 : 32;
  a.ncols = M;
  a.err = err;
  a.stage_bytes = kRows * kChunk * 4;
  a.load_bytes = a.stage_bytes;
  a.accumulate = accumulate ? 1 : 0;
  a.out_bytes_per_warp = (2 * 32 * M * 4 + 127) / 128 * 128;
  if (!planTmem(a, a.nk * a.N)) return 1;
  const size_t fixed = smemBytes(a);  // with no A stages yet
  a.ns = (int)std::min<size_t>(kMaxStages, (kSmemLimit - fixed) / a.stage_bytes);
  if (a.ns < 2) return 1;
  CUtensorMap m;
  if (!encodeMap(&m, psi, rows, D, kRows)) return 1;
  return launch<0>(m, a, nsm, s);
}

int launch_tf32_lplustimes(const float *phi_out, float *rhs, int64_t rows, int D, int M, const float *bimg,
                           bool accumulate, int *err, int nsm, cudaStream_t s) {
  if (!tf32_lplustimes_applies(D, M)) return 1;
  Tf32Args a{};
  a.A = phi_out;
  a.bimg = bimg;
  a.rows = rows;
  a.K = M;
  a.nk = 1;
  a.N = D;
  a.ncols = D;
  a.err = err;
  a.load_bytes = kRows * M * 4;  // one whole tile of the padded allocation
  a.stage_bytes = (a.load_bytes + 1023) / 1024 * 1024;
  a.accumulate = accumulate ? 1 : 0;
  a.out_bytes_per_warp = kOutSlots * 4096;
  if (!planTmem(a, a.N)) return 1;
  const size_t fixed = smemBytes(a);
  a.ns = (int)std::min<size_t>(4, (kSmemLimit - fixed) / a.stage_bytes);
  if (a.ns < 2) return 1;
  CUtensorMap m;
  if (!encodeMap(&m, rhs, rows, D, 32)) return 1;
  return launch<1>(m, a, nsm, s);
}

}  // namespace kgb
