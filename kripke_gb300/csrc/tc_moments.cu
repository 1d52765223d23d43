// tc_moments.cu -- LTimes and LPlusTimes on the GB300 tensor cores (tcgen05).
//
// Both transforms are row products C[r][n] = sum_k A[r][k] B[k][n] over the
// (zone, group) rows of the device nesting: LTimes has A = psi (K = directions)
// and B[d][m] = ell(m,d); LPlusTimes has A = phi_out (K = moments) and
// B[m][d] = ell_plus(d,m).  Replaces Kernel::LTimes
// (src/Kripke/Kernel/LTimes.cpp:54-65) and Kernel::LPlusTimes
// (src/Kripke/Kernel/LPlusTimes.cpp:49-60) when the shapes fit.
//
// Exact products from f16 digits (the Ozaki splitting, Ozaki et al. 2012,
// "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication"): every A row is scaled by a power of two
// taken from its largest element and written as S balanced 8-bit digits,
//   |A[r][k]| = 2^s_r * sum_i a_i * 2^-8i   (truncated after 8S-2 bits),
// a_i in [-128, 127] times the element's sign, and every B column likewise
// with 2^t_n and digits b_j (done on the host).  A digit has at most 8
// significant bits, so it is exact in f16 (as in bf16; f16 is used because its
// 11-bit significand lets one packed FMA form two digits from their bytes); a
// digit product is below 2^14 in
// magnitude, and for every anti-diagonal i+j the sum over k <= 128 of at most
// S products stays below 2^24, so tcgen05.mma with FP32 accumulation in tensor
// memory computes each diagonal sum D_{i+j} exactly.  The diagonals are
// recombined in integer arithmetic and rounded once:
//   C = 2^(s_r + t_n) * sum_{m=2..S+1} D_m * 2^-8m.
// Pairs with i+j > S+1 are dropped: their weight is below 2^-8(S+1) of the
// leading term.  S = 7 (54 bits) gives the FP64 form, S = 4 (30 bits) the
// mixed form.
//
// Tensor-memory layout: D_k occupies columns [(k-2)*NB, (k-1)*NB).  The B digit
// slices are stacked along N (slice j in rows [(j-1)*NB, j*NB)), so one MMA of
// A slice i against the first S+1-i slices of the stack, written at column
// (i-1)*NB, deposits every product a_i*b_j into diagonal i+j's block.
//
// Shared-memory operand layout: K-major, no swizzle ("interleaved" core
// matrices of 8 rows x 16 bytes; core matrices adjacent in K are LBO bytes
// apart, adjacent 8-row groups SBO = 128 bytes apart).  The kernel
// (tc_pipe_kernel, below) is warp-specialised and persistent, one CTA per SM;
// the B image reaches shared memory with one cp.async.bulk; every mbarrier
// wait is bounded, and on timeout the CTA records the failure, releases its
// tensor memory and returns.

#include <algorithm>
#include <cstring>

#include "kgb_internal.h"
#include "exact_round.h"

namespace kgb {

namespace {

constexpr int kTcRows = 128;            // rows per tile = MMA M
constexpr int kTcChunk = 32;            // K elements staged per A buffer

__device__ __forceinline__ uint32_t smemAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t matDesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; layout bits 61-63 = 0: no swizzle
  return d;
}

// kind::f16 instruction descriptor: FP32 accumulate (bits 4-5 = 1), f16 A and B
// (type fields at bits 7-9 and 10-12 both 0), both K-major, N >> 3, M = 128
__device__ __forceinline__ uint32_t instrDesc(int n) {
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar)));
}

__device__ __forceinline__ void ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
}

// The S balanced 8-bit digits (most significant first) of two (8S-2)-bit
// magnitudes as f16 pairs: element 0 in the low half, element 1 in the high
// half, each multiplied by its element's sign.  Adding 0x80 to every byte of
// the magnitude (the carries ripple upward and stay inside its 8S bits,
// since the magnitude is below 2^(8S-2)) turns byte b into the digit b - 128
// in [-128, 127].  Per digit, one byte permute places the two elements' bytes
// in the low bytes of the two halves, a mask puts them under the exponent of
// 1024 (the f16 value 1024 + b, exact: f16 has 11 significant bits), and one
// packed FMA forms s * (1024 + b) - s * 1152 = s * (b - 128) exactly for both
// elements, their signs s = +-1 applied through the multiplier and the offset.
template <int S>
__device__ __forceinline__ void digitPairs(uint64_t f0, uint32_t s0, uint64_t f1, uint32_t s1, uint32_t (&w)[S][4],
                                           int col) {
  static_assert(S == 4 || S == 7, "30-bit (FP32) or 54-bit (FP64) magnitudes");
  constexpr uint64_t kBias = S == 7 ? 0x0080808080808080ull : 0x80808080ull;
  const uint32_t sg = (s0 << 15) | (s1 << 31);
  const uint32_t mul = 0x3C003C00u ^ sg;  // f16x2 (s0, s1), s = +-1
  const uint32_t off = 0xE480E480u ^ sg;  // f16x2 (-1152 s0, -1152 s1)
  const uint64_t y0 = f0 + kBias, y1 = f1 + kBias;
  const uint32_t lo0 = (uint32_t)y0, hi0 = (uint32_t)(y0 >> 32), lo1 = (uint32_t)y1, hi1 = (uint32_t)(y1 >> 32);
#pragma unroll
  for (int i = 0; i < S; ++i) {
    const int byte = S - 1 - i;  // digit i is byte S-1-i of the biased magnitude
    const uint32_t x0 = byte >= 4 ? hi0 : lo0, x1 = byte >= 4 ? hi1 : lo1;
    // bytes [b0, -, b1, -], then the f16 pair (1024 + b0, 1024 + b1)
    const uint32_t sel = (uint32_t)(byte & 3) | ((uint32_t)(4 + (byte & 3)) << 8);
    const uint32_t t = (__byte_perm(x0, x1, sel) & 0x00FF00FFu) | 0x64006400u;
    uint32_t d;
    asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(d) : "r"(t), "r"(mul), "r"(off));
    w[i][col] = d;
  }
}

// Biased exponent (subnormals count as 1) and significand with the implicit bit.
__device__ __forceinline__ int expOf(double x) {
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7FF);
  return e > 0 ? e : 1;
}
__device__ __forceinline__ int expOf(float x) {
  const int e = (int)((__float_as_uint(x) >> 23) & 0xFF);
  return e > 0 ? e : 1;
}

// 64-bit right shift whose amount may reach or exceed 64 (PTX clamps it: 0)
__device__ __forceinline__ uint64_t shrClamped(uint64_t x, uint32_t n) {
  uint64_t r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(n));
  return r;
}

// Digit source: the (8S-2)-bit fixed-point magnitude of x relative to the
// row's largest exponent emax (the largest element's leading bit at 8S-3), and
// its sign: the significand placed with its leading bit at 8S-3, then shifted
// right by emax - e (emax >= e for every element of the row).
template <typename T, int S> struct Fixed;
template <int S> struct Fixed<double, S> {
  static __device__ __forceinline__ uint64_t mag(double x, int emax, uint32_t &sign) {
    static_assert(8 * S - 2 >= 53, "the significand fits the window");
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    sign = (uint32_t)(b >> 63);
    const int e = (int)((b >> 52) & 0x7FF);
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
    return shrClamped(m << (8 * S - 2 - 53), (uint32_t)(emax - (e > 0 ? e : 1)));
  }
};
template <int S> struct Fixed<float, S> {
  static __device__ __forceinline__ uint64_t mag(float x, int emax, uint32_t &sign) {
    static_assert(8 * S - 2 >= 24, "the significand fits the window");
    const uint32_t b = __float_as_uint(x);
    sign = b >> 31;
    const int e = (int)((b >> 23) & 0xFF);
    const uint64_t m = (uint64_t)((b & 0x7FFFFFu) | (e ? (1u << 23) : 0u));
    return shrClamped(m << (8 * S - 2 - 24), (uint32_t)(emax - (e > 0 ? e : 1)));
  }
};

// x * 2^e: exponent arithmetic when 2^e is a normal number, ldexp otherwise
__device__ __forceinline__ double scale2(double x, int e) {
  return (e >= -1022 && e <= 1023) ? x * __longlong_as_double((long long)(e + 1023) << 52) : ldexp(x, e);
}
__device__ __forceinline__ float scale2(float x, int e) {
  return (e >= -126 && e <= 127) ? x * __uint_as_float((uint32_t)(e + 127) << 23) : ldexpf(x, e);
}

// Combine the S diagonal sums (FP32, exact integers) into the output value.
// With A = 2^(emax-1076) sum_i a_i 2^(8(7-i)) and B likewise (FP64, S = 7),
// the kept diagonals D_m (m = i+j = 2..8) give
//   C = 2^(e0-60) * V,  V = sum_m D_m 2^(8(8-m)) = H*2^32 + L,
//   H = D2*2^16 + D3*2^8 + D4,  L = D5*2^24 + D6*2^16 + D7*2^8 + D8,
// with e0 = (emax - 1022) + (column exponent - 1022).
template <typename T, int S> struct Combine;
template <> struct Combine<double, 7> {
  // V rounded once to nearest in integer arithmetic (roundScaledOdd: bit for bit
  // the sum of the two exact doubles H*2^(e0-28) + L*2^(e0-60), without the FP64 add).
  // For K <= 128, |D_m| <= (m-1) * 128 * 2^14, so |H| < 2^38 and |L| < 2^48.
  static __device__ __forceinline__ double value(const float (&dk)[7], int e0) {
    long long d[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) d[k] = (long long)__float2int_rn(dk[k]);
    const long long h = (d[0] * 256 + d[1]) * 256 + d[2];
    const long long l = ((d[3] * 256 + d[4]) * 256 + d[5]) * 256 + d[6];
    bool ok = true;
    const double r = roundScaledOdd(h, l, e0 - 60, ok);
    if (ok) return r;
    return scale2(scale2((double)h, 32) + (double)l, e0 - 60);  // outside the normal range
  }
};
// The same for one K chunk (K <= 32): every diagonal sum is below 7*32*128^2 <
// 2^22, so each converts to an integer by the 1.5 * 2^23 offset (a float add)
// instead of a conversion instruction, and digit pairs combine in 32 bits.
struct CombineSmallK {
  static __device__ __forceinline__ double value(const float (&dk)[7], int e0) {
    int32_t d[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) d[k] = __float_as_int(dk[k] + 12582912.0f) - 0x4B400000;
    const int32_t p01 = d[0] * 256 + d[1], p34 = d[3] * 256 + d[4], p56 = d[5] * 256 + d[6];
    const long long h = (long long)p01 * 256 + d[2], l = (long long)p34 * 65536 + p56;
    bool ok = true;
    const double r = roundScaledOdd(h, l, e0 - 60, ok);
    if (ok) return r;
    return scale2(scale2((double)h, 32) + (double)l, e0 - 60);
  }
};

// FP32 (S = 4): A = 2^(emax-156) sum_i a_i 2^(8(4-i)), B = 2^(t-1052) sum_j
// b_j 2^(8(4-j)) (B from doubles), kept diagonals m = 2..5:
//   C = 2^(e0-36) * sum_m D_m 2^(8(5-m)),  e0 = (emax - 126) + (t - 1022).
template <> struct Combine<float, 4> {
  static __device__ __forceinline__ float value(const float (&dk)[4], int e0) {
    long long x = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) x = x * 256 + (long long)__float2int_rn(dk[k]);
    return scale2((float)x, e0 - 36);
  }
};

template <typename T> struct TcBias;
template <> struct TcBias<double> { static constexpr int v = 1022; };
template <> struct TcBias<float> { static constexpr int v = 126; };

// GATHER (tc_pipe_kernel): rows are (zone, moment) pairs of the device nesting [zone][group][moment]
// (the scattering's operand): row r is zone zl[r / nm], moment m0 + r % nm, and
// its element k (A) or n (C) lies ks elements after the row's base.
// ---------------------------------------------------------------------------
// Pipelined row products (the production kernel).
//
// Work items are (128-row tile, 32-column N block) pairs.  Warps 0..15 are
// workers: they split the A rows of a tile into digit slices (one 32-element K
// chunk per shared-memory stage, two stages) and, one tile later, drain the
// finished items from tensor memory (read, combine, store).  Warp 16 issues
// the MMAs.  Tensor memory holds two accumulators (2 x S x 32 columns), so the
// epilogue of one item overlaps the MMAs of the next, and the split of tile
// t+1 overlaps both.  Hand-offs are mbarriers: full[r] (16 worker-warp
// arrivals: stage r holds a chunk), empty[r] (MMA commit: stage r is free),
// accfull[s] (MMA commit: accumulator s is complete), accempty[s] (16
// worker-warp arrivals: accumulator s was read), emaxok[t % 4] (16 worker-warp
// arrivals: the tile's row exponents are in shared memory).  Every wait is
// bounded; a wait that gives up records the failure and every role stops.
// ---------------------------------------------------------------------------
constexpr int kPipeWorkers = 16;                       // worker warps
constexpr int kPipeThreads = (kPipeWorkers + 1) * 32;  // + the MMA warp
constexpr int kPipeNB = 32;                            // columns per N block
constexpr int kStagePitch = 5;                         // staged outputs per row: 4 columns + 1 pad

__device__ __forceinline__ uint64_t nowNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for the phase of the given parity: gives up (and raises the
// CTA's abort flag) after kPipeWaitNs, or as soon as another role has.  A
// legitimate wait lasts about one tile of work (tens of microseconds).
constexpr uint64_t kPipeWaitNs = 200000000ull;  // 0.2 s
__device__ __forceinline__ bool waitParityAbort(uint64_t *bar, uint32_t parity, volatile int *abort) {
  uint32_t done = 0;
  uint64_t t0 = 0;
  for (uint32_t it = 0; !done; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(parity));
    if (!done && (it & 63u) == 63u) {
      if (*abort) return false;
      const uint64_t t = nowNs();
      if (t0 == 0) t0 = t;
      else if (t - t0 > kPipeWaitNs) break;
    }
  }
  if (!done) *abort = 1;
  return done != 0;
}

__device__ __forceinline__ void arriveBar(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar)) : "memory");
}

template <typename T, int S, bool GATHER>
__global__ void __launch_bounds__(kPipeThreads, 1) tc_pipe_kernel(const TcArgs<T> a) {
  constexpr int NB = kPipeNB;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t full[2], empty[2], accfull[2], accempty[2], emaxok[4], bload, drain;
  __shared__ uint32_t tmem_slot;
  __shared__ int row_emax[4][kTcRows];
  __shared__ int abort_flag;
  volatile int *abort = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool worker = warp < kPipeWorkers;
  const int srow = warp * 8 + (lane & 7), part = lane >> 3;   // split mapping
  const int erow = (warp & 3) * 32 + lane, cgrp = warp >> 2;  // epilogue: TMEM lane quarter, 8 columns
  constexpr uint32_t kSliceBytes = kTcChunk * kTcRows * 2;
  constexpr uint32_t kBufBytes = S * kSliceBytes;
  constexpr uint32_t kLboA = (kTcRows / 8) * 128;
  constexpr uint32_t kAccCols = S * NB;             // one accumulator
  // tensor memory is allocated in powers of two: 2 x 224 columns (FP64) take 512
  constexpr uint32_t kTmemCols = 2 * kAccCols <= 256 ? 256u : 512u;
  static_assert(2 * kAccCols <= 512, "two accumulators must fit tensor memory");
  const uint32_t lboB = (uint32_t)S * NB * 16;
  const uint32_t blkBytes = (uint32_t)a.kpad * S * NB * 2;  // B image of one N block
  const int nchunks = a.kpad / kTcChunk;
  const int nb = a.nhalf;
  const int R = a.stages == 1 ? 1 : 2;  // A stages (1 only when a tile has one K chunk)
  const bool smallk = nchunks == 1;     // diagonal sums below 2^22

  const uint32_t base = smemAddr(smem_raw);
  unsigned char *al = smem_raw + (((base + 1023u) & ~1023u) - base);
  unsigned char *sB = al;
  unsigned char *sA = al + ((blkBytes * nb + 1023u) & ~1023u);
  int *sT = reinterpret_cast<int *>(sA + R * kBufBytes);
  // per-warp staging of finished outputs (contiguous rows only): [32 rows][kStagePitch]
  T *sStage = reinterpret_cast<T *>(sT + nb * NB) + warp * (32 * kStagePitch);

  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(&full[i])), "r"(kPipeWorkers));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(&empty[i])), "r"(1));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(&accfull[i])), "r"(1));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(&accempty[i])), "r"(kPipeWorkers));
    }
    for (int i = 0; i < 4; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(&emaxok[i])), "r"(kPipeWorkers));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(&bload)), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(&drain)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
    abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  for (int i = tid; i < nb * NB; i += kPipeThreads) sT[i] = a.bexp[i];
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    const uint32_t bbytes = blkBytes * nb;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(&bload)), "r"(bbytes));
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smemAddr(sB)),
                 "l"(a.bimg), "r"(bbytes), "r"(smemAddr(&bload)));
  }
  waitParityAbort(&bload, 0, abort);

  const int ntiles = (int)((a.rows + kTcRows - 1) / kTcRows);
  const bool vec = !GATHER && (a.lda * sizeof(T)) % 16 == 0;
  const int64_t kstride = GATHER ? a.ks : 1;
  auto rowBase = [&](int64_t r) -> int64_t {
    if constexpr (GATHER) {
      const int64_t q = r / a.nm;
      return (int64_t)a.zl[q] * a.zstride + a.m0 + (r - q * a.nm);
    } else {
      return r * a.lda;
    }
  };

  if (worker) {
    // ---------------- workers: split tile t, then drain tile t-1 ----------------
    // waits and the abort test are made warp-uniform: the warp-wide shuffles,
    // __syncwarp and tcgen05.ld below need every lane on the same path
    auto wwait = [&](uint64_t *bar, uint32_t parity) -> bool {
      return __all_sync(0xffffffffu, waitParityAbort(bar, parity, abort));
    };
    auto aborted = [&]() -> bool { return __any_sync(0xffffffffu, *abort != 0); };
    auto epilogue = [&](int lt, int tile) {
      const int64_t orow = (int64_t)tile * kTcRows + erow;
      const bool ovalid = orow < a.rows;
      T *crow = a.C + (ovalid ? (GATHER ? rowBase(orow) : orow * a.ldc) : 0);
      if (!wwait(&emaxok[lt & 3], (uint32_t)(lt >> 2) & 1u)) return;
      const int oemax = row_emax[lt & 3][erow] - TcBias<T>::v;
      for (int j = 0; j < nb; ++j) {
        const int p = lt * nb + j, st = p & 1;
        if (!wwait(&accfull[st], (uint32_t)(p >> 1) & 1u)) return;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t lanebase = (uint32_t)((warp & 3) * 32) << 16;
        uint32_t v[S][8];
#pragma unroll
        for (int k = 0; k < S; ++k) ld8(tmem + lanebase + (uint32_t)(st * kAccCols + k * NB + cgrp * 8), v[k]);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) arriveBar(&accempty[st]);  // the accumulator is in registers: release it
        auto combined = [&](int u, int n) -> T {
          float dk[S];
#pragma unroll
          for (int k = 0; k < S; ++k) dk[k] = __uint_as_float(v[k][u]);
          if constexpr (sizeof(T) == 8) {
            return smallk ? CombineSmallK::value(dk, oemax + sT[n]) : Combine<T, S>::value(dk, oemax + sT[n]);
          } else {
            return Combine<T, S>::value(dk, oemax + sT[n]);
          }
        };
        if (GATHER || !a.stage_out) {
          if (ovalid) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int n = j * NB + cgrp * 8 + u;
              if (n < a.N) {
                const T out = combined(u, n);
                T &dst = crow[(int64_t)n * kstride];
                dst = a.accumulate ? dst + out : out;
              }
            }
          }
        } else {
          // A lane holds 8 columns of one row; stored as they are, every store
          // instruction would touch 32 rows.  Staged through shared memory,
          // four columns at a time, each instruction writes 8 rows x 4
          // consecutive columns.
          T out[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int n = j * NB + cgrp * 8 + u;
            out[u] = (ovalid && n < a.N) ? combined(u, n) : T(0);
          }
          if constexpr (sizeof(T) == 8) {
            if (a.outexp) {
              // exponent record for the gathered consumer: one warp reduction per
              // column over each run of rows of one zone, one atomic per run
              const unsigned live = __ballot_sync(0xffffffffu, ovalid);
              const unsigned w = (unsigned)a.outexp_w;
              const unsigned run = (w >= 32u ? 0xffffffffu : (((1u << w) - 1u) << (lane & ~(w - 1u)))) & live;
              if (ovalid) {
                const int64_t zbase = (orow / a.outexp_rows) * (int64_t)a.N;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                  const int n = j * NB + cgrp * 8 + u;
                  if (n < a.N) {
                    const unsigned ex = (unsigned)((__double_as_longlong(out[u]) >> 52) & 0x7FF);
                    const unsigned m = __reduce_max_sync(run, ex);
                    if ((lane & (w - 1u)) == 0) atomicMax(a.outexp + zbase + n, (int)m);
                  }
                }
              }
            }
          }
          const int64_t rbase = (int64_t)tile * kTcRows + (warp & 3) * 32;
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
#pragma unroll
            for (int u = 0; u < 4; ++u) sStage[lane * kStagePitch + u] = out[hh * 4 + u];
            __syncwarp();
            const int n = j * NB + cgrp * 8 + hh * 4 + (lane & 3);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const int rl = (lane >> 2) + 8 * i;
              const int64_t orow2 = rbase + rl;
              if (orow2 < a.rows && n < a.N) {
                const T val = sStage[rl * kStagePitch + (lane & 3)];
                T &dst = a.C[orow2 * a.ldc + n];
                dst = a.accumulate ? dst + val : val;
              }
            }
            __syncwarp();
          }
        }
      }
    };

    int lt = 0, prev_tile = -1;
    for (int tile = blockIdx.x; tile < ntiles && !aborted(); tile += gridDim.x, ++lt) {
      const int64_t row = (int64_t)tile * kTcRows + srow;
      const bool valid = row < a.rows;
      const T *arow = a.A + (valid ? rowBase(row) : 0);
      if constexpr (!GATHER) {
        // the CTA's next tile of A rows (contiguous) into L2 while this one is split:
        // its row-exponent pass then waits on L2 instead of DRAM
        const int64_t r1 = (int64_t)(tile + gridDim.x) * kTcRows;
        if (tid == 0 && r1 < a.rows) {
          const int64_t nr = a.rows - r1 < kTcRows ? a.rows - r1 : kTcRows;
          const T *p = a.A + r1 * a.lda;
          // up to the last row's K-th element (A may be a K chunk inside wider rows),
          // rounded down to whole 16-byte units: nothing past the operand is touched
          const uint64_t bytes = ((uint64_t)((nr - 1) * a.lda + a.K) * sizeof(T)) & ~(uint64_t)15u;
          if (((uintptr_t)p & 15u) == 0 && bytes > 0 && bytes < (1ull << 31))
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"((uint32_t)bytes) : "memory");
        }
      }
      int emax = 1;
      if (a.rowexp) {
        // bound written by the kernel that produced A: no pass over the row
        if (valid) {
          if constexpr (GATHER) {
            const int64_t q = row / a.nm;
            emax = max(emax, a.rowexp[(int64_t)a.zl[q] * a.ks + a.m0 + (row - q * a.nm)]);
          } else {
            emax = max(emax, a.rowexp[row]);
          }
        }
      } else if (valid) {
        if (vec && a.K == a.kpad) {
#pragma unroll 4
          for (int c = 0; c < nchunks; ++c) {
            const T *p8 = arow + c * kTcChunk + part * 8;
            if constexpr (sizeof(T) == 8) {
              double2 v[4];
#pragma unroll
              for (int e = 0; e < 4; ++e) v[e] = *reinterpret_cast<const double2 *>(p8 + 2 * e);
#pragma unroll
              for (int e = 0; e < 4; ++e) emax = max(emax, max(expOf(v[e].x), expOf(v[e].y)));
            } else {
              float4 v[2];
#pragma unroll
              for (int e = 0; e < 2; ++e) v[e] = *reinterpret_cast<const float4 *>(p8 + 4 * e);
#pragma unroll
              for (int e = 0; e < 2; ++e)
                emax = max(emax, max(max(expOf(v[e].x), expOf(v[e].y)), max(expOf(v[e].z), expOf(v[e].w))));
            }
          }
        } else {
          for (int c = 0; c < nchunks; ++c) {
            const int k0 = c * kTcChunk + part * 8;
#pragma unroll
            for (int e = 0; e < 8; ++e)
              if (k0 + e < a.K) emax = max(emax, expOf(arow[(k0 + e) * kstride]));
          }
        }
      }
      emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 8));
      emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 16));
      if (part == 0) row_emax[lt & 3][srow] = emax;
      __syncwarp();
      if (lane == 0) arriveBar(&emaxok[lt & 3]);

      auto loadChunk = [&](int c, T (&x)[8]) {
        const int k0 = c * kTcChunk + part * 8;
        if (valid && vec && k0 + 8 <= a.K) {
          if constexpr (sizeof(T) == 8) {
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
              const double2 v = *reinterpret_cast<const double2 *>(arow + k0 + e);
              x[e] = v.x;
              x[e + 1] = v.y;
            }
          } else {
#pragma unroll
            for (int e = 0; e < 8; e += 4) {
              const float4 v = *reinterpret_cast<const float4 *>(arow + k0 + e);
              x[e] = v.x;
              x[e + 1] = v.y;
              x[e + 2] = v.z;
              x[e + 3] = v.w;
            }
          }
        } else {
#pragma unroll
          for (int e = 0; e < 8; ++e) x[e] = (valid && k0 + e < a.K) ? arow[(k0 + e) * kstride] : T(0);
        }
      };
      T xn[8];
      loadChunk(0, xn);
      for (int c = 0; c < nchunks; ++c) {
        const int q = lt * nchunks + c, r = q % R;
        T x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = xn[e];
        if (c + 1 < nchunks) loadChunk(c + 1, xn);
        uint32_t w[S][4];
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          uint32_t s0, s1;
          const uint64_t f0 = Fixed<T, S>::mag(x[e], emax, s0);
          const uint64_t f1 = Fixed<T, S>::mag(x[e + 1], emax, s1);
          digitPairs<S>(f0, s0, f1, s1, w, e >> 1);
        }
        // the MMAs that last read stage r must be done before it is overwritten
        if (q >= R && !wwait(&empty[r], (uint32_t)(q / R - 1) & 1u)) break;
        unsigned char *buf = sA + r * kBufBytes;
        const uint32_t off = part * kLboA + (srow >> 3) * 128 + (srow & 7) * 16;
#pragma unroll
        for (int i = 0; i < S; ++i)
          *reinterpret_cast<uint4 *>(buf + i * kSliceBytes + off) = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
        asm volatile("fence.proxy.async.shared::cta;");
        __syncwarp();
        if (lane == 0) arriveBar(&full[r]);
      }
      // With two stages the tile lags one behind: the next tile's split waits only for
      // the stage of the tile before this one, whose items are drained here.  With
      // one stage the next split waits for every item of this tile, which needs its
      // own accumulators drained first: drain it now.
      if (R == 1) {
        epilogue(lt, tile);
      } else {
        if (prev_tile >= 0) epilogue(lt - 1, prev_tile);
        prev_tile = tile;
      }
    }
    if (R == 2 && prev_tile >= 0 && !aborted()) epilogue(lt - 1, prev_tile);
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    int p = 0, lt = 0;
    for (int tile = blockIdx.x; tile < ntiles && !*abort; tile += gridDim.x, ++lt) {
      for (int j = 0; j < nb && !*abort; ++j, ++p) {
        const int st = p & 1;
        if (p >= 2 && !waitParityAbort(&accempty[st], (uint32_t)((p >> 1) - 1) & 1u, abort)) break;
        for (int c = 0; c < nchunks; ++c) {
          const int q = lt * nchunks + c, r = q % R;
          if (j == 0 && !waitParityAbort(&full[r], (uint32_t)(q / R) & 1u, abort)) break;
          asm volatile("tcgen05.fence::after_thread_sync;");
          const unsigned char *buf = sA + r * kBufBytes;
#pragma unroll 1
          for (int i = 1; i <= S; ++i) {
            const int ncols = NB * (S + 1 - i);
#pragma unroll 1
            for (int ks = 0; ks < kTcChunk / 16; ++ks) {
              const int kg = c * (kTcChunk / 16) + ks;
              const uint64_t da = matDesc(smemAddr(buf + (i - 1) * kSliceBytes + ks * 2 * kLboA), kLboA, 128);
              const uint64_t db = matDesc(smemAddr(sB) + j * blkBytes + kg * 2 * lboB, lboB, 128);
              mma(tmem + (uint32_t)(st * kAccCols + (i - 1) * NB), da, db, instrDesc(ncols),
                  (c > 0 || ks > 0 || i > 1) ? 1u : 0u);
            }
          }
          if (j == nb - 1) commit(&empty[r]);  // the stage's last reader
        }
        if (*abort) break;
        commit(&accfull[st]);
      }
    }
    // drain: every MMA issued (also on a failed run) must finish before tensor memory is released
    commit(&drain);
    uint32_t done = 0;
    const uint64_t t0 = nowNs();
    for (uint32_t it = 0; !done; ++it) {
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(done)
          : "r"(smemAddr(&drain)));
      if (!done && (it & 63u) == 63u && nowNs() - t0 > kPipeWaitNs) break;
    }
    if (!done) *abort = 1;
  }
  if (*abort && tid == 0) atomicExch(a.err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

template <typename T, int S, bool GATHER>
void launchPipe(const TcArgs<T> &a, cudaStream_t s) {
  const size_t blkBytes = (size_t)a.kpad * S * kPipeNB * 2;
  const size_t bufBytes = (size_t)S * kTcChunk * kTcRows * 2;
  const size_t smem = 1024 + ((blkBytes * a.nhalf + 1023) & ~(size_t)1023) + (a.stages == 1 ? 1 : 2) * bufBytes +
                      sizeof(int) * a.nhalf * kPipeNB +
                      (GATHER || !a.stage_out ? 0 : kPipeWorkers * 32 * kStagePitch * sizeof(T));
  cudaFuncSetAttribute(tc_pipe_kernel<T, S, GATHER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int64_t ntiles = (a.rows + kTcRows - 1) / kTcRows;
  const int grid = (int)(ntiles < a.nsm ? ntiles : a.nsm);
  tc_pipe_kernel<T, S, GATHER><<<grid, kPipeThreads, smem, s>>>(a);
}

}  // namespace

// f16 bit pattern of an integer digit, |v| <= 128 (exact: at most 8 significant bits).
static uint16_t halfOfDigit(int v) {
  if (v == 0) return 0;
  const uint16_t s = v < 0 ? 0x8000u : 0u;
  const unsigned a = (unsigned)(v < 0 ? -v : v);
  int e = 0;
  while ((a >> (e + 1)) != 0) ++e;  // leading bit
  return (uint16_t)(s | ((unsigned)(e + 15) << 10) | ((a << (10 - e)) & 0x3FFu));
}

// Host: digits of B (K x N, row-major in `b`) as the kernel's shared-memory image:
// per N block of NB columns, [K/8][S*NB][8] f16 (slice j rows (j-1)*NB..), and
// the per-column exponent t_n.
template <typename T>
void tc_build_b(const double *b, int K, int N, int kpad, int S, int NB, int nhalf, std::vector<uint16_t> &img,
                std::vector<int> &texp) {
  const int W = 8 * S - 2;  // fixed-point bits: below 2^(8S-2), so adding 0x80 per byte cannot carry out
  img.assign((size_t)nhalf * kpad * S * NB, 0);
  texp.assign((size_t)nhalf * NB, 0);
  uint64_t bias = 0;
  for (int j = 0; j < S; ++j) bias |= 0x80ull << (8 * j);
  // f16 patterns of every digit value -128 .. 128, built once
  static const std::vector<uint16_t> halfDigits = [] {
    std::vector<uint16_t> t(257);
    for (int v = -128; v <= 128; ++v) t[v + 128] = halfOfDigit(v);
    return t;
  }();
  for (int n = 0; n < N; ++n) {
    int emax = 1;
    for (int k = 0; k < K; ++k) {
      const double x = b[(size_t)k * N + n];
      uint64_t bits;
      std::memcpy(&bits, &x, 8);
      const int e = (int)((bits >> 52) & 0x7FF);
      emax = std::max(emax, e > 0 ? e : 1);
    }
    // column exponent: |B| < 2^(emax-1022)
    texp[n] = emax - 1022;
    const int h = n / NB, nl = n % NB;
    for (int k = 0; k < K; ++k) {
      const double x = b[(size_t)k * N + n];
      uint64_t bits;
      std::memcpy(&bits, &x, 8);
      const bool neg = (bits >> 63) != 0;
      const int e = (int)((bits >> 52) & 0x7FF);
      const uint64_t m = (bits & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
      const int sh = (e > 0 ? e : 1) - emax + (W - 53);
      const uint64_t f = sh >= 0 ? (m << sh) : (-sh >= 64 ? 0ull : (m >> (-sh)));
      const uint64_t y = f + bias;  // balanced digits: byte - 128
      for (int j = 1; j <= S; ++j) {
        const int dg = (int)((y >> (8 * (S - j))) & 0xFFu) - 128;
        const uint16_t bf = halfDigits[(neg ? -dg : dg) + 128];
        const int rowi = (j - 1) * NB + nl;
        const size_t off = (size_t)h * kpad * S * NB + (size_t)(k / 8) * (S * NB * 8) + (size_t)(rowi / 8) * 64 +
                           (size_t)(rowi % 8) * 8 + (k % 8);
        img[off] = bf;
      }
    }
  }
}

template <typename T>
void launch_tc_rows(const TcArgs<T> &a, cudaStream_t s) {
  launchPipe<T, tcDigits<T>(), false>(a, s);
}

// Scattering of pure zones on the tensor cores: K = N = groups (<= 64), rows
// gathered as (zone, moment) pairs, B = the material's order-l matrix transposed.
template <typename T>
void launch_tc_gather(const TcArgs<T> &a, cudaStream_t s) {
  launchPipe<T, tcDigits<T>(), true>(a, s);
}

template void tc_build_b<double>(const double *, int, int, int, int, int, int, std::vector<uint16_t> &, std::vector<int> &);
template void tc_build_b<float>(const double *, int, int, int, int, int, int, std::vector<uint16_t> &, std::vector<int> &);
template void launch_tc_rows<double>(const TcArgs<double> &, cudaStream_t);
template void launch_tc_rows<float>(const TcArgs<float> &, cudaStream_t);
template void launch_tc_gather<double>(const TcArgs<double> &, cudaStream_t);
template void launch_tc_gather<float>(const TcArgs<float> &, cudaStream_t);

}  // namespace kgb
