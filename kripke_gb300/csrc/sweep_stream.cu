// sweep_stream.cu -- the FP32 diamond-difference sweep with its slice operands
// streamed into shared memory by the Tensor Memory Accelerator.
//
// Same recurrence, schedule and results as the per-step kernel of sweep.cu
// (Kernel::sweepSubdomain, src/Kripke/Kernel/SweepSubdomain.cpp:86-108): tiles
// of TX x TY x tz zones on hyperplanes, one thread per (group, direction)
// chain, upwind faces in registers inside a tile and in the plane arrays
// between tiles.  What differs is how a k-slice's operands reach the block.
// The per-step kernel loads each cell's rhs and sigt when it sweeps the slice,
// so every slice starts with a memory round trip that a quarter-occupied SM
// cannot hide (the FP32 sweep measured about a quarter of HBM bandwidth).
// Here a block's 128 chains are whole groups (g0 .. g0+GB-1, every direction
// of the set), so the rhs of a whole slice of its tile is one box of the
// [nz][ny][nx][G][D] array -- {Ds directions, GB groups, TX zones, TY zones, 1}
// -- and its sigt one box of [nz][ny][nx][G]; one thread issues both copies
// for slice kk + ns while the block sweeps slice kk, so ns slices of operands
// are in flight per block, whatever the occupancy.  Boxes of partial tiles
// reach past the mesh (or start before it, in the reversed orientations) and
// read zeros there; those cells are not swept.
//
// Per cell the arithmetic is the per-step kernel's, written as the same
// expressions (the reference's association, the same contractions), and the
// fused population partial sums the cells in the same order, so psi, the
// planes and the partials are bit for bit those of sweep.cu at the same tiles.
//
// Synchronisation: stage s of ns holds slices s, s+ns, ...; the copy of a slice
// completes mbarrier full[s] (one arrival with the byte count); after a slice
// the block synchronises and thread 0 refills the stage it just left.  A wait
// is bounded (0.2 s of globaltimer); one that gives up sets *a.err and the
// block carries on with whatever the stage holds, so the launch ends and the
// host reports KGB_ERR_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "kgb_internal.h"
#include "sweep_common.h"

namespace kgb {

namespace {

constexpr uint64_t kStreamWaitNs = 200000000ull;  // 0.2 s

__device__ __forceinline__ uint32_t smemU32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t timerNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool waitStage(uint64_t *bar, uint32_t parity) {
  uint32_t done = 0;
  uint64_t t0 = 0;
  for (uint32_t it = 0; !done; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smemU32(bar)), "r"(parity)
        : "memory");
    if (!done && (it & 63u) == 63u) {
      const uint64_t t = timerNs();
      if (t0 == 0) t0 = t;
      else if (t - t0 > kStreamWaitNs) return false;
    }
  }
  return true;
}

// Bytes of one stage: the rhs box, then the sigt box (128-byte aligned)
__host__ __device__ __forceinline__ uint32_t rhsBoxBytes(int tx, int ty) { return (uint32_t)(tx * ty * kSweepThreads * 4); }
__host__ __device__ __forceinline__ uint32_t sigBoxBytes(int tx, int ty, int gb) { return (uint32_t)(tx * ty * gb * 4); }
__host__ __device__ __forceinline__ uint32_t stageBytes(int tx, int ty, int gb) {
  return rhsBoxBytes(tx, ty) + ((sigBoxBytes(tx, ty, gb) + 127u) & ~127u);
}

template <int TX, int TY, bool POP, int MINB>
__global__ void __launch_bounds__(kSweepThreads, MINB) sweep_stream_kernel(const __grid_constant__ SweepArgs<float> a,
                                                                   const __grid_constant__ CUtensorMap rmap,
                                                                   const __grid_constant__ CUtensorMap smap) {
  extern __shared__ __align__(128) unsigned char sraw[];
  __shared__ __align__(8) uint64_t full[kStreamMaxStages];
  const int ns = a.stream_ns;
  const int GB = kSweepThreads / a.Ds;  // groups per block
  const uint32_t rbytes = rhsBoxBytes(TX, TY), sbytes = sigBoxBytes(TX, TY, GB);
  const uint32_t stage = stageBytes(TX, TY, GB);
  const uint32_t sbase = smemU32(sraw);
  unsigned char *const al = sraw + (((sbase + 127u) & ~127u) - sbase);

  const int sdom = a.wave[blockIdx.z];
  const int tile = a.tile_off + blockIdx.y;
  const int cb = blockIdx.x;
  const SdomDesc sd = a.sdoms[sdom];
  const int sid = a.flip ? -sd.id : sd.id, sjd = a.flip ? -sd.jd : sd.jd, skd = a.flip ? -sd.kd : sd.kd;
  const int4 t = a.tiles[tile];
  const int nchain = a.Ds * a.Gs;
  const int c = cb * kSweepThreads + threadIdx.x;  // every block is full: Gs is a multiple of GB
  const int gl = c / a.Ds;
  const int g = sd.glo + gl;
  const int d = sd.dlo + (c - gl * a.Ds);
  const int g0 = sd.glo + cb * GB;
  const int lg = (int)threadIdx.x / a.Ds;  // group within the block

  const int ib = t.x * TX, jb = t.y * TY, kb = t.z * a.tz;
  // the boxes start at the tile's lowest global zone in i and j
  const int i0 = sd.io + (sid > 0 ? ib : a.nxs - ib - TX);
  const int j0 = sd.jo + (sjd > 0 ? jb : a.nys - jb - TY);
  const int kend = min(a.tz, a.nzs - kb);

  if (threadIdx.x == 0) {
    for (int s = 0; s < ns; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemU32(&full[s])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int kk, int s) {
    const int kq = kb + kk;
    const int kg = sd.ko + (skd > 0 ? kq : a.nzs - 1 - kq);
    const uint32_t dst = smemU32(al + (size_t)s * stage);
    const uint32_t bar = smemU32(&full[s]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(rbytes + sbytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"(&rmap), "r"(sd.dlo), "r"(g0), "r"(i0), "r"(j0), "r"(kg), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst + rbytes),
        "l"(&smap), "r"(g0), "r"(i0), "r"(j0), "r"(kg), "r"(bar)
        : "memory");
  };
  if (threadIdx.x == 0)
    for (int s = 0; s < ns && s < kend; ++s) issue(s, s);

  F32Acc pop;
  const double wd = POP ? a.w[d] : 0.0;
  const bool vu = a.vol_uniform > 0.0;
  // Per-thread bases and strides, so a cell costs few integer instructions:
  // psi of this chain at zone 0 and its stride between successive cells along i
  // of the sweep; the plane arrays at this chain, their k-slab strides and this
  // tile's row offsets within a slab; this thread's rhs and sigt entries of the
  // box for cell (ii, jj) at cells q0 + ii*qi + jj*qj of the box.
  const int64_t GD = (int64_t)a.G * a.D;
  float *const pchain = a.psi + (int64_t)g * a.D + d;
  const int64_t istep = sid > 0 ? GD : -GD;
  const int isg = sid > 0 ? 1 : -1;
  const int q0 = (sjd > 0 ? 0 : TY - 1) * TX + (sid > 0 ? 0 : TX - 1);
  const int qi = sid > 0 ? 1 : -1, qj = sjd > 0 ? TX : -TX;
  int jloc[TY], joff[TY], ioff[TX];
  bool iv[TX], jv[TY];
  float cxr[TX], cyr[TY];
  const int iloc0 = sid > 0 ? ib : a.nxs - 1 - ib;  // the tile's first cell along the sweep in i
#pragma unroll
  for (int ii = 0; ii < TX; ++ii) {
    const int ip = ib + ii;
    iv[ii] = ip < a.nxs;
    const int il = iloc0 + isg * ii;
    ioff[ii] = il * nchain;  // j-plane row of this i within a k-slab
    cxr[ii] = iv[ii] ? a.cx[(int64_t)d * a.nx + sd.io + il] : 0.f;
  }
#pragma unroll
  for (int jj = 0; jj < TY; ++jj) {
    const int jp = jb + jj;
    jv[jj] = jp < a.nys;
    jloc[jj] = sjd > 0 ? jp : a.nys - 1 - jp;
    joff[jj] = jloc[jj] * nchain;  // i-plane row of this j within a k-slab
    cyr[jj] = jv[jj] ? a.cy[(int64_t)d * a.ny + sd.jo + jloc[jj]] : 0.f;
  }
  float *const ipc = a.iplane + sd.ip + c;  // [nzs][nys][nchain]
  float *const jpc = a.jplane + sd.jp + c;  // [nzs][nxs][nchain]
  float *const kpc = a.kplane + sd.kp + c;  // [nys][nxs][nchain]
  const int64_t islab = (int64_t)a.nys * nchain, jslab = (int64_t)a.nxs * nchain;
  float bo[TX][TY];
#pragma unroll
  for (int ii = 0; ii < TX; ++ii)
#pragma unroll
    for (int jj = 0; jj < TY; ++jj)
      bo[ii][jj] = (iv[ii] && jv[jj]) ? kpc[(int64_t)jloc[jj] * jslab + ioff[ii]] : 0.f;
  // the incoming faces of a slice, loaded one slice ahead
  float lfn[TY], frn[TX];
  auto loadFaces = [&](int kk) {
    const int kq = kb + kk;
    const int k = skd > 0 ? kq : a.nzs - 1 - kq;
    const float *ik = ipc + (int64_t)k * islab;
    const float *jk = jpc + (int64_t)k * jslab;
#pragma unroll
    for (int jj = 0; jj < TY; ++jj) lfn[jj] = jv[jj] ? ik[joff[jj]] : 0.f;
#pragma unroll
    for (int ii = 0; ii < TX; ++ii) frn[ii] = iv[ii] ? jk[ioff[ii]] : 0.f;
  };
  if (kend > 0) loadFaces(0);

  bool ok = true;
  for (int kk = 0; kk < kend; ++kk) {
    const int s = kk % ns;
    const int kq = kb + kk;
    const int k = skd > 0 ? kq : a.nzs - 1 - kq;
    const float czk = a.cz[(int64_t)d * a.nz + sd.ko + k];
    float lfc[TY], fr[TX];
#pragma unroll
    for (int jj = 0; jj < TY; ++jj) lfc[jj] = lfn[jj];
#pragma unroll
    for (int ii = 0; ii < TX; ++ii) fr[ii] = frn[ii];
    if (kk + 1 < kend) loadFaces(kk + 1);
    if (!waitStage(&full[s], (uint32_t)(kk / ns) & 1u)) ok = false;
    const float *__restrict__ rs = reinterpret_cast<const float *>(al + (size_t)s * stage) + threadIdx.x;
    const float *__restrict__ ss = reinterpret_cast<const float *>(al + (size_t)s * stage + rbytes) + lg;
    float *const ik = ipc + (int64_t)k * islab;
    const int64_t zslice = (int64_t)(sd.ko + k) * a.ny;
#pragma unroll
    for (int jj = 0; jj < TY; ++jj) {
      if (!jv[jj]) continue;
      float lf = lfc[jj];
      const int64_t z0 = (zslice + (sd.jo + jloc[jj])) * a.nx + sd.io + iloc0;  // zone of cell (0, jj)
      float *pc = pchain + z0 * GD;
#pragma unroll
      for (int ii = 0; ii < TX; ++ii) {
        if (iv[ii]) {
          const int q = q0 + ii * qi + jj * qj;
          const float rv = rs[q * kSweepThreads];
          const float sv = ss[q * GB];
          // the per-step kernel's expressions (sweep.cu), so the two agree bit for bit
          const float num = rv + lf * cxr[ii] + fr[ii] * cyr[jj] + bo[ii][jj] * czk;
          const float den = cxr[ii] + cyr[jj] + czk + sv;
          const float ps = num / den;
          *pc = ps;
          lf = 2.f * ps - lf;
          fr[ii] = 2.f * ps - fr[ii];
          bo[ii][jj] = 2.f * ps - bo[ii][jj];
          if (POP) {
            if (vu) pop.add(ps);
            else pop.add((float)a.vol[z0 + isg * ii] * ps);
          }
        }
        pc += istep;
      }
      ik[joff[jj]] = lf;
    }
    float *const jk = jpc + (int64_t)k * jslab;
#pragma unroll
    for (int ii = 0; ii < TX; ++ii)
      if (iv[ii]) jk[ioff[ii]] = fr[ii];
    __syncthreads();  // every thread is done with stage s
    if (threadIdx.x == 0 && kk + ns < kend) issue(kk + ns, s);
  }
#pragma unroll
  for (int ii = 0; ii < TX; ++ii)
#pragma unroll
    for (int jj = 0; jj < TY; ++jj)
      if (iv[ii] && jv[jj]) kpc[(int64_t)jloc[jj] * jslab + ioff[ii]] = bo[ii][jj];
  if (!ok && a.err) atomicExch(a.err, 1);
  if (POP) {
    double v = pop.value() * wd;
    if (a.vol_uniform > 0.0) v *= a.vol_uniform;
    const double b = blockSum128(v);
    if (threadIdx.x == 0) a.pop[((int64_t)tile * a.nsdom + sdom) * gridDim.x + cb] = b;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 tensorMapEncoder() {
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

bool encode(CUtensorMap *m, const float *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides,
            const cuuint32_t *box) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = tensorMapEncoder();
  if (!fn) return false;
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, const_cast<float *>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int TX, int TY, bool POP, int MINB>
void launchStreamAs(const SweepArgs<float> &a, dim3 grid, cudaStream_t s, const CUtensorMap &rm,
                    const CUtensorMap &sm) {
  const size_t smem = (size_t)a.stream_ns * stageBytes(TX, TY, kSweepThreads / a.Ds) + 128;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(sweep_stream_kernel<TX, TY, POP, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  sweep_stream_kernel<TX, TY, POP, MINB><<<grid, kSweepThreads, smem, s>>>(a, rm, sm);
}

template <int TX, int TY, int MINB>
void launchStream(const SweepArgs<float> &a, dim3 grid, cudaStream_t s, const CUtensorMap &rm, const CUtensorMap &sm) {
  if (a.pop) launchStreamAs<TX, TY, true, MINB>(a, grid, s, rm, sm);
  else launchStreamAs<TX, TY, false, MINB>(a, grid, s, rm, sm);
}

}  // namespace

bool sweep_stream_applies(int D, int G, int Ds, int Gs, int tx, int ty) {
  const bool shape = tx == 4 && (ty == 4 || ty == 2);
  if (!shape || Ds < 4 || Ds > 32 || kSweepThreads % Ds != 0) return false;
  const int gb = kSweepThreads / Ds;  // 4 .. 32 groups per block: 16-byte sigt boxes
  return D % 4 == 0 && G % 4 == 0 && Gs % gb == 0;
}

bool launch_sweep_step_stream(const SweepArgs<float> &a, int ntiles, int nwave, cudaStream_t s) {
  const int gb = kSweepThreads / a.Ds;
  CUtensorMap rm, sm;
  const cuuint64_t rdims[5] = {(cuuint64_t)a.D, (cuuint64_t)a.G, (cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)a.nz};
  const cuuint64_t rstr[4] = {(cuuint64_t)a.D * 4, (cuuint64_t)a.G * a.D * 4, (cuuint64_t)a.nx * a.G * a.D * 4,
                              (cuuint64_t)a.ny * a.nx * a.G * a.D * 4};
  const cuuint32_t rbox[5] = {(cuuint32_t)a.Ds, (cuuint32_t)gb, (cuuint32_t)a.tx, (cuuint32_t)a.ty, 1};
  const cuuint64_t sdims[4] = {(cuuint64_t)a.G, (cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)a.nz};
  const cuuint64_t sstr[3] = {(cuuint64_t)a.G * 4, (cuuint64_t)a.nx * a.G * 4, (cuuint64_t)a.ny * a.nx * a.G * 4};
  const cuuint32_t sbox[4] = {(cuuint32_t)gb, (cuuint32_t)a.tx, (cuuint32_t)a.ty, 1};
  if (!encode(&rm, a.rhs, 5, rdims, rstr, rbox) || !encode(&sm, a.sigt, 4, sdims, sstr, sbox)) return false;
  const int nchain = a.Ds * a.Gs;
  dim3 grid(nchain / kSweepThreads, ntiles, nwave);
  // 4x2 at seven blocks per SM (72 registers, a few cold values spilled): 7.44
  // against 8.04 ms per 64^3 x 64-group x 128-direction sweep without the bound
  if (a.tx == 4 && a.ty == 4) launchStream<4, 4, 1>(a, grid, s, rm, sm);
  else launchStream<4, 2, 7>(a, grid, s, rm, sm);
  return true;
}

}  // namespace kgb
