// sweep_stream.cu -- the FP32 diamond-difference sweep with its slice operands
// streamed into shared memory by the Tensor Memory Accelerator.
//
// Same recurrence, schedule and results as the per-step kernel of sweep.cu
// (Kernel::sweepSubdomain, src/Kripke/Kernel/SweepSubdomain.cpp:86-108): tiles
// of TX x TY x tz zones on hyperplanes, one thread per (group, direction)
// chain, upwind faces in registers inside a tile and in the plane arrays
// between tiles.  What differs is how a k-slice's operands reach the block.
// The per-step kernel loads each cell's rhs and sigt and the slice's entering
// faces when it sweeps the slice, so every slice starts with a memory round
// trip that a quarter-occupied SM cannot hide (the FP32 sweep measured about a
// quarter of HBM bandwidth), and the faces it holds in registers bound the
// tile footprint.  Here a block's 128 chains are whole groups (g0 .. g0+GB-1,
// every direction of the set), so everything a slice reads is a handful of
// boxes: its rhs is one box of the [nz][ny][nx][G][D] array -- {Ds directions,
// GB groups, TX zones, TY zones, 1} -- its sigt one box of [nz][ny][nx][G],
// its entering i and j faces one box each of the plane arrays (TY and TX rows
// of the block's 128 chains), and the tile's entering k faces one box, loaded
// once.  One thread issues a slice's copies ns slices ahead of the block, so
// operands are in flight whatever the occupancy, and the entering faces need no
// registers until they are used, which lets a 4x4 footprint keep five blocks
// per SM.  Boxes of partial tiles reach past the mesh (or start before it, in
// the reversed orientations): zeros or other tiles' rows land in shared memory
// there, and those cells are not swept.
//
// Per cell the arithmetic is the per-step kernel's, written as the same
// expressions (the reference's association, the same contractions), and the
// fused population partial sums the cells in the same order, so psi, the
// planes and the partials are bit for bit those of sweep.cu at the same tiles.
//
// Synchronisation: stage s of ns holds slices s, s+ns, ...; the copies of a
// slice complete mbarrier full[s] (one arrival with the byte count); after a
// slice the block synchronises and thread 0 refills the stage it just left.
// The outgoing faces are plain stores: a face row is read by TMA only in the
// next hyperplane step's launch.  A wait is bounded (0.2 s of globaltimer);
// one that gives up sets *a.err and the block carries on with whatever the
// stage holds, so the launch ends and the host reports KGB_ERR_TIMEOUT.
//
// Measured on a 64^3-zone, 64-group, 128-direction mixed sweep (GB300): 6.3 ms
// at 4x4x8-16 tiles against 9.9 ms for the per-step kernel's best (4x2x16);
// L2 eviction hints (streamed operands first, faces last) measured 0.2-0.3 ms
// slower and are not used.
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

// Bytes of one stage: the rhs box, the sigt box (padded to 128 bytes), then
// the slice's entering i faces (TY rows of the block's bt chains) and j faces
// (TX rows).  The k faces of the tile have their own buffer, filled once.
// bt = chains per block (gb groups x Ds directions).
__host__ __device__ __forceinline__ uint32_t rhsBoxBytes(int tx, int ty, int bt) { return (uint32_t)(tx * ty * bt * 4); }
__host__ __device__ __forceinline__ uint32_t sigBoxBytes(int tx, int ty, int gb) { return (uint32_t)(tx * ty * gb * 4); }
__host__ __device__ __forceinline__ uint32_t faceRowBytes(int bt) { return (uint32_t)(bt * 4); }
__host__ __device__ __forceinline__ uint32_t stageBytes(int tx, int ty, int gb, int bt) {
  return rhsBoxBytes(tx, ty, bt) + ((sigBoxBytes(tx, ty, gb) + 127u) & ~127u) + (uint32_t)(tx + ty) * faceRowBytes(bt);
}
__host__ __device__ __forceinline__ uint32_t streamSmemBytes(int tx, int ty, int gb, int bt, int ns) {
  return (uint32_t)ns * stageBytes(tx, ty, gb, bt) + (uint32_t)(tx * ty) * faceRowBytes(bt) + 128u;
}

// The five boxes: rhs [nz][ny][nx][G][D] and sigt [nz][ny][nx][G] (global zones),
// and the plane arrays of every subdomain as rows of nchain values -- i planes
// [nsdom*nzs*nys][nchain], j planes [nsdom*nzs*nxs][nchain], k planes
// [nsdom*nys][nxs][nchain].
struct StreamMaps {
  CUtensorMap rhs, sig, ipl, jpl, kpl;
};

__device__ __forceinline__ void tmaLoad2(uint32_t dst, const CUtensorMap *m, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(m), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

template <int TX, int TY, bool POP, int MINB, int BT>
__global__ void __launch_bounds__(BT, MINB) sweep_stream_kernel(const __grid_constant__ SweepArgs<float> a,
                                                                   const __grid_constant__ StreamMaps maps) {
  extern __shared__ __align__(128) unsigned char sraw[];
  __shared__ __align__(8) uint64_t full[kStreamMaxStages], kbar;
  const int ns = a.stream_ns;
  // BT chains per block (GB whole groups), a compile-time constant so that the
  // per-cell shared-memory offsets are (measured: a runtime block size cost 10 %)
  const int GB = BT / a.Ds;
  const uint32_t rbytes = rhsBoxBytes(TX, TY, BT), sbytes = sigBoxBytes(TX, TY, GB);
  const uint32_t frow = faceRowBytes(BT);
  const uint32_t foff = rbytes + ((sbytes + 127u) & ~127u);  // the face rows within a stage
  const uint32_t stage = stageBytes(TX, TY, GB, BT);
  const uint32_t sbase = smemU32(sraw);
  unsigned char *const al = sraw + (((sbase + 127u) & ~127u) - sbase);
  const float *const kfs = reinterpret_cast<const float *>(al + (size_t)ns * stage);  // the tile's k faces

  const int sdom = a.wave[blockIdx.z];
  const int tile = a.tile_off + blockIdx.y;
  const int cb = blockIdx.x;
  const SdomDesc sd = a.sdoms[sdom];
  const int sid = a.flip ? -sd.id : sd.id, sjd = a.flip ? -sd.jd : sd.jd, skd = a.flip ? -sd.kd : sd.kd;
  const int4 t = a.tiles[tile];
  const int nchain = a.Ds * a.Gs;
  const int c = cb * BT + threadIdx.x;  // every block is full: Gs is a multiple of GB
  const int gl = c / a.Ds;
  const int g = sd.glo + gl;
  const int d = sd.dlo + (c - gl * a.Ds);
  const int g0 = sd.glo + cb * GB;
  const int lg = (int)threadIdx.x / a.Ds;  // group within the block

  const int ib = t.x * TX, jb = t.y * TY, kb = t.z * a.tz;
  // the tile's lowest zone in i and j within the zone set (boxes start there)
  const int ilo = sid > 0 ? ib : a.nxs - ib - TX;
  const int jlo = sjd > 0 ? jb : a.nys - jb - TY;
  const int kend = min(a.tz, a.nzs - kb);

  if (threadIdx.x == 0) {
    for (int s = 0; s < ns; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemU32(&full[s])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemU32(&kbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // plane rows of this subdomain's chunks
  const int irow0 = (int)(sd.ip / nchain), jrow0 = (int)(sd.jp / nchain), krow0 = (int)(sd.kp / ((int64_t)nchain * a.nxs));
  auto issue = [&](int kk, int s) {
    const int kq = kb + kk;
    const int k = skd > 0 ? kq : a.nzs - 1 - kq;
    const int kg = sd.ko + k;
    const uint32_t dst = smemU32(al + (size_t)s * stage);
    const uint32_t bar = smemU32(&full[s]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(rbytes + sbytes + (uint32_t)(TX + TY) * frow)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"(&maps.rhs), "r"(sd.dlo), "r"(g0), "r"(sd.io + ilo), "r"(sd.jo + jlo), "r"(kg), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst + rbytes),
        "l"(&maps.sig), "r"(g0), "r"(sd.io + ilo), "r"(sd.jo + jlo), "r"(kg), "r"(bar)
        : "memory");
    tmaLoad2(dst + foff, &maps.ipl, cb * BT, irow0 + k * a.nys + jlo, bar);
    tmaLoad2(dst + foff + TY * frow, &maps.jpl, cb * BT, jrow0 + k * a.nxs + ilo, bar);
  };
  if (threadIdx.x == 0) {
    const uint32_t kb_ = smemU32(&kbar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(kb_),
                 "r"((uint32_t)(TX * TY) * frow)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smemU32(kfs)),
        "l"(&maps.kpl), "r"(cb * BT), "r"(ilo), "r"(krow0 + jlo), "r"(kb_)
        : "memory");
    for (int s = 0; s < ns && s < kend; ++s) issue(s, s);
  }

  F32Acc pop;
  const double wd = POP ? a.w[d] : 0.0;
  const bool vu = a.vol_uniform > 0.0;
  // Per-thread bases and strides, so a cell costs few integer instructions:
  // psi of this chain at zone 0 and its stride between successive cells along i
  // of the sweep; the plane arrays at this chain, their k-slab strides and this
  // tile's row offsets within a slab; box positions of cell (ii, jj): q0 + ii*qi
  // + jj*qj, face row iq0 + ii*qi of the j faces, jq0 + jj*qjr of the i faces.
  const int64_t GD = (int64_t)a.G * a.D;
  float *const pchain = a.psi + (int64_t)g * a.D + d;
  const int64_t istep = sid > 0 ? GD : -GD;
  const int isg = sid > 0 ? 1 : -1;
  const int iq0 = sid > 0 ? 0 : TX - 1, jq0 = sjd > 0 ? 0 : TY - 1;
  const int qi = sid > 0 ? 1 : -1, qjr = sjd > 0 ? 1 : -1;
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

  bool ok = waitStage(&kbar, 0u);
  float bo[TX][TY];
#pragma unroll
  for (int ii = 0; ii < TX; ++ii)
#pragma unroll
    for (int jj = 0; jj < TY; ++jj)
      bo[ii][jj] = kfs[((jq0 + jj * qjr) * TX + iq0 + ii * qi) * BT + threadIdx.x];

  for (int kk = 0; kk < kend; ++kk) {
    const int s = kk % ns;
    const int kq = kb + kk;
    const int k = skd > 0 ? kq : a.nzs - 1 - kq;
    const float czk = a.cz[(int64_t)d * a.nz + sd.ko + k];
    if (!waitStage(&full[s], (uint32_t)(kk / ns) & 1u)) ok = false;
    const unsigned char *const st = al + (size_t)s * stage;
    const float *__restrict__ rs = reinterpret_cast<const float *>(st) + threadIdx.x;
    const float *__restrict__ ss = reinterpret_cast<const float *>(st + rbytes) + lg;
    const float *__restrict__ ifs = reinterpret_cast<const float *>(st + foff) + threadIdx.x;
    const float *__restrict__ jfs = reinterpret_cast<const float *>(st + foff + TY * frow) + threadIdx.x;
    float fr[TX];
#pragma unroll
    for (int ii = 0; ii < TX; ++ii) fr[ii] = jfs[(iq0 + ii * qi) * BT];
    float *const ik = ipc + (int64_t)k * islab;
    const int64_t zslice = (int64_t)(sd.ko + k) * a.ny;
#pragma unroll
    for (int jj = 0; jj < TY; ++jj) {
      if (!jv[jj]) continue;
      float lf = ifs[(jq0 + jj * qjr) * BT];
      const int64_t z0 = (zslice + (sd.jo + jloc[jj])) * a.nx + sd.io + iloc0;  // zone of cell (0, jj)
      float *pc = pchain + z0 * GD;
#pragma unroll
      for (int ii = 0; ii < TX; ++ii) {
        if (iv[ii]) {
          const int q = (jq0 + jj * qjr) * TX + iq0 + ii * qi;
          const float rv = rs[q * BT];
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
    const double b = blockSumWarps(v);
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

template <int TX, int TY, bool POP, int MINB, int BT>
void launchStreamAs(const SweepArgs<float> &a, dim3 grid, cudaStream_t s, const StreamMaps &m) {
  const size_t smem = streamSmemBytes(TX, TY, BT / a.Ds, BT, a.stream_ns);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(sweep_stream_kernel<TX, TY, POP, MINB, BT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  sweep_stream_kernel<TX, TY, POP, MINB, BT><<<grid, BT, smem, s>>>(a, m);
}

template <int TX, int TY, int MINB>
void launchStream(const SweepArgs<float> &a, dim3 grid, cudaStream_t s, const StreamMaps &m, int bt) {
  if (bt == 96) {
    if (a.pop) launchStreamAs<TX, TY, true, MINB, 96>(a, grid, s, m);
    else launchStreamAs<TX, TY, false, MINB, 96>(a, grid, s, m);
  } else {
    if (a.pop) launchStreamAs<TX, TY, true, MINB, 128>(a, grid, s, m);
    else launchStreamAs<TX, TY, false, MINB, 128>(a, grid, s, m);
  }
}

}  // namespace

int stream_block_chains(int Ds, int Gs) {
  // Whole groups per block, GB a multiple of 4 (16-byte sigt boxes) dividing the
  // group set, 128 or 96 chains (the kernel's two compiled block sizes): 4, 8, 16
  // or 32 directions per set fill 128 chains, 12 and 24 fill 96.
  if (Ds < 4 || Ds % 4 != 0 || Ds > kSweepThreads / 4) return 0;
  for (int gb = kSweepThreads / Ds / 4 * 4; gb >= 4; gb -= 4)
    if (Gs % gb == 0 && (gb * Ds == 128 || gb * Ds == 96)) return gb * Ds;
  return 0;
}

bool sweep_stream_applies(int D, int G, int Ds, int Gs, int tx, int ty) {
  const bool shape = tx == 4 && (ty == 4 || ty == 2);
  return shape && D % 4 == 0 && G % 4 == 0 && stream_block_chains(Ds, Gs) > 0;
}

bool launch_sweep_step_stream(const SweepArgs<float> &a, int ntiles, int nwave, cudaStream_t s) {
  const int bt = stream_block_chains(a.Ds, a.Gs), gb = bt / a.Ds;
  const cuuint64_t nch = (cuuint64_t)a.Ds * a.Gs, ns = (cuuint64_t)a.nsdom;
  StreamMaps m;
  const cuuint64_t rdims[5] = {(cuuint64_t)a.D, (cuuint64_t)a.G, (cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)a.nz};
  const cuuint64_t rstr[4] = {(cuuint64_t)a.D * 4, (cuuint64_t)a.G * a.D * 4, (cuuint64_t)a.nx * a.G * a.D * 4,
                              (cuuint64_t)a.ny * a.nx * a.G * a.D * 4};
  const cuuint32_t rbox[5] = {(cuuint32_t)a.Ds, (cuuint32_t)gb, (cuuint32_t)a.tx, (cuuint32_t)a.ty, 1};
  const cuuint64_t sdims[4] = {(cuuint64_t)a.G, (cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)a.nz};
  const cuuint64_t sstr[3] = {(cuuint64_t)a.G * 4, (cuuint64_t)a.nx * a.G * 4, (cuuint64_t)a.ny * a.nx * a.G * 4};
  const cuuint32_t sbox[4] = {(cuuint32_t)gb, (cuuint32_t)a.tx, (cuuint32_t)a.ty, 1};
  const cuuint64_t idims[2] = {nch, ns * a.nzs * a.nys}, jdims[2] = {nch, ns * a.nzs * a.nxs};
  const cuuint64_t kdims[3] = {nch, (cuuint64_t)a.nxs, ns * a.nys};
  const cuuint64_t pstr[2] = {nch * 4, nch * 4 * a.nxs};
  const cuuint32_t ibox[2] = {(cuuint32_t)bt, (cuuint32_t)a.ty}, jbox[2] = {(cuuint32_t)bt, (cuuint32_t)a.tx};
  const cuuint32_t kbox[3] = {(cuuint32_t)bt, (cuuint32_t)a.tx, (cuuint32_t)a.ty};
  if (!encode(&m.rhs, a.rhs, 5, rdims, rstr, rbox) || !encode(&m.sig, a.sigt, 4, sdims, sstr, sbox) ||
      !encode(&m.ipl, a.iplane, 2, idims, pstr, ibox) || !encode(&m.jpl, a.jplane, 2, jdims, pstr, jbox) ||
      !encode(&m.kpl, a.kplane, 3, kdims, pstr, kbox))
    return false;
  dim3 grid((unsigned)(nch / bt), ntiles, nwave);
  // occupancy bounds: 4x4 at five blocks per SM (92 registers), 4x2 at seven (72)
  if (a.tx == 4 && a.ty == 4) launchStream<4, 4, 5>(a, grid, s, m, bt);
  else launchStream<4, 2, 7>(a, grid, s, m, bt);
  return true;
}

}  // namespace kgb
