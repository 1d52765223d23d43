// sweep.cu -- diamond-difference transport sweep on GB300.
//
// Replaces Kernel::sweepSubdomain (src/Kripke/Kernel/SweepSubdomain.cpp:26-111,
// CUDA policy Arch/SweepSubdomains.h:246-269).  Per cell, in upwind order:
//   psi = (rhs + psi_lf*2mu/dx + psi_fr*2eta/dy + psi_bo*2xi/dz)
//         / (2mu/dx + 2eta/dy + 2xi/dz + sigt)
//   psi_lf = 2 psi - psi_lf, psi_fr = 2 psi - psi_fr, psi_bo = 2 psi - psi_bo
// evaluated with the reference's association ((rhs + a)+b)+c and ((x+y)+z)+s.
//
// Schedule: a subdomain's zone set is cut into tiles of tx x ty x tz
// zones.  In the sweep's own orientation a tile (a,b,c) depends only on
// (a-1,b,c), (a,b-1,c), (a,b,c-1), so all tiles with a+b+c = step form a
// hyperplane that runs concurrently; one step sweeps one tile hyperplane of
// every subdomain in the wave (all eight octants at once), launched in parts
// on separate streams so one part's last partial wave of blocks runs beside
// the other parts' blocks (the caller's choice).  Inside a tile each
// thread owns one (group, direction) chain and walks the tile's cells in
// upwind order; its upwind faces stay in registers (psi_lf one value, psi_fr
// one per tile column, psi_bo one per tile column x row).  The reference's
// i/j/k plane fields are the running face buffers between tiles, with chains
// fastest, so every global access of a warp is a contiguous run.
//
// FP64 on GB300 issues at 1/61 of the FP32 rate and one IEEE divide costs
// about ten FP64 slots (in FP32 the divide's latency sits on the cell-to-cell
// dependency chain), so on a uniform mesh the denominator's reciprocal is
// tabulated per (sigt class, direction): den = ((cx+cy)+cz) + sigt is formed
// exactly as per cell (same operands, same association, same precision) and
// rounded once to 1/den; the cell then multiplies (psi differs from num/den by
// at most 1.5 ulp).
//
// The transposed (adjoint) sweep is the same recurrence run from the opposite
// corner (flip): along a direction the diamond-difference coupling of two
// cells is a product of 2c/den and -1 face factors, and read backwards it
// differs only in which end's c = 2|cos|/delta enters, so on a mesh with
// varying spacing the transpose is the reversed sweep conjugated by the cell
// volumes, which the caller applies.
//
// The tile body is a device function shared by the per-step launches here
// and by the persistent batched sweep (batch.cu), which passes COH = true to
// read the running face planes through L2 only: there the tiles of one step
// read faces written by other blocks earlier in the same launch.
//
// The population edit (Kernel::population) is fused: each thread accumulates
// volume * psi over its cells (FP64, or compensated FP32 in the mixed form),
// scales by w(d), and each block writes one partial; a fixed-order reduction
// over the partials follows the sweep.
//
// In the mixed form the LPlusTimes that precedes the sweep
// (SteadyStateSolver.cpp:69-71) can be fused too (FUSE): a thread keeps its
// direction's row of ell_plus in registers and forms each cell's rhs from the
// zone's phi_out moments in the order the SIMT LPlusTimes kernel sums them
// (ascending moment, one FMA chain), so the swept psi is bit-for-bit that of
// the unfused iteration while rhs is neither written nor read.
#include "kgb_internal.h"
#include "sweep_common.h"

namespace kgb {

namespace {

template <bool COH, typename T>
__device__ __forceinline__ T ldFace(const T *p) {
  if constexpr (COH) return __ldcg(p);
  else return *p;
}

// Asynchronous copy of one element into this thread's own shared-memory slot.
template <typename T>
__device__ __forceinline__ void cpAsync(T *dst, const T *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src),
               "n"((int)sizeof(T))
               : "memory");
}

// Row exponent bound for the next LTimes: the largest biased exponent of the
// row's psi among the rexp_w lanes that share this group (the lanes of one
// group and direction set are consecutive chains, aligned to rexp_w), folded
// into rowexp by one lane with an atomic max.  One warp reduction per run of
// rexp_w lanes (each run names only its own lanes); four shuffle steps
// instead cost the FP64 sweep of a 64^3-zone, 64-group, 128-direction
// problem 1.1 ms per iteration, this 0.3.
__device__ __forceinline__ void rowExpMax(int *rowexp, int w, unsigned mask, double ps, int64_t row) {
  const unsigned ex = (unsigned)((__double_as_longlong(ps) >> 52) & 0x7FFu);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned run = w >= 32 ? mask : (((1u << w) - 1u) << (lane & ~(unsigned)(w - 1))) & mask;
  const unsigned m = __reduce_max_sync(run, ex);
  if ((lane & (unsigned)(w - 1)) == 0) atomicMax(rowexp + row, (int)m);
}

}  // namespace

// One tile of one subdomain for one block of chains: tile is the index into
// a.tiles, cb the chain block (chains cb*blockDim.x + threadIdx.x) of ncb.
// Shared-memory slots per k-slice of the operand streaming (PFM 0: none,
// 1: rhs only, 2: rhs, the incoming faces of per-step launches and sigt for
// footprints up to 4x2, which keeps the buffers within 48 KB of static
// shared memory); the buffers hold two slices.
template <int TX, int TY, bool RECIP, bool COH, int PFM>
constexpr int sweepSlots() {
  return PFM == 0 ? 0
                  : TX * TY + (PFM == 2 && TX * TY <= 8 && !COH ? TX + TY : 0) +
                        (PFM == 2 && TX * TY <= 8 && !RECIP ? TX * TY : 0);
}

template <typename T, int TX, int TY, bool RECIP, bool POP, bool COH, bool FUSE = false, int PFM = 0, bool LTF = false>
__device__ __forceinline__ void sweepTile(const SweepArgs<T> &a, const int sdom, const int tile, const int cb,
                                          const int ncb, T (*rbuf)[kSweepThreads] = nullptr,
                                          T (*ltb)[kSweepThreads] = nullptr) {
  // LTF: every thread of the block owns a chain (the caller launches it only when the
  // chain count is a multiple of the block), so the slice barriers below are block-wide
  static_assert(!LTF || (!COH && !FUSE && PFM == 0), "fused LTimes: per-step mixed sweep only");
  const SdomDesc sd = a.sdoms[sdom];
  // the adjoint sweep (transposed operator) runs every direction in its reversed orientation
  const int sid = a.flip ? -sd.id : sd.id, sjd = a.flip ? -sd.jd : sd.jd, skd = a.flip ? -sd.kd : sd.kd;
  const int4 t = a.tiles[tile];
  const int nchain = a.Ds * a.Gs;
  const int c = cb * blockDim.x + threadIdx.x;
  typename AccOf<T>::type pop;
  double wd = 0.0;
  if (c < nchain) {
    // this warp's lanes with a chain (whole groups of rexp_w lanes)
    const int nlive = nchain - (c - (int)(threadIdx.x & 31u));
    const unsigned rmask = nlive >= 32 ? 0xffffffffu : ((1u << nlive) - 1u);
    const int gl = c / a.Ds;
    const int dl = c - gl * a.Ds;
    const int g = sd.glo + gl;
    const int d = sd.dlo + dl;
    if (POP) wd = a.w[d];

    // Oriented coordinates i' run along the sweep; i = id > 0 ? i' : nxs-1-i'.
    // Partial tiles only occur at the downwind end, so an invalid cell never
    // precedes a valid one in a row.
    const int ib = t.x * TX, jb = t.y * TY, kb = t.z * a.tz;
    int iloc[TX], jloc[TY];
    bool iv[TX], jv[TY];
    T cxr[TX], cyr[TY];
#pragma unroll
    for (int ii = 0; ii < TX; ++ii) {
      const int ip = ib + ii;
      iv[ii] = ip < a.nxs;
      iloc[ii] = sid > 0 ? ip : a.nxs - 1 - ip;
      cxr[ii] = iv[ii] ? a.cx[(int64_t)d * a.nx + sd.io + iloc[ii]] : T(0);
    }
#pragma unroll
    for (int jj = 0; jj < TY; ++jj) {
      const int jp = jb + jj;
      jv[jj] = jp < a.nys;
      jloc[jj] = sjd > 0 ? jp : a.nys - 1 - jp;
      cyr[jj] = jv[jj] ? a.cy[(int64_t)d * a.ny + sd.jo + jloc[jj]] : T(0);
    }

    T *const ipl = a.iplane + sd.ip;  // [nzs][nys][nchain]
    T *const jpl = a.jplane + sd.jp;  // [nzs][nxs][nchain]
    T *const kpl = a.kplane + sd.kp;  // [nys][nxs][nchain]

    T bo[TX][TY];
#pragma unroll
    for (int ii = 0; ii < TX; ++ii)
#pragma unroll
      for (int jj = 0; jj < TY; ++jj)
        bo[ii][jj] = (iv[ii] && jv[jj]) ? ldFace<COH>(kpl + ((int64_t)jloc[jj] * a.nxs + iloc[ii]) * nchain + c) : T(0);

    T ep[FUSE ? kFuseMaxM : 1];
    if constexpr (FUSE) {
#pragma unroll
      for (int m = 0; m < kFuseMaxM; ++m) ep[m] = m < a.M ? a.ellp[(int64_t)d * a.M + m] : T(0);
    }
    const T *__restrict__ rhs = a.rhs;
    T *__restrict__ psi = a.psi;
    const int kend = min(a.tz, a.nzs - kb);
    // FP64: the next k-slice's operands stream into shared memory (each thread
    // its own slots, rbuf[2 * kSlots][threads] from the kernel) while this slice
    // is swept, so a slice's first cell does not wait on memory (measured 34.0 ->
    // 32.8 ms per 64^3 sweep with rhs alone, 32.1 with faces and sigt classes;
    // the FP32 sweep, bound by its chain latency rather than the FP64 pipe, ran
    // slower with it).  Faces only in per-step launches: in the persistent
    // batched sweep a face address is rewritten by other SMs within the launch
    // and must be read through L2.
    static_assert(PFM == 0 || !FUSE, "the fused prologue forms rhs itself");
    constexpr bool PF = PFM > 0;
    constexpr bool PFX = PFM == 2 && TX * TY <= 8;
    constexpr int kFaces = PFX && !COH ? TX + TY : 0, kSig = PFX && !RECIP ? TX * TY : 0;
    constexpr int kSlots = sweepSlots<TX, TY, RECIP, COH, PFM>();
    static_assert(kSlots == TX * TY + kFaces + kSig || !PF, "slot layout");
    auto slot = [&](int buf, int i) -> T & { return rbuf[buf * kSlots + i][threadIdx.x]; };
    int cn[TY][TX];  // RECIP: the next slice's sigt classes, loaded a slice ahead
    auto prefetchSlice = [&](int kk2, int buf) {
      const int kq2 = kb + kk2;
      const int k2 = skd > 0 ? kq2 : a.nzs - 1 - kq2;
      const int64_t zs2 = (int64_t)(sd.ko + k2) * a.ny;
#pragma unroll
      for (int jj = 0; jj < TY; ++jj) {
        const int64_t zrow2 = (zs2 + (sd.jo + jloc[jj])) * a.nx + sd.io;
#pragma unroll
        for (int ii = 0; ii < TX; ++ii)
          if (iv[ii] && jv[jj]) {
            const int64_t zg = (zrow2 + iloc[ii]) * a.G + g;
            cpAsync(&slot(buf, jj * TX + ii), rhs + zg * a.D + d);
            if constexpr (RECIP) cn[jj][ii] = a.cls[zg];
            else if constexpr (kSig > 0) cpAsync(&slot(buf, TX * TY + kFaces + jj * TX + ii), a.sigt + zg);
          }
      }
      if constexpr (kFaces > 0) {
#pragma unroll
        for (int ii = 0; ii < TX; ++ii)
          if (iv[ii]) cpAsync(&slot(buf, TX * TY + ii), jpl + ((int64_t)k2 * a.nxs + iloc[ii]) * nchain + c);
#pragma unroll
        for (int jj = 0; jj < TY; ++jj)
          if (jv[jj])
            cpAsync(&slot(buf, TX * TY + TX + jj), ipl + ((int64_t)k2 * a.nys + jloc[jj]) * nchain + c);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    if constexpr (PF) prefetchSlice(0, 0);
    for (int kk = 0; kk < kend; ++kk) {
      const int kq = kb + kk;
      const int k = skd > 0 ? kq : a.nzs - 1 - kq;
      int cc[TY][TX];  // RECIP: this slice's sigt classes
      if constexpr (PF && RECIP) {
#pragma unroll
        for (int jj = 0; jj < TY; ++jj)
#pragma unroll
          for (int ii = 0; ii < TX; ++ii) cc[jj][ii] = cn[jj][ii];
      }
      if constexpr (PF) {
        if (kk + 1 < kend) {
          prefetchSlice(kk + 1, (kk + 1) & 1);
          asm volatile("cp.async.wait_group 1;" ::: "memory");  // this slice's copies have landed
        } else {
          asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
      }
      const T czk = a.cz[(int64_t)d * a.nz + sd.ko + k];
      T pv[LTF ? TY : 1][LTF ? TX : 1];  // LTF: this slice's psi values (0 at cells off the mesh)
      if constexpr (LTF) {
#pragma unroll
        for (int jj = 0; jj < TY; ++jj)
#pragma unroll
          for (int ii = 0; ii < TX; ++ii) pv[jj][ii] = T(0);
      }
      // The slice's loads do not depend on the upwind chain: issue them all
      // before the first cell so their latency overlaps.
      T rv[TY][TX], sv[TY][TX];
      const int64_t zslice = (int64_t)(sd.ko + k) * a.ny;
#pragma unroll
      for (int jj = 0; jj < TY; ++jj) {
        const int64_t zrow = (zslice + (sd.jo + jloc[jj])) * a.nx + sd.io;
#pragma unroll
        for (int ii = 0; ii < TX; ++ii) {
          const int64_t z = zrow + iloc[ii];
          if (iv[ii] && jv[jj]) {
            if constexpr (FUSE) {
              // unconditional loads (the index is clamped to the row; beyond M the
              // coefficient is zero and the FMA leaves the sum unchanged) so the
              // compiler can issue them ahead of the chain
              const T *__restrict__ ph = a.phiout + (z * a.G + g) * a.M;
              const int mlast = a.M - 1;
              T acc = T(0);
#pragma unroll
              for (int m = 0; m < kFuseMaxM; ++m) acc += ep[m] * __ldg(ph + min(m, mlast));
              rv[jj][ii] = acc;
            } else if constexpr (PF) {
              rv[jj][ii] = slot(kk & 1, jj * TX + ii);
            } else {
              rv[jj][ii] = rhs[(z * a.G + g) * a.D + d];
            }
            if constexpr (PF) {
              if constexpr (RECIP) sv[jj][ii] = a.inv[(int64_t)cc[jj][ii] * a.D + d];
              else if constexpr (kSig > 0) sv[jj][ii] = slot(kk & 1, TX * TY + kFaces + jj * TX + ii);
              else sv[jj][ii] = a.sigt[z * a.G + g];
            } else if (RECIP) {
              sv[jj][ii] = a.inv[(int64_t)a.cls[z * a.G + g] * a.D + d];
            } else {
              sv[jj][ii] = a.sigt[z * a.G + g];
            }
          } else {
            rv[jj][ii] = T(0);
            sv[jj][ii] = T(1);
          }
        }
      }
      T fr[TX];
#pragma unroll
      for (int ii = 0; ii < TX; ++ii) {
        if constexpr (kFaces > 0) fr[ii] = iv[ii] ? slot(kk & 1, TX * TY + ii) : T(0);
        else fr[ii] = iv[ii] ? ldFace<COH>(jpl + ((int64_t)k * a.nxs + iloc[ii]) * nchain + c) : T(0);
      }
#pragma unroll
      for (int jj = 0; jj < TY; ++jj) {
        if (!jv[jj]) continue;
        const int j = jloc[jj];
        T *const lfp = ipl + ((int64_t)k * a.nys + j) * nchain + c;
        T lf;
        if constexpr (kFaces > 0) lf = slot(kk & 1, TX * TY + TX + jj);
        else lf = ldFace<COH>(lfp);
        const int64_t zrow = (zslice + (sd.jo + j)) * a.nx + sd.io;
#pragma unroll
        for (int ii = 0; ii < TX; ++ii) {
          if (!iv[ii]) continue;
          const int64_t z = zrow + iloc[ii];
          const int64_t e = (z * a.G + g) * a.D + d;
          const T num = rv[jj][ii] + lf * cxr[ii] + fr[ii] * cyr[jj] + bo[ii][jj] * czk;
          T ps;
          if (RECIP) {
            ps = num * sv[jj][ii];
          } else {
            const T den = cxr[ii] + cyr[jj] + czk + sv[jj][ii];
            ps = num / den;
          }
          psi[e] = ps;
          if constexpr (LTF) pv[jj][ii] = ps;
          if constexpr (sizeof(T) == 8) {
            if (a.rowexp) rowExpMax(a.rowexp, a.rexp_w, rmask, ps, z * a.G + g);
          }
          lf = T(2) * ps - lf;
          fr[ii] = T(2) * ps - fr[ii];
          bo[ii][jj] = T(2) * ps - bo[ii][jj];
          if (POP) {
            if (a.vol_uniform > 0.0) pop.add(ps);
            else pop.add((T)a.vol[z] * ps);
          }
        }
        *lfp = lf;
      }
#pragma unroll
      for (int ii = 0; ii < TX; ++ii)
        if (iv[ii]) jpl[((int64_t)k * a.nxs + iloc[ii]) * nchain + c] = fr[ii];
      if constexpr (LTF) {
        // The slice's moments of this subdomain: the block's psi values go to shared
        // memory (two buffers, alternating by slice, so one barrier per slice), then each
        // thread takes (group, moment) pairs of the block's chains and, for every cell,
        // sums ell[d][m] psi over the group's directions in the block (ascending), and
        // adds the sum to phiacc.
        T(*sm)[kSweepThreads] = ltb + (kk & 1) * (TX * TY);
#pragma unroll
        for (int jj = 0; jj < TY; ++jj)
#pragma unroll
          for (int ii = 0; ii < TX; ++ii) sm[jj * TX + ii][threadIdx.x] = pv[jj][ii];
        __syncthreads();
        const int c0 = cb * (int)blockDim.x;
        const int gfirst = c0 / a.Ds, glast = (c0 + (int)blockDim.x - 1) / a.Ds;
        const int npair = (glast - gfirst + 1) * a.M;
        for (int p = threadIdx.x; p < npair; p += blockDim.x) {
          const int gi = p / a.M, m = p - gi * a.M;
          const int gl2 = gfirst + gi;
          const int cs = max(gl2 * a.Ds, c0), ce = min(gl2 * a.Ds + a.Ds, c0 + (int)blockDim.x);
          T acc[TY][TX];
#pragma unroll
          for (int jj = 0; jj < TY; ++jj)
#pragma unroll
            for (int ii = 0; ii < TX; ++ii) acc[jj][ii] = T(0);
          for (int ch = cs; ch < ce; ++ch) {
            const T e = a.ell[(int64_t)(sd.dlo + ch - gl2 * a.Ds) * a.M + m];
#pragma unroll
            for (int jj = 0; jj < TY; ++jj)
#pragma unroll
              for (int ii = 0; ii < TX; ++ii) acc[jj][ii] += e * sm[jj * TX + ii][ch - c0];
          }
          const int64_t gz = sd.glo + gl2;
#pragma unroll
          for (int jj = 0; jj < TY; ++jj)
#pragma unroll
            for (int ii = 0; ii < TX; ++ii)
              if (iv[ii] && jv[jj]) {
                const int64_t z = (zslice + (sd.jo + jloc[jj])) * a.nx + sd.io + iloc[ii];
                atomicAdd(a.phiacc + (z * a.G + gz) * a.M + m, acc[jj][ii]);
              }
        }
      }
    }
#pragma unroll
    for (int ii = 0; ii < TX; ++ii)
#pragma unroll
      for (int jj = 0; jj < TY; ++jj)
        if (iv[ii] && jv[jj]) kpl[((int64_t)jloc[jj] * a.nxs + iloc[ii]) * nchain + c] = bo[ii][jj];
  }
  if (POP) {
    double v = pop.value() * wd;
    if (a.vol_uniform > 0.0) v *= a.vol_uniform;
    const double b = blockSum128(v);
    if (threadIdx.x == 0) a.pop[((int64_t)tile * a.nsdom + sdom) * ncb + cb] = b;
  }
}

template <typename T, int TX, int TY, bool RECIP, bool POP, bool FUSE = false, bool LTF = false>
__global__ void __launch_bounds__(kSweepThreads) sweep_step_kernel(const __grid_constant__ SweepArgs<T> a) {
  constexpr int PFM = (sizeof(T) == 8 && !FUSE && !LTF) ? 2 : 0;
  constexpr int kSlots = sweepSlots<TX, TY, RECIP, false, PFM>();
  __shared__ T rbuf[kSlots > 0 ? 2 * kSlots : 1][kSweepThreads];
  __shared__ T ltb[LTF ? 2 * TX * TY : 1][kSweepThreads];
  sweepTile<T, TX, TY, RECIP, POP, false, FUSE, PFM, LTF>(a, a.wave[blockIdx.z], a.tile_off + blockIdx.y,
                                                          blockIdx.x, gridDim.x, rbuf, ltb);
}

namespace {
__device__ __forceinline__ unsigned long long globalNs() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative launch (all blocks resident): arrivals
// are counted in bar[0]; the last block resets the count and advances the
// generation bar[1], which the others wait on -- for at most limit_ns
// (globaltimer), after which they record the failure in *err and go on.
// Once *err is set no block waits any more, so a failed launch ends quickly;
// its outputs are then undefined, but every access stays where it would be.
__device__ __forceinline__ void gridBarrier(unsigned int *bar, unsigned int nblocks, int *err,
                                            unsigned long long limit_ns) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int *gen = bar + 1;
    volatile int *failed = err;
    const unsigned int g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == nblocks - 1u) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const unsigned long long t0 = globalNs();
      while (*gen == g && !*failed) {
        __nanosleep(64);
        if (globalNs() - t0 >= limit_ns) {
          atomicExch(err, 1);
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
}
}  // namespace

// Persistent sweep of many independent problems: every block takes work items
// of the current global step (one tile of one subdomain for one chain block
// of one problem); a grid barrier separates the steps.  Faces between tiles
// move through the plane arrays, read through L2.
template <typename T, int TX, int TY>
__global__ void __launch_bounds__(kSweepThreads) batch_sweep_kernel(const SweepArgs<T> *__restrict__ inst,
                                                                   const BatchSweepPlan p) {
  // FP64: rhs of the next slice streamed into shared memory (read-only in the launch);
  // one buffer serves both sigt variants (their slot counts agree for rhs only)
  constexpr int PFM = sizeof(T) == 8 ? 1 : 0;
  constexpr int kSlots = sweepSlots<TX, TY, true, true, PFM>();
  static_assert(kSlots == sweepSlots<TX, TY, false, true, PFM>(), "one buffer for both variants");
  __shared__ T rbuf[kSlots > 0 ? 2 * kSlots : 1][kSweepThreads];
  const unsigned int nb = gridDim.x;
  for (int i = blockIdx.x; i < p.nzero; i += gridDim.x) {
    const BatchZero z = p.zero[i];
    const SweepArgs<T> &a = inst[z.inst];
    if (z.plane == 3) {  // the problem's psi row-exponent record
      for (int64_t e = z.begin + threadIdx.x; e < z.end; e += blockDim.x) a.rowexp[e] = 0;
      continue;
    }
    T *base = z.plane == 0 ? a.iplane : (z.plane == 1 ? a.jplane : a.kplane);
    for (int64_t e = z.begin + threadIdx.x; e < z.end; e += blockDim.x) base[e] = T(0);
  }
  gridBarrier(p.bar, nb, p.err, p.wait_ns);
  for (int st = 0; st < p.nsteps; ++st) {
    for (int i = p.step_off[st] + blockIdx.x; i < p.step_off[st + 1]; i += gridDim.x) {
      const int4 w = p.items[i];
      const SweepArgs<T> &a = inst[w.x];
      const int ncb = (a.Ds * a.Gs + kSweepThreads - 1) / kSweepThreads;
      if (a.cls != nullptr) sweepTile<T, TX, TY, true, true, true, false, PFM>(a, w.y, w.z, w.w, ncb, rbuf);
      else sweepTile<T, TX, TY, false, true, true, false, PFM>(a, w.y, w.z, w.w, ncb, rbuf);
    }
    gridBarrier(p.bar, nb, p.err, p.wait_ns);
  }
}

namespace {
template <typename T, int TX, int TY, bool FUSE>
void launchTileAs(const SweepArgs<T> &a, dim3 grid, cudaStream_t s) {
  const bool recip = a.cls != nullptr && a.inv != nullptr;
  const bool pop = a.pop != nullptr;
  if (recip && pop) sweep_step_kernel<T, TX, TY, true, true, FUSE><<<grid, kSweepThreads, 0, s>>>(a);
  else if (recip) sweep_step_kernel<T, TX, TY, true, false, FUSE><<<grid, kSweepThreads, 0, s>>>(a);
  else if (pop) sweep_step_kernel<T, TX, TY, false, true, FUSE><<<grid, kSweepThreads, 0, s>>>(a);
  else sweep_step_kernel<T, TX, TY, false, false, FUSE><<<grid, kSweepThreads, 0, s>>>(a);
}
// the fused LPlusTimes prologue and LTimes epilogue exist for the mixed form only
template <typename T, int TX, int TY>
void launchTile(const SweepArgs<T> &a, dim3 grid, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (a.phiout != nullptr) return launchTileAs<T, TX, TY, true>(a, grid, s);
    if (a.phiacc != nullptr && a.pop != nullptr) {  // the epilogue rides on the fused population
      const bool recip = a.cls != nullptr && a.inv != nullptr;
      if (recip) sweep_step_kernel<T, TX, TY, true, true, false, true><<<grid, kSweepThreads, 0, s>>>(a);
      else sweep_step_kernel<T, TX, TY, false, true, false, true><<<grid, kSweepThreads, 0, s>>>(a);
      return;
    }
  }
  launchTileAs<T, TX, TY, false>(a, grid, s);
}
}  // namespace

template <typename T>
void launch_sweep_step(const SweepArgs<T> &a, int ntiles, int nwave, cudaStream_t s) {
  const int nchain = a.Ds * a.Gs;
  dim3 grid((nchain + kSweepThreads - 1) / kSweepThreads, ntiles, nwave);
  if (a.tx == 4 && a.ty == 4) launchTile<T, 4, 4>(a, grid, s);
  else if (a.tx == 4 && a.ty == 2) launchTile<T, 4, 2>(a, grid, s);
  else launchTile<T, 2, 2>(a, grid, s);
}

template <typename T>
int batch_sweep_grid(int tx, int ty, int nsm) {
  int nb = 0;
  if (tx == 4 && ty == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_sweep_kernel<T, 4, 4>, kSweepThreads, 0);
  else if (tx == 4 && ty == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_sweep_kernel<T, 4, 2>, kSweepThreads, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_sweep_kernel<T, 2, 2>, kSweepThreads, 0);
  return nb * nsm;
}

template <typename T>
cudaError_t launch_batch_sweep(const SweepArgs<T> *inst, const BatchSweepPlan &p, int tx, int ty, int grid,
                               cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kSweepThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (tx == 4 && ty == 4) return cudaLaunchKernelEx(&cfg, batch_sweep_kernel<T, 4, 4>, inst, p);
  if (tx == 4 && ty == 2) return cudaLaunchKernelEx(&cfg, batch_sweep_kernel<T, 4, 2>, inst, p);
  return cudaLaunchKernelEx(&cfg, batch_sweep_kernel<T, 2, 2>, inst, p);
}

template int batch_sweep_grid<double>(int, int, int);
template int batch_sweep_grid<float>(int, int, int);
template cudaError_t launch_batch_sweep<double>(const SweepArgs<double> *, const BatchSweepPlan &, int, int, int,
                                                cudaStream_t);
template cudaError_t launch_batch_sweep<float>(const SweepArgs<float> *, const BatchSweepPlan &, int, int, int,
                                               cudaStream_t);
template void launch_sweep_step<double>(const SweepArgs<double> &, int, int, cudaStream_t);
template void launch_sweep_step<float>(const SweepArgs<float> &, int, int, cudaStream_t);

}  // namespace kgb
