// sweep.cu -- diamond-difference transport sweep on GB300.
//
// Replaces Kernel::sweepSubdomain (src/Kripke/Kernel/SweepSubdomain.cpp:26-111,
// CUDA policy Arch/SweepSubdomains.h:246-269).  Per cell, in upwind order:
//   psi = (rhs + psi_lf*2mu/dx + psi_fr*2eta/dy + psi_bo*2xi/dz)
//         / (2mu/dx + 2eta/dy + 2xi/dz + sigt)
//   psi_lf = 2 psi - psi_lf, psi_fr = 2 psi - psi_fr, psi_bo = 2 psi - psi_bo
// evaluated with the reference's association ((rhs + a)+b)+c and ((x+y)+z)+s.
//
// Schedule: a subdomain's zone set is cut into tiles of kTileX x kTileY x tz
// zones.  In the sweep's own orientation a tile (a,b,c) depends only on
// (a-1,b,c), (a,b-1,c), (a,b,c-1), so all tiles with a+b+c = step form a
// hyperplane that runs concurrently; one launch sweeps one tile hyperplane of
// every subdomain in the wave (all eight octants at once).  Inside a tile each
// thread owns one (group, direction) chain and walks the tile's cells in
// upwind order; its upwind faces stay in registers (psi_lf one value, psi_fr
// one per tile column, psi_bo one per tile column x row).  The reference's
// i/j/k plane fields are the running face buffers between tiles, with chains
// fastest, so every global access of a warp is a contiguous run.
#include "kgb_internal.h"

namespace kgb {

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(kSweepThreads) sweep_step_kernel(const SweepArgs<T> a) {
  const SdomDesc sd = a.sdoms[a.wave[blockIdx.z]];
  const int4 t = a.tiles[a.tile_off + blockIdx.y];
  const int nchain = a.Ds * a.Gs;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchain) return;  // no block-level synchronisation below
  const int gl = c / a.Ds;
  const int dl = c - gl * a.Ds;
  const int g = sd.glo + gl;
  const int d = sd.dlo + dl;

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
    iloc[ii] = sd.id > 0 ? ip : a.nxs - 1 - ip;
    cxr[ii] = iv[ii] ? a.cx[(int64_t)d * a.nx + sd.io + iloc[ii]] : T(0);
  }
#pragma unroll
  for (int jj = 0; jj < TY; ++jj) {
    const int jp = jb + jj;
    jv[jj] = jp < a.nys;
    jloc[jj] = sd.jd > 0 ? jp : a.nys - 1 - jp;
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
      bo[ii][jj] = (iv[ii] && jv[jj]) ? kpl[((int64_t)jloc[jj] * a.nxs + iloc[ii]) * nchain + c] : T(0);

  const int kend = min(a.tz, a.nzs - kb);
  for (int kk = 0; kk < kend; ++kk) {
    const int kq = kb + kk;
    const int k = sd.kd > 0 ? kq : a.nzs - 1 - kq;
    const T czk = a.cz[(int64_t)d * a.nz + sd.ko + k];
    T fr[TX];
#pragma unroll
    for (int ii = 0; ii < TX; ++ii) fr[ii] = iv[ii] ? jpl[((int64_t)k * a.nxs + iloc[ii]) * nchain + c] : T(0);
#pragma unroll
    for (int jj = 0; jj < TY; ++jj) {
      if (!jv[jj]) continue;
      const int j = jloc[jj];
      T *const lfp = ipl + ((int64_t)k * a.nys + j) * nchain + c;
      T lf = *lfp;
      const int64_t zrow = ((int64_t)(sd.ko + k) * a.ny + (sd.jo + j)) * a.nx + sd.io;
#pragma unroll
      for (int ii = 0; ii < TX; ++ii) {
        if (!iv[ii]) continue;
        const int64_t z = zrow + iloc[ii];
        const int64_t e = (z * a.G + g) * a.D + d;
        const T r = a.rhs[e];
        const T st = a.sigt[z * a.G + g];
        const T num = r + lf * cxr[ii] + fr[ii] * cyr[jj] + bo[ii][jj] * czk;
        const T den = cxr[ii] + cyr[jj] + czk + st;
        const T ps = num / den;
        a.psi[e] = ps;
        lf = T(2) * ps - lf;
        fr[ii] = T(2) * ps - fr[ii];
        bo[ii][jj] = T(2) * ps - bo[ii][jj];
      }
      *lfp = lf;
    }
#pragma unroll
    for (int ii = 0; ii < TX; ++ii)
      if (iv[ii]) jpl[((int64_t)k * a.nxs + iloc[ii]) * nchain + c] = fr[ii];
  }
#pragma unroll
  for (int ii = 0; ii < TX; ++ii)
#pragma unroll
    for (int jj = 0; jj < TY; ++jj)
      if (iv[ii] && jv[jj]) kpl[((int64_t)jloc[jj] * a.nxs + iloc[ii]) * nchain + c] = bo[ii][jj];
}

template <typename T>
void launch_sweep_step(const SweepArgs<T> &a, int ntiles, int nwave, cudaStream_t s) {
  const int nchain = a.Ds * a.Gs;
  dim3 grid((nchain + kSweepThreads - 1) / kSweepThreads, ntiles, nwave);
  sweep_step_kernel<T, kTileX, kTileY><<<grid, kSweepThreads, 0, s>>>(a);
}

template void launch_sweep_step<double>(const SweepArgs<double> &, int, int, cudaStream_t);
template void launch_sweep_step<float>(const SweepArgs<float> &, int, int, cudaStream_t);

}  // namespace kgb
