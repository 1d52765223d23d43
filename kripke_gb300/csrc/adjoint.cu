// adjoint.cu -- response, adjoint source, gradient assembly and convergence
// norms for the hand-written adjoint of the source iteration.
//
// Response (absorption rate in a detector region):
//   R = sum_z det(z) vol(z) sum_g siga(g,z) phiw(g,z),   phiw = sum_d w(d) psi(d,g,z),
//   siga(g,z) = sigt_zonal(g,z) - sum_mix f * sum_g' sigs(mat, 0, g', g).
// The converged forward state solves A psi = b, A = H - L+ S L (H the
// diamond-difference transport operator, H^-1 the sweep) and b = L+ Q.  The
// adjoint solves A^T lambda = dR/dpsi = w(d) vol det siga.
//
// Transposed sweep.  Along one direction the diamond-difference map from rhs
// to psi couples two cells by products of (2 c/den) and (-1) pass-through
// factors, where c = 2|cos|/delta of the cell a face enters.  Reversing the
// path exchanges the cell whose c appears, and the products differ by the
// ratio of c_x(i) c_y(j) c_z(k) at the two ends, which is proportional to
// 1/(dx_i dy_j dz_k).  Hence H^-T = V Rev V^-1 with Rev the same sweep run
// from the opposite corner and V the diagonal of cell volumes (the identity
// up to a constant on a uniform mesh).  With lambda~ = V^-1 lambda:
//   lambda~ = Rev( L^T (S^T L+^T lambda~ + nu / V) ),   L^T nu = dR/dpsi,
// i.e. the forward iteration with L and L+ exchanged (transposed), S
// transposed over groups, the reversed sweep, and a moment-0 source
// nu/V = det siga (vol/V) / c0 where ell(0,d) = c0 w(d).
// Gradients at the fixed point (mu = L+^T lambda, phi0 = (L psi)_0, f_m the
// zone's fraction of material m):
//   dR/dsigt[m][g]   = E[m][g] - sum_z f_m sum_d lambda psi
//   dR/dsigs0[m][g]  = -E[m][g] + sum_z f_m mu(0,g,z) phi0(g,z)   (in-group P0 entry)
//   dR/dq            = sum_{g,z} f_0 mu(0,g,z)
//   E[m][g]          = sum_z det vol f_m phiw(g,z)
// Every reduction runs over (group, block of zones) in a fixed order, so the
// results do not depend on scheduling.
#include "kgb_internal.h"

namespace kgb {

namespace {
constexpr int kAdjThreads = 128;
constexpr int kAcc = 13;  // [m*4 + k] for material m < 3 and term k < 4, then the response

__device__ __forceinline__ double cellVolume(const MixArgs &a, int64_t z) {
  const int64_t i = z % a.nx, j = (z / a.nx) % a.ny, k = z / ((int64_t)a.nx * a.ny);
  return a.dx[i] * a.dy[j] * a.dz[k];
}

// siga(g, z): the zone's sigt minus the mix-weighted P0 out-scattering of group g
template <typename T>
__device__ __forceinline__ double absorption(const MixArgs &a, const T *sigt, int64_t z, int g) {
  double sa = (double)sigt[z * a.G + g];
  const int ms = a.zmix_start[z], mc = a.zmix_count[z];
  for (int x = 0; x < mc; ++x) sa -= a.mix_frac[ms + x] * a.colsum[a.mix_mat[ms + x] * a.G + g];
  return sa;
}

template <typename T>
__global__ void adjoint_source_kernel(T *__restrict__ phi_out, int M, const T *__restrict__ sigt, const MixArgs a,
                                      double inv_c0) {
  const int64_t n = a.Z * a.G;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = r / a.G;
    const int g = (int)(r - z * a.G);
    const double dz = a.det[z];
    if (dz == 0.0) continue;
    const double sa = absorption(a, sigt, z, g);
    phi_out[r * M] += (T)(dz * sa * (a.vol[z] / cellVolume(a, z)) * inv_c0);
  }
}

// Block (zone block bx, group g); each warp takes whole (zone, group) rows,
// lanes stride the directions, and the row sums are reduced in a fixed lane
// order.  lam == nullptr: response and E only.  psi0 supplies the moments
// phi0 of the sigma_s term (the same state as psi at a fixed point; the
// previous iterate in the unrolled gradient; nullptr: a zero state).
template <typename T>
__global__ void __launch_bounds__(kAdjThreads) response_kernel(const T *__restrict__ psi, const T *__restrict__ psi0,
                                                               const T *__restrict__ lam,
                                                               int D, const double *__restrict__ w,
                                                               const double *__restrict__ ell0,
                                                               const double *__restrict__ ellp0,
                                                               const T *__restrict__ sigt, const MixArgs a, int zpb,
                                                               double *__restrict__ partials) {
  __shared__ double red[kAdjThreads / 32][kAcc];
  const int g = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t z0 = (int64_t)blockIdx.x * zpb;
  const int64_t z1 = min(a.Z, z0 + zpb);
  const bool adj = lam != nullptr;
  double acc[kAcc];
#pragma unroll
  for (int i = 0; i < kAcc; ++i) acc[i] = 0.0;
  for (int64_t z = z0 + warp; z < z1; z += kAdjThreads / 32) {
    const int64_t r = z * a.G + g;
    const T *p = psi + r * D;
    double phw = 0.0, ph0 = 0.0, lp = 0.0, mu0 = 0.0;
    if (adj) {
      const T *l = lam + r * D;
      const T *p0 = psi0 ? psi0 + r * D : nullptr;
      for (int d = lane; d < D; d += 32) {
        const double pd = (double)p[d], ld = (double)l[d];
        phw += w[d] * pd;
        if (p0) ph0 += ell0[d] * (double)p0[d];
        lp += ld * pd;
        mu0 += ellp0[d] * ld;
      }
    } else {
      for (int d = lane; d < D; d += 32) phw += w[d] * (double)p[d];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      phw += __shfl_xor_sync(0xffffffffu, phw, o);
      ph0 += __shfl_xor_sync(0xffffffffu, ph0, o);
      lp += __shfl_xor_sync(0xffffffffu, lp, o);
      mu0 += __shfl_xor_sync(0xffffffffu, mu0, o);
    }
    if (lane == 0) {
      const double dv = a.det[z] * a.vol[z];
      const double vg = adj ? cellVolume(a, z) : 0.0;  // lambda = vg * lambda~, mu = vg * mu~
      double sa = (double)sigt[r];
      const int ms = a.zmix_start[z], mc = a.zmix_count[z];
      for (int x = 0; x < mc; ++x) {
        const int mat = a.mix_mat[ms + x];
        const double f = a.mix_frac[ms + x];
        sa -= f * a.colsum[mat * a.G + g];
        acc[mat * 4 + 0] += dv * f * phw;
        if (adj) {
          acc[mat * 4 + 1] += f * vg * lp;
          acc[mat * 4 + 2] += f * vg * mu0 * ph0;
          acc[mat * 4 + 3] += f * vg * mu0;
        }
      }
      acc[12] += dv * sa * phw;
    }
  }
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < kAcc; ++i) red[warp][i] = acc[i];
  __syncthreads();
  if (threadIdx.x < kAcc) {
    double s = 0.0;
    for (int wv = 0; wv < kAdjThreads / 32; ++wv) s += red[wv][threadIdx.x];
    partials[((int64_t)g * gridDim.x + blockIdx.x) * kAcc + threadIdx.x] = s;
  }
}

__global__ void response_finish_kernel(const double *__restrict__ partials, int nb, int G, double *__restrict__ out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < G * kAcc; t += gridDim.x * blockDim.x) {
    const int g = t / kAcc, i = t - g * kAcc;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += partials[((int64_t)g * nb + b) * kAcc + i];
    out[t] = s;
  }
}

// max |phi(r,0) - prev(r)| and max |phi(r,0)| over rows, then prev = phi(.,0).  Non-negative doubles (and +inf, NaN) order
// like their bit patterns, so the maxima reduce as unsigned integers.
template <typename T>
__global__ void change_norm_kernel(const T *__restrict__ phi, int M, double *__restrict__ prev, int64_t rows,
                                   unsigned long long *__restrict__ out) {
  unsigned long long dmax = 0ull, amax = 0ull;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const double v = (double)phi[r * M];
    const unsigned long long dd = (unsigned long long)__double_as_longlong(fabs(v - prev[r]));
    const unsigned long long aa = (unsigned long long)__double_as_longlong(fabs(v));
    dmax = dd > dmax ? dd : dmax;
    amax = aa > amax ? aa : amax;
    prev[r] = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long d2 = __shfl_xor_sync(0xffffffffu, dmax, o);
    const unsigned long long a2 = __shfl_xor_sync(0xffffffffu, amax, o);
    dmax = d2 > dmax ? d2 : dmax;
    amax = a2 > amax ? a2 : amax;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, dmax);
    atomicMax(out + 1, amax);
  }
}

// sigt_zonal(g, z) = sum over the zone's mix elements, in order and from 0,
// of fraction * sigma_t(mat, g) -- the generator's operation order, without
// contraction into fused multiply-adds.
template <typename T>
__global__ void material_sigt_kernel(T *__restrict__ sigt, const double *__restrict__ st, const MixArgs a) {
  const int64_t n = a.Z * a.G;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = r / a.G;
    const int g = (int)(r - z * a.G);
    double s = 0.0;
    const int ms = a.zmix_start[z], mc = a.zmix_count[z];
    for (int x = 0; x < mc; ++x) s = __dadd_rn(s, __dmul_rn(a.mix_frac[ms + x], st[a.mix_mat[ms + x] * a.G + g]));
    sigt[r] = (T)s;
  }
}

int gridRows(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 8 ? (b > 0 ? b : 1) : 152 * 8);
}
}  // namespace

template <typename T>
void launch_adjoint_source(T *phi_out, int M, const T *sigt, const MixArgs &a, double inv_c0, cudaStream_t s) {
  adjoint_source_kernel<T><<<gridRows(a.Z * a.G), 256, 0, s>>>(phi_out, M, sigt, a, inv_c0);
}

template <typename T>
void launch_response(const T *psi, const T *psi0, const T *lam, int D, const double *w, const double *ell0,
                     const double *ellp0, const T *sigt, const MixArgs &a, double *partials, int nblocks_z,
                     double *out, cudaStream_t s) {
  const int zpb = (int)((a.Z + nblocks_z - 1) / nblocks_z);
  response_kernel<T><<<dim3(nblocks_z, a.G), kAdjThreads, 0, s>>>(psi, psi0, lam, D, w, ell0, ellp0, sigt, a, zpb,
                                                                  partials);
  response_finish_kernel<<<(a.G * kAcc + 127) / 128, 128, 0, s>>>(partials, nblocks_z, a.G, out);
}

template <typename T>
void launch_change_norm(const T *phi, int M, double *prev, int64_t rows, unsigned long long *out, cudaStream_t s) {
  change_norm_kernel<T><<<gridRows(rows), 256, 0, s>>>(phi, M, prev, rows, out);
}

template <typename T>
void launch_material_sigt(T *sigt, const double *sigt_mat, const MixArgs &a, cudaStream_t s) {
  material_sigt_kernel<T><<<gridRows(a.Z * a.G), 256, 0, s>>>(sigt, sigt_mat, a);
}

#define KGB_ADJ_INST(T)                                                                                          \
  template void launch_adjoint_source<T>(T *, int, const T *, const MixArgs &, double, cudaStream_t);            \
  template void launch_response<T>(const T *, const T *, const T *, int, const double *, const double *,         \
                                   const double *, const T *, const MixArgs &, double *, int, double *,          \
                                   cudaStream_t);                                                                \
  template void launch_change_norm<T>(const T *, int, double *, int64_t, unsigned long long *, cudaStream_t);    \
  template void launch_material_sigt<T>(T *, const double *, const MixArgs &, cudaStream_t);
KGB_ADJ_INST(double)
KGB_ADJ_INST(float)
#undef KGB_ADJ_INST

}  // namespace kgb
