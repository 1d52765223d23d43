// xpose.cu -- move a field chunk between Kripke's host nesting and the device
// nesting, and fill kernels (Kernel::kConst, src/Kripke/Kernel.h:37-55).
//
// A chunk is addressed by up to four logical indices (e.g. direction, group,
// zone).  The host offset is sum(idx * host_stride) with the strides of the
// chunk's nesting; the device offset is sum(idx * device_stride), where a zone
// index is first mapped from the zone set's local numbering
// (k*nys + j)*nxs + i to the global zone (src/Kripke/Generate/Space.cpp:92-93).
// Threads walk the chunk with the device-fastest index fastest, so device
// accesses are contiguous; the host side is a strided gather that the L2
// absorbs.  These run only when data enters or leaves the GPU.
#include "kgb_internal.h"

namespace kgb {

namespace {
struct Offsets {
  int64_t h, o;
};

__device__ __forceinline__ Offsets offsetsOf(const XposeDesc &x, int64_t t) {
  int64_t idx[4] = {0, 0, 0, 0};
  for (int q = x.nd - 1; q >= 0; --q) {
    const int dim = x.iter[q];
    idx[dim] = t % x.n[dim];
    t /= x.n[dim];
  }
  Offsets r{0, x.obase};
  for (int dim = 0; dim < x.nd; ++dim) {
    r.h += idx[dim] * x.hs[dim];
    if (dim == x.zdim) {
      const int64_t zl = idx[dim];
      const int64_t i = zl % x.nxs;
      const int64_t j = (zl / x.nxs) % x.nys;
      const int64_t k = zl / ((int64_t)x.nxs * x.nys);
      const int64_t zg = ((k + x.ko) * x.ny + (j + x.jo)) * x.nx + (i + x.io);
      r.o += zg * x.os[dim];
    } else {
      r.o += idx[dim] * x.os[dim];
    }
  }
  return r;
}

template <typename Td>
__global__ void upload_kernel(const double *__restrict__ staging, Td *__restrict__ dev, const XposeDesc x, int64_t total) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const Offsets o = offsetsOf(x, t);
    dev[o.o] = (Td)staging[o.h];
  }
}

template <typename Td>
__global__ void download_kernel(const Td *__restrict__ dev, double *__restrict__ staging, const XposeDesc x, int64_t total) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const Offsets o = offsetsOf(x, t);
    staging[o.h] = (double)dev[o.o];
  }
}

template <typename T>
__global__ void fill_kernel(T *__restrict__ p, int64_t n, T v) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) p[t] = v;
}

int64_t totalOf(const XposeDesc &x) {
  int64_t n = 1;
  for (int d = 0; d < x.nd; ++d) n *= x.n[d];
  return n;
}

int gridFor(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = 152 * 32;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}
}  // namespace

template <typename Td>
void launch_upload_xpose(const double *staging, Td *dev, const XposeDesc &x, cudaStream_t s) {
  const int64_t n = totalOf(x);
  if (n > 0) upload_kernel<Td><<<gridFor(n), 256, 0, s>>>(staging, dev, x, n);
}

template <typename Td>
void launch_download_xpose(const Td *dev, double *staging, const XposeDesc &x, cudaStream_t s) {
  const int64_t n = totalOf(x);
  if (n > 0) download_kernel<Td><<<gridFor(n), 256, 0, s>>>(dev, staging, x, n);
}

template <typename T>
void launch_fill(T *p, int64_t n, double v, cudaStream_t s) {
  if (n > 0) fill_kernel<T><<<gridFor(n), 256, 0, s>>>(p, n, (T)v);
}

template void launch_upload_xpose<double>(const double *, double *, const XposeDesc &, cudaStream_t);
template void launch_upload_xpose<float>(const double *, float *, const XposeDesc &, cudaStream_t);
template void launch_download_xpose<double>(const double *, double *, const XposeDesc &, cudaStream_t);
template void launch_download_xpose<float>(const float *, double *, const XposeDesc &, cudaStream_t);
template void launch_fill<double>(double *, int64_t, double, cudaStream_t);
template void launch_fill<float>(float *, int64_t, double, cudaStream_t);

// ---------------------------------------------------------------------------
// sigt classes for the sweep's tabulated reciprocals (set-up only)
// ---------------------------------------------------------------------------
namespace {
template <typename T> struct KeyOf;
template <> struct KeyOf<double> {
  static __device__ __forceinline__ unsigned long long of(double v) { return (unsigned long long)__double_as_longlong(v); }
};
template <> struct KeyOf<float> {
  static __device__ __forceinline__ unsigned long long of(float v) { return (unsigned long long)__float_as_uint(v); }
};

// splitmix64 finaliser
__device__ __forceinline__ unsigned int hashKey(unsigned long long k) {
  k ^= k >> 30;
  k *= 0xbf58476d1ce4e5b9ull;
  k ^= k >> 27;
  k *= 0x94d049bb133111ebull;
  k ^= k >> 31;
  return (unsigned int)k;
}

// Every element probes at most kMaxProbe slots (no waiting on other threads);
// a key already present is found by a plain load, so the atomics touch only
// the first arrival of each distinct value.  A probe run that long means the
// table is far fuller than the 65535 classes the sweep can index: the
// overflow flag is raised and every thread stops inserting.
constexpr unsigned int kMaxProbe = 4096;
template <typename T>
__global__ void class_insert_kernel(const T *__restrict__ sig, int64_t n, unsigned long long *table, int *overflow) {
  constexpr unsigned int mask = (1u << kClassTableBits) - 1u;
  const volatile int *ovf = overflow;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n && !*ovf;
       e += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = KeyOf<T>::of(sig[e]);
    if (key == kClassEmpty) {
      *overflow = 1;
      continue;
    }
    unsigned int h = hashKey(key) & mask;
    bool placed = false;
    for (unsigned int probe = 0; probe < kMaxProbe; ++probe, h = (h + 1u) & mask) {
      const unsigned long long cur = __ldcg(table + h);
      if (cur == key) {
        placed = true;
        break;
      }
      if (cur == kClassEmpty) {
        const unsigned long long prev = atomicCAS(table + h, kClassEmpty, key);
        if (prev == kClassEmpty || prev == key) {
          placed = true;
          break;
        }
      }
    }
    if (!placed) *overflow = 1;
  }
}

// lower bound of sig[e] among the ncls sorted distinct values
template <typename T>
__global__ void class_lookup_kernel(const T *__restrict__ sig, int64_t n, const T *__restrict__ uniq, int ncls,
                                    uint16_t *__restrict__ cls) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const T v = sig[e];
    int lo = 0, hi = ncls;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (uniq[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    cls[e] = (uint16_t)lo;
  }
}

int setupGrid(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}
}  // namespace

template <typename T>
void launch_class_insert(const T *sig, int64_t n, unsigned long long *table, int *overflow, cudaStream_t s) {
  class_insert_kernel<T><<<setupGrid(n), 256, 0, s>>>(sig, n, table, overflow);
}
template <typename T>
void launch_class_lookup(const T *sig, int64_t n, const T *uniq, int ncls, uint16_t *cls, cudaStream_t s) {
  class_lookup_kernel<T><<<setupGrid(n), 256, 0, s>>>(sig, n, uniq, ncls, cls);
}
template void launch_class_insert<double>(const double *, int64_t, unsigned long long *, int *, cudaStream_t);
template void launch_class_insert<float>(const float *, int64_t, unsigned long long *, int *, cudaStream_t);
template void launch_class_lookup<double>(const double *, int64_t, const double *, int, uint16_t *, cudaStream_t);
template void launch_class_lookup<float>(const float *, int64_t, const float *, int, uint16_t *, cudaStream_t);

}  // namespace kgb
