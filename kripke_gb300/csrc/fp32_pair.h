// fp32_pair.h -- paired FP32 multiply-add shared by the SIMT FP32 kernels of the
// mixed form (LTimes, scattering).
#pragma once

namespace kgb {
namespace {

// (c0, c1) = (a0, a1) * x + (c0, c1): two FP32 multiply-adds, each rounded once to nearest,
// in one paired instruction (bit for bit two __fmaf_rn)
__device__ __forceinline__ void fma2Rn(float &c0, float &c1, float a0, float a1, float x) {
  asm("{\n\t.reg .b64 ra, rb, rc;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %4};\n\tmov.b64 rc, {%0, %1};\n\t"
      "fma.rn.f32x2 rc, ra, rb, rc;\n\tmov.b64 {%0, %1}, rc;\n\t}"
      : "+f"(c0), "+f"(c1)
      : "f"(a0), "f"(a1), "f"(x));
}

}  // namespace
}  // namespace kgb
