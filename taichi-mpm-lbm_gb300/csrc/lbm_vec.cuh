// Arithmetic on one value (float) or on two lanes at once (float2) with the same rounding.
//
// The float2 forms use the packed FP32 instructions of sm_100 and later (add/sub/mul/fma
// .rn.f32x2). Each lane of a packed result is the result of the scalar round-to-nearest
// operation on that lane's operands, so code written once against these helpers gives
// bit-identical per-cell results for V = float and V = float2, while the float2
// instantiation issues half the floating-point instructions for two cells.
#pragma once

#include <cuda_runtime.h>

namespace fsi {

template <class V>
__device__ __forceinline__ V splat(float a);
template <>
__device__ __forceinline__ float splat<float>(float a) { return a; }
template <>
__device__ __forceinline__ float2 splat<float2>(float a) { return make_float2(a, a); }

// ------------------------------------------------------------------ scalar
__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float vneg(float a) { return -a; }
__device__ __forceinline__ float vdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float vrcp(float a) { return __frcp_rn(a); }

// ------------------------------------------------------------------ two lanes
// add/sub are issued as PTX add/sub.rn.f32x2. A packed multiply whose single use is an
// addition was observed to be merged with it into a fused multiply-add (a different
// rounding) even with the rounding modifier spelled out and contraction disabled, so the
// packed multiply is written as a fused multiply-add with a -0 addend instead.
#define FSI_F32X2_OP(name, op)                                                          \
  __device__ __forceinline__ float2 name(float2 a, float2 b) {                          \
    float2 r;                                                                           \
    asm("{.reg .b64 pa, pb, pd;\n\t"                                                    \
        "mov.b64 pa, {%2, %3};\n\t"                                                     \
        "mov.b64 pb, {%4, %5};\n\t" op " pd, pa, pb;\n\t"                              \
        "mov.b64 {%0, %1}, pd;}"                                                        \
        : "=f"(r.x), "=f"(r.y)                                                          \
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                      \
    return r;                                                                           \
  }
FSI_F32X2_OP(vadd, "add.rn.f32x2")
FSI_F32X2_OP(vsub, "sub.rn.f32x2")
#undef FSI_F32X2_OP

// a * b as fma(a, b, -0): the same correctly rounded product (and the same signed zero),
// but as a fused operation it cannot be merged with a following addition.
__device__ __forceinline__ float2 vmul(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 pa, pb, pc, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "mov.b64 pc, {%6, %6};\n\t"
      "fma.rn.f32x2 pd, pa, pb, pc;\n\t"
      "mov.b64 {%0, %1}, pd;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(-0.0f));
  return r;
}

__device__ __forceinline__ float2 vneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 vmul(float2 a, float b) { return vmul(a, make_float2(b, b)); }
__device__ __forceinline__ float2 vmul(float a, float2 b) { return vmul(make_float2(a, a), b); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 vfma(float a, float2 b, float2 c) {
  return __ffma2_rn(make_float2(a, a), b, c);
}
__device__ __forceinline__ float2 vadd(float2 a, float b) { return vadd(a, make_float2(b, b)); }
__device__ __forceinline__ float2 vadd(float a, float2 b) { return vadd(make_float2(a, a), b); }
__device__ __forceinline__ float2 vsub(float a, float2 b) { return vsub(make_float2(a, a), b); }
__device__ __forceinline__ float2 vsub(float2 a, float b) { return vsub(a, make_float2(b, b)); }
__device__ __forceinline__ float2 vdiv(float2 a, float2 b) {
  return make_float2(__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y));
}
__device__ __forceinline__ float2 vrcp(float2 a) { return make_float2(__frcp_rn(a.x), __frcp_rn(a.y)); }

// Lane access for code that handles the lanes of a V separately.
template <class V>
struct Lanes;
template <>
struct Lanes<float> {
  static constexpr int n = 1;
  static __device__ __forceinline__ float get(float v, int) { return v; }
  static __device__ __forceinline__ void set(float& v, int, float x) { v = x; }
};
template <>
struct Lanes<float2> {
  static constexpr int n = 2;
  static __device__ __forceinline__ float get(float2 v, int l) { return l == 0 ? v.x : v.y; }
  static __device__ __forceinline__ void set(float2& v, int l, float x) {
    if (l == 0) v.x = x; else v.y = x;
  }
};

}  // namespace fsi
