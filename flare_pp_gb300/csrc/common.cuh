// Shared device helpers for the flare_pp_gb300 kernels (sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/flare_pp_gb300.h"

namespace fpp {

constexpr int kMaxL = 8;    // largest lmax of the B2 kernels
constexpr int kMaxN = 16;   // largest radial order N
enum CutoffKind { kQuadratic = 0, kCosine = 1 };

// 32-byte aligned FP64 quadruple (r, x, y, z of a pair; x, y, z of an atom).
struct alignas(32) dvec4 {
  double x, y, z, w;
};

// Time budget for every device-side wait (mbarrier or flag), read from the
// global nanosecond timer.  A wait that runs out records an error in the
// device status word and returns instead of hanging the GPU.
constexpr unsigned long long kWaitBudgetNs = 2000000000ull;

struct DeviceStatus {
  int code;    // 0 = ok, otherwise an FPP_ERR_* value
  int where;   // kernel-specific location tag
  int info;    // kernel-specific detail (an index)
  int pad;
};

__device__ __forceinline__ void set_status(DeviceStatus *st, int code,
                                           int where, int info) {
  if (st != nullptr && atomicCAS(&st->code, 0, code) == 0) {
    st->where = where;
    st->info = info;
  }
}

// Explicitly rounded FP64 arithmetic: the neighbor builder must reproduce the
// reference's distances bit for bit, so no multiply-add may be contracted.
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// Fused multiply-add in the argument's own precision (an unqualified fma on
// floats can resolve to the double overload, i.e. FP64 instructions).
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) {
  return __fma_rn(a, b, c);
}

__device__ __forceinline__ float sqrt_t(float a) { return sqrtf(a); }
__device__ __forceinline__ double sqrt_t(double a) { return sqrt(a); }
__device__ __forceinline__ float fabs_t(float a) { return fabsf(a); }
__device__ __forceinline__ double fabs_t(double a) { return fabs(a); }
__device__ __forceinline__ float cos_t(float a) { return cosf(a); }
__device__ __forceinline__ double cos_t(double a) { return cos(a); }
__device__ __forceinline__ float sin_t(float a) { return sinf(a); }
__device__ __forceinline__ double sin_t(double a) { return sin(a); }

// Two independent fused multiply-adds (round to nearest) in one paired FP32
// instruction: d = a * b + c lane by lane, the same results as two fmaf.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;"
      : "=l"(d)
      : "l"(*reinterpret_cast<const unsigned long long *>(&a)),
        "l"(*reinterpret_cast<const unsigned long long *>(&b)),
        "l"(*reinterpret_cast<const unsigned long long *>(&c)));
  return *reinterpret_cast<const float2 *>(&d);
}

__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;"
      : "=l"(d)
      : "l"(*reinterpret_cast<const unsigned long long *>(&a)),
        "l"(*reinterpret_cast<const unsigned long long *>(&b)));
  return *reinterpret_cast<const float2 *>(&d);
}

// Kahan-Babuska (Neumaier) compensated accumulator in FP32.
struct CompSum {
  float s, c;
  __device__ __forceinline__ CompSum() : s(0.f), c(0.f) {}
  __device__ __forceinline__ void add(float x) {
    float t = s + x;
    if (fabsf(s) >= fabsf(x))
      c += (s - t) + x;
    else
      c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ float value() const { return s + c; }
};

__host__ __device__ __forceinline__ int ceil_div(int a, int b) {
  return (a + b - 1) / b;
}

}  // namespace fpp
