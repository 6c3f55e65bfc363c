// Pair geometry shared by the neighbor builder and the descriptor kernels.
//
// Two evaluations of the periodic image vector of a pair (i, j, s):
//   * exact_image_cell: the reference's FP64 formula and operation order
//     (structure.cpp:69-77): im = ((x_j - x_i) + s1 a1) + s2 a2) + s3 a3,
//     dist = sqrt((x^2 + y^2) + z^2), every operation explicitly rounded.
//     It decides neighbor membership and the descriptor cutoff filter, and it
//     is what the FP64 paths return.
//   * image_ff: the same vector in float-float arithmetic (FP32 operations
//     only; FP64 instructions are scarce on this GPU) from positions split
//     as hi + lo floats and lattice vectors split the same way.  Its error is
//     below ~1e-10 A for cells up to ~100 A, far below FP32 rounding, so the mixed
//     path's FP32 pair vectors come from it, and a distance whose float-float
//     value lies more than a small margin from a cutoff is decided without
//     FP64.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace fpp {

// Neighbor keys (j << kKeyBits) | shift index: ordered by j, then shift, as
// the reference lists them; decoded with shifts (n_shift <= 2^kKeyBits).
constexpr int kKeyBits = 20;
constexpr long long kKeyMask = (1LL << kKeyBits) - 1;

// What a kernel needs to recompute a pair's exact FP64 distance from the
// neighbor list (wp == nullptr: the caller's FP64 pair table is authoritative).
struct NbGeom {
  const dvec4 *wp;         // wrapped FP64 positions
  const long long *keys;   // per pair (j << kKeyBits) | shift index
  double cell[9];          // lattice vectors as rows
  int sweep, ns;           // shifts per direction: ns = 2 sweep + 1
};

__device__ __forceinline__ double shift_add(double v, int s, double c) {
  if (s == 0) {
    if ((__double_as_longlong(v) << 1) != 0) return v;  // v + (+-0) == v unless v is a zero
    return dadd(v, dmul(0.0, c));
  }
  if (s == 1) return dadd(v, c);
  if (s == -1) return dadd(v, -c);
  return dadd(v, dmul((double)s, c));
}

__device__ __forceinline__ double exact_image_cell(const dvec4 &wi, const dvec4 &wj,
                                                   const double *cell, int s1, int s2,
                                                   int s3, double im[3]) {
  double diff[3] = {dsub(wj.x, wi.x), dsub(wj.y, wi.y), dsub(wj.z, wi.z)};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double v = shift_add(diff[k], s1, cell[0 * 3 + k]);
    v = shift_add(v, s2, cell[1 * 3 + k]);
    im[k] = shift_add(v, s3, cell[2 * 3 + k]);
  }
  return __dsqrt_rn(dadd(dadd(dmul(im[0], im[0]), dmul(im[1], im[1])),
                         dmul(im[2], im[2])));
}

__device__ __forceinline__ void decode_shift(int sidx, int ns, int sweep, int &s1, int &s2,
                                             int &s3) {
  s3 = sidx % ns - sweep;
  s2 = (sidx / ns) % ns - sweep;
  s1 = sidx / (ns * ns) - sweep;
}

// Exact FP64 distance of pair p of atom i (out of line: the FP32 kernels
// reach it only for pairs within ~1e-6 relative of a cutoff).
static __device__ __noinline__ double exact_pair_dist(const NbGeom &g, int i, long long p) {
  const long long key = g.keys[p];
  const int j = (int)(key >> kKeyBits);
  int s1, s2, s3;
  decode_shift((int)(key & kKeyMask), g.ns, g.sweep, s1, s2, s3);
  double im[3];
  return exact_image_cell(g.wp[i], g.wp[j], g.cell, s1, s2, s3, im);
}

// ---------------------------------------------------------------------------
// Float-float arithmetic (Dekker / Knuth error-free transformations).
// ---------------------------------------------------------------------------
struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return ff{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff ff_norm(float hi, float lo) {
  const float s = hi + lo;
  return ff{s, lo - (s - hi)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = ff_two_sum(a.hi, b.hi);
  return ff_norm(s.hi, s.lo + (a.lo + b.lo));
}

// s * a for a small integer s, exact product of the leading parts
__device__ __forceinline__ ff ff_scale(ff a, int s) {
  const float fs = (float)s;
  const float p = fs * a.hi;
  const float e = fmaf(fs, a.hi, -p);
  return ff_norm(p, e + fs * a.lo);
}

__device__ __forceinline__ ff ff_sqr(ff a) {
  const float p = a.hi * a.hi;
  const float e = fmaf(a.hi, a.hi, -p);
  return ff_norm(p, e + 2.0f * a.hi * a.lo);
}

// Lattice vectors and shift decoding for the float-float image.
struct CellFF {
  float hi[9], lo[9];
};

// im = (x_j - x_i) + s1 a1 + s2 a2 + s3 a3 and |im|^2, float-float.
__device__ __forceinline__ void image_ff(const float4 &pi_hi, const float4 &pi_lo,
                                         const float4 &pj_hi, const float4 &pj_lo,
                                         const CellFF &c, int s1, int s2, int s3,
                                         ff im[3], ff &r2) {
  const float ih[3] = {pi_hi.x, pi_hi.y, pi_hi.z}, il[3] = {pi_lo.x, pi_lo.y, pi_lo.z};
  const float jh[3] = {pj_hi.x, pj_hi.y, pj_hi.z}, jl[3] = {pj_lo.x, pj_lo.y, pj_lo.z};
  const int sv[3] = {s1, s2, s3};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const ff d = ff_two_sum(jh[k], -ih[k]);
    ff v = ff_norm(d.hi, d.lo + (jl[k] - il[k]));
#pragma unroll
    for (int a = 0; a < 3; a++)
      if (sv[a] != 0) v = ff_add(v, ff_scale(ff{c.hi[a * 3 + k], c.lo[a * 3 + k]}, sv[a]));
    im[k] = v;
  }
  r2 = ff_add(ff_add(ff_sqr(im[0]), ff_sqr(im[1])), ff_sqr(im[2]));
}

// sqrt of a float-float value to ~1 ulp of FP32 (one correction step).
__device__ __forceinline__ float ff_sqrt_f(ff x) {
  if (!(x.hi > 0.0f)) return 0.0f;
  const float r0 = sqrtf(x.hi);
  const float e = fmaf(-r0, r0, x.hi) + x.lo;
  return fmaf(e, 0.5f / r0, r0);
}

}  // namespace fpp
