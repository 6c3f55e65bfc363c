// Per-neighbor bases on the device: chebyshev x cutoff radial functions and
// real spherical harmonics with Cartesian gradients.
//
// Radial: T_n((r - r1)/(rc - r1)) with T_0 = 1, T_1 = x, T_n = 2x T_{n-1} -
// T_{n-2}, zero outside [r1, rc], times the quadratic (r - rc)^2 or cosine
// (cos(pi r / rc) + 1)/2 cutoff -- the functions of src/flare_pp/radial.cpp:
// 138-169 and src/flare_pp/cutoffs.cpp:44-73.
//
// Harmonics: the orthonormal real harmonics without Condon-Shortley phase at
// index l*l + l + m (the convention of src/flare_pp/y_grad.cpp:667), derived
// here from the solid-harmonic recurrence
//   r^l Y_lm = N_lm Q_l^|m|(z, r^2) T_m(x, y) (* sqrt 2 for m != 0),
//   T_m = Re / Im (x + i y)^|m|, Q_m^m = (2m-1)!!, Q_{m+1}^m = (2m+1) z Q_m^m,
//   Q_l^m = ((2l-1) z Q_{l-1}^m - (l+m-1) r^2 Q_{l-2}^m) / (l - m),
// evaluated on the unit vector; gradients differentiate the recurrence and
// use grad Y(r) = (grad R(u) - l Y(u) u) / |r|.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace fpp {

// Normalisation N_lm * (sqrt 2 if m > 0) at [l*(kMaxL+1) + m]; its FP32
// hi/lo split (so FP32 evaluation carries no systematic rounding of the
// constants) is further divided by D_lm = prod_{k=m+2..l} (k - m), the factor
// the division-free FP32 recurrence leaves in Q_l^m.  Double factorials
// (2m-1)!! at [m].
struct HarmonicTables {
  double norm[(kMaxL + 1) * (kMaxL + 1)];
  float norm_hi[(kMaxL + 1) * (kMaxL + 1)];
  float norm_lo[(kMaxL + 1) * (kMaxL + 1)];
  double dfact[kMaxL + 1];
  float dfact_f[kMaxL + 1];  // exact in FP32 (at most 15!! = 2027025)
};
static __constant__ HarmonicTables c_harm;  // uploaded by upload_harmonic_tables()

// N_lm * v (FP32: N_lm / D_lm * v), with the constant kept to ~48 bits in FP32
__device__ __forceinline__ double norm_scale(int k, double v) { return c_harm.norm[k] * v; }
__device__ __forceinline__ float norm_scale(int k, float v) {
  return fmaf(c_harm.norm_hi[k], v, c_harm.norm_lo[k] * v);
}

// g_n and dg_n/dr into out_g[n * stride], out_dg[n * stride].
// (cos(pi r / rc) + 1) / 2 and its derivative, out of line: the quadratic
// cutoff is the common case, and the trigonometric code (whose range reduction
// has FP64 steps) stays off its instruction stream.
template <typename T>
static __device__ __noinline__ void cosine_cutoff(T r, T rc, T &fc, T &dfc) {
  const T pi = T(3.14159265358979323846);
  fc = T(0.5) * (cos_t(pi * r / rc) + T(1));
  dfc = -pi * sin_t(pi * r / rc) / (T(2) * rc);
}

// FP32: the argument is (r - r1) (cinv_hi + cinv_lo) with the reciprocal
// 1 / (rc - r1) split hi/lo in FP64 (FP32 callers always pass it); FP64: the
// correctly rounded division.
template <typename T>
__device__ __forceinline__ void radial_basis(T r, T r1, T rc, int N, int cutoff_kind,
                                             T *out_g, T *out_dg, int stride,
                                             T cinv_hi = T(0), T cinv_lo = T(0)) {
  T fc, dfc;
  if (r > rc) {
    fc = T(0);
    dfc = T(0);
  } else if (cutoff_kind == kQuadratic) {
    T d = r - rc;
    fc = d * d;
    dfc = T(2) * d;
  } else {
    cosine_cutoff(r, rc, fc, dfc);
  }
  const bool inside = !(r < r1 || r > rc);
  // x by the hi/lo reciprocal (FP32) or a correctly rounded division (FP64):
  // a rounded reciprocal alone would shift every pair's argument the same way
  // and bias the descriptors in FP32.  FP32 has no division fallback: the
  // divide's special-case handling issued FP64-pipe instructions even where
  // a branch around it was never taken.
  T c, x;
  if constexpr (sizeof(T) == 4) {
    c = cinv_hi;
    x = fma_t(r - r1, cinv_hi, (r - r1) * cinv_lo);
  } else {
    c = T(1) / (rc - r1);
    x = (r - r1) / (rc - r1);
  }
  T tm2 = 0, tm1 = 0, dm2 = 0, dm1 = 0;
  for (int n = 0; n < N; n++) {
    T t, dt;
    if (n == 0) {
      t = T(1);
      dt = T(0);
    } else if (n == 1) {
      t = x;
      dt = c;
    } else {
      t = T(2) * x * tm1 - tm2;
      dt = T(2) * tm1 * c + T(2) * x * dm1 - dm2;
    }
    tm2 = tm1;
    tm1 = t;
    dm2 = dm1;
    dm1 = dt;
    T gv = inside ? t : T(0), dv = inside ? dt : T(0);
    out_g[n * stride] = gv * fc;
    if (out_dg) out_dg[n * stride] = dv * fc + gv * dfc;
  }
}

// Register version: g[n], dg[n] for n < N in fully unrolled arrays.
template <typename T>
__device__ __forceinline__ void radial_basis_reg(T r, T r1, T rc, int N, int cutoff_kind,
                                                 T (&g)[kMaxN], T (&dg)[kMaxN],
                                                 T cinv_hi = T(0), T cinv_lo = T(0)) {
  T fc, dfc;
  if (r > rc) {
    fc = T(0);
    dfc = T(0);
  } else if (cutoff_kind == kQuadratic) {
    const T d = r - rc;
    fc = d * d;
    dfc = T(2) * d;
  } else {
    cosine_cutoff(r, rc, fc, dfc);
  }
  const bool inside = !(r < r1 || r > rc);
  T c, x;
  if constexpr (sizeof(T) == 4) {  // split reciprocal, as in radial_basis
    c = cinv_hi;
    x = fma_t(r - r1, cinv_hi, (r - r1) * cinv_lo);
  } else {
    c = T(1) / (rc - r1);
    x = (r - r1) / (rc - r1);
  }
  T tm2 = 0, tm1 = 0, dm2 = 0, dm1 = 0;
#pragma unroll
  for (int n = 0; n < kMaxN; n++) {
    T t, dt;
    if (n == 0) {
      t = T(1);
      dt = T(0);
    } else if (n == 1) {
      t = x;
      dt = c;
    } else {
      t = T(2) * x * tm1 - tm2;
      dt = T(2) * tm1 * c + T(2) * x * dm1 - dm2;
    }
    tm2 = tm1;
    tm1 = t;
    dm2 = dm1;
    dm1 = dt;
    const T gv = inside ? t : T(0), dv = inside ? dt : T(0);
    g[n] = (n < N) ? gv * fc : T(0);
    dg[n] = (n < N) ? dv * fc + gv * dfc : T(0);
  }
}

// Y_lm at out[lm * stride]; with grad != nullptr also the Cartesian gradient
// at grad[(3*lm + k) * stride].
template <typename T>
__device__ __forceinline__ void real_harmonics(T x, T y, T z, int lmax, T *out,
                                               T *grad, int stride) {
  const T r = sqrt_t(x * x + y * y + z * z);
  const T ir = T(1) / r;
  const T ux = x * ir, uy = y * ir, uz = z * ir;
  T A = T(1), B = T(0), Aprev = T(1), Bprev = T(0);
  for (int m = 0; m <= lmax; m++) {
    if (m > 0) {
      Aprev = A;
      Bprev = B;
      T a2 = ux * A - uy * B;
      T b2 = uy * A + ux * B;
      A = a2;
      B = b2;
    }
    // derivatives of A_m, B_m with respect to x and y
    const T Ax = T(m) * Aprev, Ay = -T(m) * Bprev;
    const T Bx = T(m) * Bprev, By = T(m) * Aprev;
    T q2 = 0, q1 = 0, qz2 = 0, qz1 = 0, qr2 = 0, qr1 = 0;
    for (int l = m; l <= lmax; l++) {
      T q, qz, qr;
      if (l == m) {
        q = sizeof(T) == 4 ? T(c_harm.dfact_f[m]) : T(c_harm.dfact[m]);
        qz = T(0);
        qr = T(0);
      } else if (l == m + 1) {
        q = T(2 * m + 1) * uz * q1;
        qz = T(2 * m + 1) * q1;
        qr = T(0);
      } else if constexpr (sizeof(T) == 4) {
        // division-free: q carries the factor D_l = prod_{k=m+2..l} (k - m),
        // which the FP32 normalisation table divides out (no per-pair
        // divisions, and no rounded reciprocal of l - m)
        const T a = T(2 * l - 1);
        const T bc = T((l + m - 1) * (l - 1 >= m + 2 ? l - 1 - m : 1));
        q = a * uz * q1 - bc * q2;
        qz = a * (q1 + uz * qz1) - bc * qz2;
        qr = a * uz * qr1 - bc * (q2 + qr2);
      } else {
        const T a = T(2 * l - 1), b = T(l + m - 1), dv = T(l - m);
        q = (a * uz * q1 - b * q2) / dv;
        qz = (a * (q1 + uz * qz1) - b * qz2) / dv;
        qr = (a * uz * qr1 - b * (q2 + qr2)) / dv;
      }
      q2 = q1;
      q1 = q;
      qz2 = qz1;
      qz1 = qz;
      qr2 = qr1;
      qr1 = qr;
      const int kn = l * (kMaxL + 1) + m;
      const int ip = l * l + l + m;
      const T R = norm_scale(kn, q * A);
      out[ip * stride] = R;
      if (grad) {
        const T Rx = norm_scale(kn, qr * T(2) * ux * A + q * Ax);
        const T Ry = norm_scale(kn, qr * T(2) * uy * A + q * Ay);
        const T Rz = norm_scale(kn, (qz + qr * T(2) * uz) * A);
        grad[(3 * ip + 0) * stride] = (Rx - T(l) * R * ux) * ir;
        grad[(3 * ip + 1) * stride] = (Ry - T(l) * R * uy) * ir;
        grad[(3 * ip + 2) * stride] = (Rz - T(l) * R * uz) * ir;
      }
      if (m > 0) {
        const int im = l * l + l - m;
        const T S = norm_scale(kn, q * B);
        out[im * stride] = S;
        if (grad) {
          const T Sx = norm_scale(kn, qr * T(2) * ux * B + q * Bx);
          const T Sy = norm_scale(kn, qr * T(2) * uy * B + q * By);
          const T Sz = norm_scale(kn, (qz + qr * T(2) * uz) * B);
          grad[(3 * im + 0) * stride] = (Sx - T(l) * S * ux) * ir;
          grad[(3 * im + 1) * stride] = (Sy - T(l) * S * uy) * ir;
          grad[(3 * im + 2) * stride] = (Sz - T(l) * S * uz) * ir;
        }
      }
    }
  }
}

// The same harmonics with gradients, handed to visit(lm, Y, dY/dx, dY/dy,
// dY/dz) one by one as the recurrence produces them (nothing is stored).
template <typename T, typename Visit>
__device__ __forceinline__ void harmonics_visit(T x, T y, T z, int lmax, Visit visit) {
  const T r = sqrt_t(x * x + y * y + z * z);
  const T ir = T(1) / r;
  const T ux = x * ir, uy = y * ir, uz = z * ir;
  T A = T(1), B = T(0), Aprev = T(1), Bprev = T(0);
  for (int m = 0; m <= lmax; m++) {
    if (m > 0) {
      Aprev = A;
      Bprev = B;
      const T a2 = ux * A - uy * B;
      const T b2 = uy * A + ux * B;
      A = a2;
      B = b2;
    }
    const T Ax = T(m) * Aprev, Ay = -T(m) * Bprev;
    const T Bx = T(m) * Bprev, By = T(m) * Aprev;
    T q2 = 0, q1 = 0, qz2 = 0, qz1 = 0, qr2 = 0, qr1 = 0;
    for (int l = m; l <= lmax; l++) {
      T q, qz, qr;
      if (l == m) {
        q = sizeof(T) == 4 ? T(c_harm.dfact_f[m]) : T(c_harm.dfact[m]);
        qz = T(0);
        qr = T(0);
      } else if (l == m + 1) {
        q = T(2 * m + 1) * uz * q1;
        qz = T(2 * m + 1) * q1;
        qr = T(0);
      } else if constexpr (sizeof(T) == 4) {
        // division-free: q carries the factor D_l = prod_{k=m+2..l} (k - m),
        // which the FP32 normalisation table divides out (no per-pair
        // divisions, and no rounded reciprocal of l - m)
        const T a = T(2 * l - 1);
        const T bc = T((l + m - 1) * (l - 1 >= m + 2 ? l - 1 - m : 1));
        q = a * uz * q1 - bc * q2;
        qz = a * (q1 + uz * qz1) - bc * qz2;
        qr = a * uz * qr1 - bc * (q2 + qr2);
      } else {
        const T a = T(2 * l - 1), b = T(l + m - 1), dv = T(l - m);
        q = (a * uz * q1 - b * q2) / dv;
        qz = (a * (q1 + uz * qz1) - b * qz2) / dv;
        qr = (a * uz * qr1 - b * (q2 + qr2)) / dv;
      }
      q2 = q1;
      q1 = q;
      qz2 = qz1;
      qz1 = qz;
      qr2 = qr1;
      qr1 = qr;
      const int kn = l * (kMaxL + 1) + m;
      {
        const T R = norm_scale(kn, q * A);
        const T Rx = norm_scale(kn, qr * T(2) * ux * A + q * Ax);
        const T Ry = norm_scale(kn, qr * T(2) * uy * A + q * Ay);
        const T Rz = norm_scale(kn, (qz + qr * T(2) * uz) * A);
        visit(l * l + l + m, R, (Rx - T(l) * R * ux) * ir, (Ry - T(l) * R * uy) * ir,
              (Rz - T(l) * R * uz) * ir);
      }
      if (m > 0) {
        const T S = norm_scale(kn, q * B);
        const T Sx = norm_scale(kn, qr * T(2) * ux * B + q * Bx);
        const T Sy = norm_scale(kn, qr * T(2) * uy * B + q * By);
        const T Sz = norm_scale(kn, (qz + qr * T(2) * uz) * B);
        visit(l * l + l - m, S, (Sx - T(l) * S * ux) * ir, (Sy - T(l) * S * uy) * ir,
              (Sz - T(l) * S * uz) * ir);
      }
    }
  }
}

// FP32 harmonics with gradients handed to visit(lm, Y, (dY/dx, dY/dy), dY/dz)
// with the x and y components formed together by paired FP32 instructions
// (the same recurrence and normalisation as harmonics_visit<float>).
template <typename Visit>
__device__ __forceinline__ void harmonics_visit_f2(float x, float y, float z, int lmax,
                                                   Visit visit) {
  const float r = sqrtf(x * x + y * y + z * z);
  const float ir = 1.0f / r;
  const float ux = x * ir, uy = y * ir, uz = z * ir;
  const float2 uxy = make_float2(ux, uy), ir2 = make_float2(ir, ir);
  float A = 1.0f, B = 0.0f, Aprev = 1.0f, Bprev = 0.0f;
#pragma unroll
  for (int m = 0; m <= lmax; m++) {
    if (m > 0) {
      Aprev = A;
      Bprev = B;
      const float a2 = ux * A - uy * B;
      const float b2 = uy * A + ux * B;
      A = a2;
      B = b2;
    }
    const float2 Axy = make_float2(float(m) * Aprev, -float(m) * Bprev);
    const float2 Bxy = make_float2(float(m) * Bprev, float(m) * Aprev);
    float q2 = 0, q1 = 0, qz2 = 0, qz1 = 0, qr2 = 0, qr1 = 0;
#pragma unroll
    for (int l = m; l <= lmax; l++) {
      float q, qz, qr;
      if (l == m) {
        q = c_harm.dfact_f[m];
        qz = 0.0f;
        qr = 0.0f;
      } else if (l == m + 1) {
        q = float(2 * m + 1) * uz * q1;
        qz = float(2 * m + 1) * q1;
        qr = 0.0f;
      } else {
        // division-free: the D_lm factor is divided out by the normalisation
        const float a = float(2 * l - 1);
        const float bc = float((l + m - 1) * (l - 1 >= m + 2 ? l - 1 - m : 1));
        q = a * uz * q1 - bc * q2;
        qz = a * (q1 + uz * qz1) - bc * qz2;
        qr = a * uz * qr1 - bc * (q2 + qr2);
      }
      q2 = q1;
      q1 = q;
      qz2 = qz1;
      qz1 = qz;
      qr2 = qr1;
      qr1 = qr;
      const int kn = l * (kMaxL + 1) + m;
      const float nh = c_harm.norm_hi[kn], nl = c_harm.norm_lo[kn];
      const float2 nh2 = make_float2(nh, nh), nl2 = make_float2(nl, nl);
      const float2 q2v = make_float2(q, q);
      const float tq = qr * 2.0f;
      auto emit = [&](int lm, float C, float2 Cxy) {
        const float qc = q * C;
        const float R = fmaf(nh, qc, nl * qc);
        const float t = tq * C;
        const float2 sxy = ffma2(make_float2(t, t), uxy, fmul2(q2v, Cxy));
        const float2 Rxy = ffma2(nh2, sxy, fmul2(nl2, sxy));
        const float sz = (qz + tq * uz) * C;
        const float Rz = fmaf(nh, sz, nl * sz);
        const float lR = float(l) * R;
        const float2 gxy = fmul2(ffma2(make_float2(-lR, -lR), uxy, Rxy), ir2);
        visit(lm, R, gxy, (Rz - lR * uz) * ir);
      };
      emit(l * l + l + m, A, Axy);
      if (m > 0) emit(l * l + l - m, B, Bxy);
    }
  }
}

}  // namespace fpp
