// B3 bispectrum: coupling tables and the per-atom device stages.
//
// src/flare_pp/descriptors/b3.cpp:134-240 computes, per atom,
//   B3[(n1 <= n2 <= n3), (l1, l2, l3)] =
//       Re sum_{m1+m2+m3=0} W(l1 l2 l3; m1 m2 m3) c[n1,l1m1] c[n2,l2m2] c[n3,l3m3]
// on complex single-bond coefficients c (complex harmonics with the
// Condon-Shortley phase, src/flare_pp/y_grad.cpp:24), with the triangles
// (l1, l2, l3) in loop order l1, l2, l3 and |l1-l2| <= l3 <= l1+l2.
//
// The complex coefficients are a fixed linear map of the real ones that the
// B2 stages already accumulate: with R = c[l, m], S = c[l, -m] (real, m > 0),
//   c[l, +m] = (-1)^m (R + i S) / sqrt 2,  c[l, -m] = (R - i S) / sqrt 2.
// So the forward reuses the real accumulation, and the adjoint maps the
// holomorphic derivative u = dE/dc back to dE/dc_real, after which the B2
// pair-force kernel applies unchanged.
//
// W is the Wigner 3j symbol from Racah's formula.  The reference's table for
// lmax = 4 (descriptors/wigner3j.cpp:590-1986) holds 0 at the 57 symbols whose
// exact value is a non-integer rational (+-1/3, +-1/6): its generated source
// writes them as C++ integer divisions.  The tables here reproduce that.
//
// Included by exactly one translation unit (the constant bank is static).
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>
#include <vector>

#include "common.cuh"

namespace fpp {

constexpr int kB3MaxL = 4;
constexpr int kB3MaxTerms = 2112;  // sum over lmax 0..4 of the m-terms (2052)
constexpr int kB3MaxLs = 130;      // sum over lmax 0..4 of (n_ls + 1)

struct B3Tables {
  int ls_off[kB3MaxL + 2];    // start of each lmax's triangle offsets in beg[]
  int beg[kB3MaxLs];          // per triangle: first term (absolute index)
  unsigned idx[kB3MaxTerms];  // i1 | i2 << 8 | i3 << 16 (harmonic index l*l+l+m)
  double w[kB3MaxTerms];
  float wf[kB3MaxTerms];      // w rounded to FP32 (the FP32 kernels convert nothing)
};

static __constant__ B3Tables c_b3;
// The coupling coefficient of term e in the kernel's precision.
template <typename T> __device__ __forceinline__ T b3_w(int e);
template <> __device__ __forceinline__ float b3_w<float>(int e) { return c_b3.wf[e]; }
template <> __device__ __forceinline__ double b3_w<double>(int e) { return c_b3.w[e]; }

inline double b3_factorial(int n) {
  double f = 1.0;
  for (int k = 2; k <= n; k++) f *= k;
  return f;
}

// Wigner 3j symbol by Racah's formula (all factorials <= 13! are exact).
inline double b3_wigner3j(int l1, int l2, int l3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0 || l3 < std::abs(l1 - l2) || l3 > l1 + l2) return 0.0;
  if (std::abs(m1) > l1 || std::abs(m2) > l2 || std::abs(m3) > l3) return 0.0;
  const double tri = b3_factorial(l1 + l2 - l3) * b3_factorial(l1 - l2 + l3) *
                     b3_factorial(-l1 + l2 + l3) / b3_factorial(l1 + l2 + l3 + 1);
  const double pre = tri * b3_factorial(l1 + m1) * b3_factorial(l1 - m1) *
                     b3_factorial(l2 + m2) * b3_factorial(l2 - m2) *
                     b3_factorial(l3 + m3) * b3_factorial(l3 - m3);
  int kmin = 0;
  if (l2 - l3 - m1 > kmin) kmin = l2 - l3 - m1;
  if (l1 - l3 + m2 > kmin) kmin = l1 - l3 + m2;
  int kmax = l1 + l2 - l3;
  if (l1 - m1 < kmax) kmax = l1 - m1;
  if (l2 + m2 < kmax) kmax = l2 + m2;
  double s = 0.0;
  for (int k = kmin; k <= kmax; k++) {
    const double d = b3_factorial(k) * b3_factorial(l3 - l2 + k + m1) *
                     b3_factorial(l3 - l1 + k - m2) * b3_factorial(l1 + l2 - l3 - k) *
                     b3_factorial(l1 - k - m1) * b3_factorial(l2 - k + m2);
    s += ((k & 1) ? -1.0 : 1.0) / d;
  }
  const double sign = ((l1 - l2 - m3) % 2 != 0) ? -1.0 : 1.0;
  return sign * std::sqrt(pre) * s;
}

// The coefficient compute_B3 applies for this lmax (see the header comment).
inline double b3_reference_coeff(int l1, int l2, int l3, int m1, int m2, int m3,
                                 int lmax) {
  const double w = b3_wigner3j(l1, l2, l3, m1, m2, m3);
  if (lmax == 4 && w != 0.0 && std::fabs(w) < 1.0) {
    const double inv2 = 1.0 / (w * w);
    const double k = std::round(std::sqrt(inv2));
    if (k > 1.0 && std::fabs(inv2 - k * k) < 1e-9 * inv2) return 0.0;
  }
  return w;
}

inline int b3_n_ls(int lmax) {
  int n = 0;
  for (int l1 = 0; l1 <= lmax; l1++)
    for (int l2 = 0; l2 <= lmax; l2++)
      for (int l3 = 0; l3 <= lmax; l3++)
        if (std::abs(l1 - l2) <= l3 && l3 <= l1 + l2) n++;
  return n;
}

inline int upload_b3_tables(cudaStream_t stream) {
  static B3Tables t;  // 25 KB: not on the stack
  int nt = 0, nb = 0;
  for (int lmax = 0; lmax <= kB3MaxL; lmax++) {
    t.ls_off[lmax] = nb;
    for (int l1 = 0; l1 <= lmax; l1++)
      for (int l2 = 0; l2 <= lmax; l2++)
        for (int l3 = 0; l3 <= lmax; l3++) {
          if (std::abs(l1 - l2) > l3 || l3 > l1 + l2) continue;
          t.beg[nb++] = nt;
          for (int m1 = -l1; m1 <= l1; m1++)
            for (int m2 = -l2; m2 <= l2; m2++) {
              const int m3 = -m1 - m2;
              if (std::abs(m3) > l3) continue;
              // every (m1, m2) with |m3| <= l3 in loop order, zeros included,
              // so that the term offsets within a triangle are fixed
              const double w = b3_reference_coeff(l1, l2, l3, m1, m2, m3, lmax);
              if (nt >= kB3MaxTerms) return -1;
              t.idx[nt] = (unsigned)(l1 * l1 + l1 + m1) |
                          ((unsigned)(l2 * l2 + l2 + m2) << 8) |
                          ((unsigned)(l3 * l3 + l3 + m3) << 16);
              t.w[nt] = w;
              t.wf[nt] = (float)w;
              nt++;
            }
        }
    t.beg[nb++] = nt;  // end of the last triangle of this lmax
  }
  t.ls_off[kB3MaxL + 1] = nb;
  cudaError_t e =
      cudaMemcpyToSymbolAsync(c_b3, &t, sizeof(t), 0, cudaMemcpyHostToDevice, stream);
  return e == cudaSuccess ? 0 : -1;
}

// Real single-bond block c (nr x H, row stride ldc, default H) -> complex (zr, zi) with
// row stride H + 1 (padded so that lanes on different radial rows hit
// different banks).  Lane-strided; the caller synchronizes the warp.
template <typename T>
__device__ __forceinline__ void b3_to_complex(const T *__restrict__ c, int nr, int H,
                                              T *__restrict__ zr, T *__restrict__ zi,
                                              int lane, int ldc = -1) {
  const int HC = ldc < 0 ? H : ldc;  // row stride of c
  const T is2 = T(0.70710678118654752440);
  for (int k = lane; k < nr * H; k += 32) {
    const int n = k / H, lm = k - n * H;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) l++;
    const int m = lm - l * l - l;
    const int am = m < 0 ? -m : m;
    const T R = c[n * HC + l * l + l + am];
    const T S = c[n * HC + l * l + l - am];
    T re, im;
    if (m == 0) {
      re = R;
      im = T(0);
    } else if (m > 0) {
      const T sg = (am & 1) ? T(-1) : T(1);
      re = sg * R * is2;
      im = sg * S * is2;
    } else {
      re = R * is2;
      im = -S * is2;
    }
    zr[n * (H + 1) + lm] = re;
    zi[n * (H + 1) + lm] = im;
  }
}

// (re, im) pairs for 8-byte (FP32) / 16-byte (FP64) shared-memory accesses.
template <typename T> struct V2T;
template <> struct V2T<float> { using type = float2; };
template <> struct V2T<double> { using type = double2; };
template <typename T> using V2 = typename V2T<T>::type;

// b3_to_complex with the complex block interleaved: z[n * (H + 1) + lm] = (re, im).
template <typename T>
__device__ __forceinline__ void b3_to_complex2(const T *__restrict__ c, int nr, int H,
                                               V2<T> *__restrict__ z, int lane, int ldc = -1) {
  const int HC = ldc < 0 ? H : ldc;
  const T is2 = T(0.70710678118654752440);
  for (int k = lane; k < nr * H; k += 32) {
    const int n = k / H, lm = k - n * H;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) l++;
    const int m = lm - l * l - l;
    const int am = m < 0 ? -m : m;
    const T R = c[n * HC + l * l + l + am];
    const T S = c[n * HC + l * l + l - am];
    V2<T> v;
    if (m == 0) {
      v.x = R;
      v.y = T(0);
    } else if (m > 0) {
      const T sg = (am & 1) ? T(-1) : T(1);
      v.x = sg * R * is2;
      v.y = sg * S * is2;
    } else {
      v.x = R * is2;
      v.y = -S * is2;
    }
    z[n * (H + 1) + lm] = v;
  }
}

// p[r * n_ls + t] for every radial triple r (table tri: n1 | n2<<8 | n3<<16)
// and triangle t, from the interleaved complex block; lanes take triples, all
// lanes walk the same term list (the coefficients and harmonic indices are
// uniform loads from constant memory).
template <int LM, typename T>
__device__ __forceinline__ void b3_contract_fixed(const V2<T> *__restrict__ z1,
                                                  const V2<T> *__restrict__ z2,
                                                  const V2<T> *__restrict__ z3,
                                                  T *__restrict__ prow);

template <typename T, int LM = -1>
__device__ __forceinline__ void b3_contract(int lmax, int n_ls, int n_tri, int H,
                                             const int *__restrict__ tri,
                                             const V2<T> *__restrict__ z, T *__restrict__ p,
                                             int lane) {
  const int H1 = H + 1;
  if constexpr (LM >= 0) {
    // lmax = LM: every term unrolled (the same terms in the same order)
    for (int r = lane; r < n_tri; r += 32) {
      const int tr = tri[r];
      b3_contract_fixed<LM, T>(z + (tr & 0xff) * H1, z + ((tr >> 8) & 0xff) * H1,
                               z + (tr >> 16) * H1, p + r * n_ls);
    }
    return;
  }
  const int *beg = c_b3.beg + c_b3.ls_off[lmax];
  for (int t = 0; t < n_ls; t++) {
    const int e0 = beg[t], e1 = beg[t + 1];
    for (int r = lane; r < n_tri; r += 32) {
      const int tr = tri[r];
      const V2<T> *z1 = z + (tr & 0xff) * H1, *z2 = z + ((tr >> 8) & 0xff) * H1;
      const V2<T> *z3 = z + (tr >> 16) * H1;
      T acc = T(0);
      for (int e = e0; e < e1; e++) {
        const unsigned ix = c_b3.idx[e];
        const V2<T> a = z1[ix & 0xff], b = z2[(ix >> 8) & 0xff], c = z3[ix >> 16];
        const T xr = a.x * b.x - a.y * b.y, xi = a.x * b.y + a.y * b.x;
        acc += b3_w<T>(e) * (xr * c.x - xi * c.y);
      }
      p[r * n_ls + t] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// The term tables at compile time, in upload_b3_tables' order (lmax blocks,
// triangles l1, l2, l3 in loop order, then m1, m2): for a fixed lmax the
// adjoint below unrolls every term, so indices and coefficient addresses are
// constants and the per-term sums stay in registers.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int b3_iabs(int v) { return v < 0 ? -v : v; }
__host__ __device__ constexpr bool b3_tri_ok(int l1, int l2, int l3) {
  return !(b3_iabs(l1 - l2) > l3 || l3 > l1 + l2);
}
__host__ __device__ constexpr int b3_tri_terms(int l1, int l2, int l3) {
  int n = 0;
  for (int m1 = -l1; m1 <= l1; m1++)
    for (int m2 = -l2; m2 <= l2; m2++)
      if (b3_iabs(m1 + m2) <= l3) n++;
  return n;
}
// absolute index of the first term of triangle (L1, L2, L3) of block LM
__host__ __device__ constexpr int b3_tri_first(int LM, int L1, int L2, int L3) {
  int nt = 0;
  for (int lm = 0; lm <= LM; lm++)
    for (int l1 = 0; l1 <= lm; l1++)
      for (int l2 = 0; l2 <= lm; l2++)
        for (int l3 = 0; l3 <= lm; l3++) {
          if (!b3_tri_ok(l1, l2, l3)) continue;
          if (lm == LM && l1 == L1 && l2 == L2 && l3 == L3) return nt;
          nt += b3_tri_terms(l1, l2, l3);
        }
  return -1;
}
// index of triangle (L1, L2, L3) within block LM (the column of w)
__host__ __device__ constexpr int b3_tri_index(int LM, int L1, int L2, int L3) {
  int t = 0;
  for (int l1 = 0; l1 <= LM; l1++)
    for (int l2 = 0; l2 <= LM; l2++)
      for (int l3 = 0; l3 <= LM; l3++) {
        if (!b3_tri_ok(l1, l2, l3)) continue;
        if (l1 == L1 && l2 == L2 && l3 == L3) return t;
        t++;
      }
  return -1;
}
// offset of term (M1, M2) within its triangle
__host__ __device__ constexpr int b3_term_offset(int L1, int L2, int L3, int M1, int M2) {
  int n = 0;
  for (int m1 = -L1; m1 <= L1; m1++)
    for (int m2 = -L2; m2 <= L2; m2++) {
      if (b3_iabs(m1 + m2) > L3) continue;
      if (m1 == M1 && m2 == M2) return n;
      n++;
    }
  return -1;
}

template <int B, int E, typename F>
__device__ __forceinline__ void b3_static_for(F &&f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    b3_static_for<B + 1, E>(f);
  }
}

// One triangle of the adjoint for the lane's rows: p1 in registers (indexed
// by lm, every index a compile-time constant), p2 and p3 lane-private rows in
// shared memory (stride 32).  The terms of each m1 sum into a register pair
// before the one update of p1[l1 m1]; the rows of positions 2 and 3 sum in
// registers over the whole triangle before their one update.
template <int LM, int L1, int L2, int L3, typename T, int NLS, int HH>
__device__ __forceinline__ void b3_adjoint_triangle(const V2<T> *__restrict__ z1,
                                                    const V2<T> *__restrict__ z2,
                                                    const V2<T> *__restrict__ z3,
                                                    const T (&wr)[NLS], V2<T> (&p1)[HH],
                                                    V2<T> *p2, V2<T> *p3) {
  constexpr int t = b3_tri_index(LM, L1, L2, L3);
  constexpr int q0 = b3_tri_first(LM, L1, L2, L3);
  static_assert(t >= 0 && t < NLS && q0 >= 0, "triangle outside the tables");
  const T wq = wr[t];
  V2<T> s2[2 * L2 + 1], s3[2 * L3 + 1];
#pragma unroll
  for (int j = 0; j < 2 * L2 + 1; j++) s2[j] = V2<T>{T(0), T(0)};
#pragma unroll
  for (int j = 0; j < 2 * L3 + 1; j++) s3[j] = V2<T>{T(0), T(0)};
  b3_static_for<0, 2 * L1 + 1>([&](auto j1) {
    constexpr int m1 = decltype(j1)::value - L1;
    const V2<T> a = z1[L1 * L1 + L1 + m1];
    V2<T> s1{T(0), T(0)};
    b3_static_for<0, 2 * L2 + 1>([&](auto j2) {
      constexpr int m2 = decltype(j2)::value - L2;
      constexpr int m3 = -m1 - m2;
      if constexpr (b3_iabs(m3) <= L3) {
        constexpr int q = q0 + b3_term_offset(L1, L2, L3, m1, m2);
        const T f = wq * b3_w<T>(q);
        const V2<T> b = z2[L2 * L2 + L2 + m2], c = z3[L3 * L3 + L3 + m3];
        // f a and f b once, then each complex product added by multiply-adds
        const V2<T> fa{f * a.x, f * a.y}, fb{f * b.x, f * b.y};
        s1.x = fma_t(fb.x, c.x, s1.x);
        s1.x = fma_t(-fb.y, c.y, s1.x);
        s1.y = fma_t(fb.x, c.y, s1.y);
        s1.y = fma_t(fb.y, c.x, s1.y);
        V2<T> &t2 = s2[m2 + L2], &t3 = s3[m3 + L3];
        t2.x = fma_t(fa.x, c.x, t2.x);
        t2.x = fma_t(-fa.y, c.y, t2.x);
        t2.y = fma_t(fa.x, c.y, t2.y);
        t2.y = fma_t(fa.y, c.x, t2.y);
        t3.x = fma_t(fa.x, b.x, t3.x);
        t3.x = fma_t(-fa.y, b.y, t3.x);
        t3.y = fma_t(fa.x, b.y, t3.y);
        t3.y = fma_t(fa.y, b.x, t3.y);
      }
    });
    V2<T> &d = p1[L1 * L1 + L1 + m1];
    d.x += s1.x;
    d.y += s1.y;
  });
#pragma unroll
  for (int j = 0; j < 2 * L2 + 1; j++) {
    V2<T> &d = p2[(L2 * L2 + j) * 32];
    d.x += s2[j].x;
    d.y += s2[j].y;
  }
#pragma unroll
  for (int j = 0; j < 2 * L3 + 1; j++) {
    V2<T> &d = p3[(L3 * L3 + j) * 32];
    d.x += s3[j].x;
    d.y += s3[j].y;
  }
}

// The forward sum of one triangle for one radial triple, terms in table order.
template <int LM, int L1, int L2, int L3, typename T>
__device__ __forceinline__ T b3_contract_triangle(const V2<T> *__restrict__ z1,
                                                  const V2<T> *__restrict__ z2,
                                                  const V2<T> *__restrict__ z3) {
  constexpr int q0 = b3_tri_first(LM, L1, L2, L3);
  static_assert(q0 >= 0, "triangle outside the tables");
  // per m1: S = sum_m2 w_q b c (complex), then Re(a S) once
  T acc = T(0);
  b3_static_for<0, 2 * L1 + 1>([&](auto j1) {
    constexpr int m1 = decltype(j1)::value - L1;
    V2<T> sm{T(0), T(0)};
    b3_static_for<0, 2 * L2 + 1>([&](auto j2) {
      constexpr int m2 = decltype(j2)::value - L2;
      constexpr int m3 = -m1 - m2;
      if constexpr (b3_iabs(m3) <= L3) {
        constexpr int q = q0 + b3_term_offset(L1, L2, L3, m1, m2);
        const V2<T> b = z2[L2 * L2 + L2 + m2], c = z3[L3 * L3 + L3 + m3];
        const T br = b.x * c.x - b.y * c.y, bi = b.x * c.y + b.y * c.x;
        const T w = b3_w<T>(q);
        sm.x = fma_t(w, br, sm.x);
        sm.y = fma_t(w, bi, sm.y);
      }
    });
    const V2<T> a = z1[L1 * L1 + L1 + m1];
    acc = fma_t(a.x, sm.x, acc);
    acc = fma_t(-a.y, sm.y, acc);
  });
  return acc;
}

template <int LM, typename T>
__device__ __forceinline__ void b3_contract_fixed(const V2<T> *__restrict__ z1,
                                                  const V2<T> *__restrict__ z2,
                                                  const V2<T> *__restrict__ z3,
                                                  T *__restrict__ prow) {
  b3_static_for<0, LM + 1>([&](auto i1) {
    b3_static_for<0, LM + 1>([&](auto i2) {
      b3_static_for<0, LM + 1>([&](auto i3) {
        constexpr int l1 = decltype(i1)::value, l2 = decltype(i2)::value,
                      l3 = decltype(i3)::value;
        if constexpr (b3_tri_ok(l1, l2, l3))
          prow[b3_tri_index(LM, l1, l2, l3)] = b3_contract_triangle<LM, l1, l2, l3, T>(z1, z2, z3);
      });
    });
  });
}

// Every triangle of block LM, in table order.
// triangles of block LM (b3_n_ls at compile time)
__host__ __device__ constexpr int b3_n_triangles(int LM) {
  int t = 0;
  for (int l1 = 0; l1 <= LM; l1++)
    for (int l2 = 0; l2 <= LM; l2++)
      for (int l3 = 0; l3 <= LM; l3++)
        if (b3_tri_ok(l1, l2, l3)) t++;
  return t;
}

template <int LM, typename T, int NLS, int HH>
__device__ __forceinline__ void b3_adjoint_fixed(const V2<T> *__restrict__ z1,
                                                 const V2<T> *__restrict__ z2,
                                                 const V2<T> *__restrict__ z3,
                                                 const T (&wr)[NLS], V2<T> (&p1)[HH],
                                                 V2<T> *p2, V2<T> *p3) {
  b3_static_for<0, LM + 1>([&](auto i1) {
    b3_static_for<0, LM + 1>([&](auto i2) {
      b3_static_for<0, LM + 1>([&](auto i3) {
        constexpr int l1 = decltype(i1)::value, l2 = decltype(i2)::value,
                      l3 = decltype(i3)::value;
        if constexpr (b3_tri_ok(l1, l2, l3))
          b3_adjoint_triangle<LM, l1, l2, l3, T, NLS, HH>(z1, z2, z3, wr, p1, p2, p3);
      });
    });
  });
}

// Adjoint of b3_contract: for dE/dp = w, the holomorphic derivative
// u = dE/dc summed into u2[n * H + lm] = (re, im).  Lanes take radial triples
// in rounds of 32; within a round lane r only updates the rows n1(r), n2(r),
// n3(r) of its own triple, so it accumulates into three private rows in
// shared memory, priv[(pos * H + lm) * 32 + lane] (conflict-free banks, no
// atomics).  After each round the private rows are summed into u2 by output
// entry, over lanes in a fixed rotated order.  The caller zeroes u2 and
// synchronizes the warp before and after.
// u2[n, lm] += the private rows of one round, over lanes j in a fixed rotated
// order (lanes read different banks) and positions with n_pos(j) == n.  Each
// lane reads its own triple once; the others come by shuffle, in loops whose
// trip counts are the same for every lane.
template <typename T>
__device__ __forceinline__ void b3_reduce_private(int r0, int n_tri, int H, int nr,
                                                  const int *__restrict__ tri,
                                                  const V2<T> *__restrict__ priv,
                                                  V2<T> *__restrict__ u2, int lane) {
  const int own = r0 + lane < n_tri ? tri[r0 + lane] : -1;
  const int total = nr * H;
  for (int k0 = 0; k0 < total; k0 += 32) {
    const int k = k0 + lane;
    const bool act = k < total;
    const int n = act ? k / H : -1;
    const int lm = act ? k - n * H : 0;
    V2<T> acc{T(0), T(0)};
    for (int j0 = 0; j0 < 32; j0++) {
      const int j = (j0 + lane) & 31;
      const int tj = __shfl_sync(0xffffffffu, own, j);
      if (tj < 0) continue;  // no triple in this round's slot j
      const V2<T> *col = priv + (size_t)lm * 32 + j;
      if ((tj & 0xff) == n) {
        const V2<T> v = col[0];
        acc.x += v.x;
        acc.y += v.y;
      }
      if (((tj >> 8) & 0xff) == n) {
        const V2<T> v = col[H * 32];
        acc.x += v.x;
        acc.y += v.y;
      }
      if ((tj >> 16) == n) {
        const V2<T> v = col[(2 * H) * 32];
        acc.x += v.x;
        acc.y += v.y;
      }
    }
    if (act) {
      u2[k].x += acc.x;
      u2[k].y += acc.y;
    }
  }
}

// b3_reduce_private for npos (1 or 2) positions pos0 .. pos0 + npos - 1 of
// the triples, their rows at rows[(p * H + lm) * 32 + lane], p < npos.  The
// lanes whose triple holds row n at those positions come from one ballot per
// position and row value; each output entry then visits just those lanes, in
// the order lane, lane + 1, ... (mod 32) and position by position within a
// lane, the order of the full slot scan, so the sums are the same.
template <typename T>
__device__ __forceinline__ void b3_reduce_rows(int r0, int n_tri, int H, int nr,
                                               const int *__restrict__ tri,
                                               const V2<T> *__restrict__ rows, int pos0,
                                               int npos, V2<T> *__restrict__ u2, int lane) {
  const int own = r0 + lane < n_tri ? tri[r0 + lane] : -1;
  // the rows of this lane's triple at the positions summed here (-1: none)
  const int row0 = own < 0 ? -1 : (own >> (8 * pos0)) & 0xff;
  const int row1 = (own < 0 || npos < 2) ? -1 : (own >> (8 * (pos0 + 1))) & 0xff;
  const int total = nr * H;
  for (int k0 = 0; k0 < total; k0 += 32) {
    const int k = k0 + lane;
    const bool act = k < total;
    const int n = act ? k / H : -1;
    const int lm = act ? k - n * H : 0;
    // the contributing lanes for each row value n of this group of outputs
    unsigned m0 = 0u, m1 = 0u;
    const int nlo = k0 / H, nhi = min(k0 + 31, total - 1) / H;
    for (int nn = nlo; nn <= nhi; nn++) {
      const unsigned b0 = __ballot_sync(0xffffffffu, row0 == nn);
      const unsigned b1 = __ballot_sync(0xffffffffu, row1 == nn);
      if (nn == n) {
        m0 = b0;
        m1 = b1;
      }
    }
    V2<T> acc{T(0), T(0)};
    const unsigned any = m0 | m1;
    unsigned r = __funnelshift_r(any, any, lane);  // bit b: lane (b + lane) mod 32
    while (r) {
      const int b = __ffs(r) - 1;
      r &= r - 1u;
      const int j = (b + lane) & 31;
      const V2<T> *col = rows + (size_t)lm * 32 + j;
      if ((m0 >> j) & 1u) {
        const V2<T> v = col[0];
        acc.x += v.x;
        acc.y += v.y;
      }
      if ((m1 >> j) & 1u) {
        const V2<T> v = col[(size_t)H * 32];
        acc.x += v.x;
        acc.y += v.y;
      }
    }
    if (act) {
      u2[k].x += acc.x;
      u2[k].y += acc.y;
    }
  }
}

// The adjoint with every term unrolled for lmax = LM.  Each lane first copies
// its triple's row of w into registers, so the rows of the first round (wa)
// may share memory with the private rows; the rows of later rounds (wb, triple
// r >= 32 at wb + (r - 32) n_ls) are kept apart.
template <typename T, int LM>
__device__ __forceinline__ void b3_contract_adjoint_fixed(int n_tri, int H, int nr,
                                                          const int *__restrict__ tri,
                                                          const V2<T> *__restrict__ z,
                                                          const T *wa, const T *wb,
                                                          V2<T> *priv, V2<T> *__restrict__ u2,
                                                          int lane) {
  constexpr int NLS = b3_n_triangles(LM);
  constexpr int HH = (LM + 1) * (LM + 1);
  const int H1 = H + 1;
  for (int r0 = 0; r0 < n_tri; r0 += 32) {
    const int r = r0 + lane;
    const bool live = r < n_tri;
    const int tr = live ? tri[r] : 0;
    T wr[NLS];
    const T *wrow = r < 32 ? wa + r * NLS : wb + (r - 32) * NLS;
#pragma unroll
    for (int t = 0; t < NLS; t++) wr[t] = live ? wrow[t] : T(0);
    V2<T> p1[HH];  // position 1 in registers, positions 2 and 3 in priv
#pragma unroll
    for (int k = 0; k < HH; k++) p1[k] = V2<T>{T(0), T(0)};
    __syncwarp();  // every row is in registers before the private rows are zeroed
    for (int k = 0; k < 2 * H; k++) priv[k * 32 + lane] = V2<T>{T(0), T(0)};
    if (live) {
      const int n1 = tr & 0xff, n2 = (tr >> 8) & 0xff, n3 = tr >> 16;
      b3_adjoint_fixed<LM, T, NLS, HH>(z + n1 * H1, z + n2 * H1, z + n3 * H1, wr, p1,
                                       priv + lane, priv + (size_t)H * 32 + lane);
    }
    __syncwarp();
    b3_reduce_rows<T>(r0, n_tri, H, nr, tri, priv, 1, 2, u2, lane);  // positions 2, 3
    __syncwarp();
#pragma unroll
    for (int k = 0; k < HH; k++) priv[k * 32 + lane] = p1[k];
    __syncwarp();
    b3_reduce_rows<T>(r0, n_tri, H, nr, tri, priv, 0, 1, u2, lane);  // position 1
    __syncwarp();
  }
}

template <typename T>
__device__ __forceinline__ void b3_contract_adjoint(int lmax, int n_ls, int n_tri, int H,
                                                    int nr, const int *__restrict__ tri,
                                                    const V2<T> *__restrict__ z,
                                                    const T *__restrict__ w,
                                                    V2<T> *__restrict__ priv,
                                                    V2<T> *__restrict__ u2, int lane) {
  const int H1 = H + 1;
  const int *beg = c_b3.beg + c_b3.ls_off[lmax];
  for (int r0 = 0; r0 < n_tri; r0 += 32) {
    const int r = r0 + lane;
    const bool live = r < n_tri;
    const int tr = live ? tri[r] : 0;
    for (int k = 0; k < 3 * H; k++) priv[k * 32 + lane] = V2<T>{T(0), T(0)};
    if (live) {
      const int n1 = tr & 0xff, n2 = (tr >> 8) & 0xff, n3 = tr >> 16;
      const V2<T> *z1 = z + n1 * H1, *z2 = z + n2 * H1, *z3 = z + n3 * H1;
      V2<T> *p1 = priv + lane;
      V2<T> *p2 = priv + (size_t)H * 32 + lane;
      V2<T> *p3 = priv + (size_t)(2 * H) * 32 + lane;
      for (int t = 0; t < n_ls; t++) {
        const int e0 = beg[t], e1 = beg[t + 1];
        const T wq = w[r * n_ls + t];
        for (int q = e0; q < e1; q++) {
          const unsigned ix = c_b3.idx[q];
          const int i1 = ix & 0xff, i2 = (ix >> 8) & 0xff, i3 = ix >> 16;
          const T f = wq * b3_w<T>(q);
          const V2<T> a = z1[i1], b = z2[i2], c = z3[i3];
          V2<T> s1 = p1[i1 * 32], s2 = p2[i2 * 32], s3 = p3[i3 * 32];
          s1.x += f * (b.x * c.x - b.y * c.y);
          s1.y += f * (b.x * c.y + b.y * c.x);
          s2.x += f * (a.x * c.x - a.y * c.y);
          s2.y += f * (a.x * c.y + a.y * c.x);
          s3.x += f * (a.x * b.x - a.y * b.y);
          s3.y += f * (a.x * b.y + a.y * b.x);
          p1[i1 * 32] = s1;
          p2[i2 * 32] = s2;
          p3[i3 * 32] = s3;
        }
      }
    }
    __syncwarp();
    b3_reduce_private<T>(r0, n_tri, H, nr, tri, priv, u2, lane);
    __syncwarp();
  }
}

}  // namespace fpp
