// B2 descriptor forward pass and its adjoint (forces and virial without the
// stored descriptor_force_dervs tensor).
//
// Forward (one warp per atom), src/flare_pp/descriptors/b2.cpp:244-399 and
// :181-242:
//   c[(s N + n) H + lm] = sum_j g_n(r_ij) Y_lm(r_ij)   over neighbors of species s
//                          with r_ij <= cutoffs[s_i][s_j]
//   p[(n1, n2 >= n1, l)] = sum_m c[n1, lm] c[n2, lm],  |p| in FP64
// The neighbor bases are computed one neighbor per lane and staged in shared
// memory; each lane then owns one (l, m) column and accumulates all radial
// channels in registers (compensated in FP32).
//
// Adjoint (one warp per atom), lammps_plugins/lammps_descriptor.cpp:250-304 and
// pair_flare.cpp:141-175:
//   w = dE/dp, u[n1, lm] = sum_n2 (W + W^T)[n1, n2, l] c[n2, lm]
//   f_ij = dE/dr_ij = sum_{n, lm} u[s_j N + n, lm] d(g_n Y_lm)/dr_ij
// with the bases recomputed per pair.  Forces are then gathered per atom from
// f_ij and the reverse pair's f_ji, so the result is deterministic.
#include <cuda_fp16.h>

#include <algorithm>

#include "basis.cuh"
#include "b2_kernels.h"
#include "b3.cuh"
#include "common.cuh"
#include "tc_prims.cuh"

namespace fpp {

int upload_descriptor_tables(cudaStream_t stream) { return upload_b3_tables(stream); }

void fill_fp32_cutoffs(B2Args &a) {
  a.r1f = (float)a.r1;
  for (int k = 0; k < kMaxSpecies * kMaxSpecies; k++) {
    const double rc = a.cutoffs[k];
    a.cutoffs32[k] = (float)rc;
    // fl32(r) < cut_lo  =>  r <= fl32(r) (1 + 2^-24) < rc, and symmetrically
    a.cut_lo[k] = nextafterf((float)(rc * (1.0 - 1e-6)), 0.0f);
    a.cut_hi[k] = nextafterf((float)(rc * (1.0 + 1e-6)), 3.0e38f);
    const double ci = rc > a.r1 ? 1.0 / (rc - a.r1) : 0.0;
    a.cinv_hi[k] = (float)ci;
    a.cinv_lo[k] = (float)(ci - (double)a.cinv_hi[k]);
  }
}

// Descriptor filter r <= rc of b2.cpp:277 / b3.cpp:258 for pair p of atom i,
// FP32 first: only pairs within the band around rc use the FP64 distance,
// recomputed from the positions (or read from the caller's FP64 table).
static __device__ __noinline__ bool band_keep(const dvec4 *__restrict__ rel,
                                              const NbGeom *geom, int i, long long p,
                                              double rc) {
  const double r = geom ? exact_pair_dist(*geom, i, p) : rel[p].x;
  return r <= rc;
}

__device__ __forceinline__ bool keep_pair32(const B2Args &a, int k, float rf,
                                            const dvec4 *__restrict__ rel,
                                            const NbGeom *geom, int i, long long p) {
  if (rf < a.cut_lo[k]) return true;
  if (rf > a.cut_hi[k]) return false;
  return band_keep(rel, geom, i, p, a.cutoffs[k]);  // out of line: FP64
}
int b3_n_ls_host(int lmax) { return b3_n_ls(lmax); }

int upload_harmonic_tables(cudaStream_t stream) {
  HarmonicTables t;
  const double pi = 3.14159265358979323846;
  for (int l = 0; l <= kMaxL; l++)
    for (int m = 0; m <= kMaxL; m++) {
      double v = 0;
      if (m <= l) {
        double f = 1;
        for (int k = l - m + 1; k <= l + m; k++) f *= k;  // (l+m)!/(l-m)!
        v = sqrt((2 * l + 1) / (4 * pi) / f);
        if (m > 0) v *= sqrt(2.0);
      }
      t.norm[l * (kMaxL + 1) + m] = v;
      double dl = 1;  // D_lm of the division-free FP32 recurrence
      for (int k = m + 2; k <= l; k++) dl *= k - m;
      const double vf = v / dl;
      t.norm_hi[l * (kMaxL + 1) + m] = (float)vf;
      t.norm_lo[l * (kMaxL + 1) + m] = (float)(vf - (double)(float)vf);
    }
  for (int m = 0; m <= kMaxL; m++) {
    double d = 1;
    for (int k = 1; k < 2 * m; k += 2) d *= k;
    t.dfact[m] = d;
    t.dfact_f[m] = (float)d;
  }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_harm, &t, sizeof(t), 0,
                                          cudaMemcpyHostToDevice, stream);
  return e == cudaSuccess ? 0 : -1;
}

// Running sum; compensated (Neumaier) when T is float.
template <typename T> struct Acc {
  T s = T(0), c = T(0);
  __device__ __forceinline__ void add(T x) {
    if (sizeof(T) == 4) {
      T t = s + x;
      if (fabs_t(s) >= fabs_t(x))
        c += (s - t) + x;
      else
        c += (x - t) + s;
      s = t;
    } else {
      s += x;
    }
  }
};

// x^2 + y^2 + z^2 of a pair vector, rounded as the host computes it.
__device__ __forceinline__ double rsq_exact(const dvec4 &r) {
  return dadd(dadd(dmul(r.y, r.y), dmul(r.z, r.z)), dmul(r.w, r.w));
}

// The pair style's filter rsq < rc^2 (pair_flare.cpp:150) for the FP32
// kernels, out of line: inline, its FP64 instructions were issued (predicated
// off) for every pair of the non-strict default as well.
static __device__ __noinline__ bool strict_keep(const dvec4 *__restrict__ rel, long long p,
                                                double rc) {
  return rsq_exact(rel[p]) < dmul(rc, rc);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Error-free sum a + b = s + e (Knuth's two-sum), FP32.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Warp sum of the float-float values (hi, lo), kept as float-float: FP32
// arithmetic only (FP64 instructions are scarce on this GPU).
__device__ __forceinline__ void ff_warp_sum(float &hi, float &lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    float s, e;
    two_sum(hi, h2, s, e);
    e += lo + l2;
    hi = s + e;
    lo = e - (hi - s);
  }
}

// Descriptor shape known at compile time for the common settings (N, lmax,
// n_species), or read from the arguments (the generic instantiation).  With
// the sizes constant, the radial / harmonic loops unroll and the shared-memory
// and u indices fold into immediate offsets.
template <int NT, int LT, int NST> struct Shape {
  static constexpr int kN = NT > 0 ? NT : 0;
  static constexpr int kNR = (NT > 0 && NST > 0) ? NT * NST : 0;  // radial channels
  static constexpr int kL1 = LT >= 0 ? LT + 1 : 0;
  static __device__ __forceinline__ int N(const B2Args &a) { return NT > 0 ? NT : a.N; }
  static __device__ __forceinline__ int lmax(const B2Args &a) { return LT >= 0 ? LT : a.lmax; }
  static __device__ __forceinline__ int NS(const B2Args &a) {
    return NST > 0 ? NST : a.n_species;
  }
};
using GenericShape = Shape<0, -1, 0>;

// f(shape) with the compile-time shape matching a, else the generic one.
// The FP64 (reference-precision) kernels are instantiated generic only.
template <typename T, typename F>
int with_shape(const B2Args &a, F &&f) {
  if constexpr (sizeof(T) == 4) {
    if (a.kind == kB2) {
      if (a.n_species == 2 && a.N == 12 && a.lmax == 4) return f(Shape<12, 4, 2>{});
      if (a.n_species == 2 && a.N == 10 && a.lmax == 4) return f(Shape<10, 4, 2>{});
      if (a.n_species == 2 && a.N == 8 && a.lmax == 3) return f(Shape<8, 3, 2>{});
      if (a.n_species == 1 && a.N == 8 && a.lmax == 3) return f(Shape<8, 3, 1>{});
    } else if (a.kind == kB3) {
      // the shape-specialised single-bond and pair stages; the bispectrum
      // contraction and its adjoint keep runtime loops
      if (a.n_species == 1 && a.N == 6 && a.lmax == 3) return f(Shape<6, 3, 1>{});
    }
  }
  return f(GenericShape{});
}

// ---------------------------------------------------------------------------
// Forward: one warp per atom.
//   1. stage the bases of up to W neighbors (one neighbor per lane) and list
//      the staged neighbors by species (warp ballots);
//   2. lane = (l, m) column: for each species, run over its listed neighbors
//      accumulating the N radial channels in registers (plain sums over 16
//      neighbors, Kahan-folded into per-channel sums within the window; the
//      folded sum carries over to the next window in shared memory);
//   3. B2 contraction per radial pair (n1, n2 >= n1) into shared memory with
//      a compensated norm, then the normalized / split outputs.
// ---------------------------------------------------------------------------
template <typename T> struct FwdLayout {
  int W, GP;            // window, padded radial stride (multiple of 4)
  size_t stage, csum;   // bytes: staging (reused for p), c sums + compensation
  size_t lists, cz;     // species lists; B3: complex c (re, im), rows padded to H+1
  size_t total;
};

template <typename T>
__host__ __device__ inline FwdLayout<T> fwd_layout(const B2Args &a) {
  FwdLayout<T> L;
  L.W = a.window;
  L.GP = (a.N + 3) & ~3;
  // c rows padded to a multiple of 4 entries (16-byte aligned rows)
  const int sbp = a.n_species * a.N * ((a.H + 3) & ~3);
  size_t st = sizeof(T) * ((size_t)L.W * L.GP + (size_t)a.H * (L.W + 1));
  size_t pb = sizeof(T) * (size_t)a.n_d;
  L.stage = ((st > pb ? st : pb) + 15) & ~(size_t)15;
  // FP32: running sums only (compensated within a window); FP64: running
  // sums and their compensation terms across windows
  L.csum = (sizeof(T) * (sizeof(T) == 8 ? 2 : 1) * (size_t)sbp + 15) & ~(size_t)15;
  L.lists = (sizeof(int) * ((size_t)a.n_species * L.W + 2 * L.W + a.n_species) + 15) & ~(size_t)15;
  L.cz = a.kind == kB3
             ? (sizeof(T) * 2 * (size_t)a.n_species * a.N * (a.H + 1) + 15) & ~(size_t)15
             : 0;
  L.total = L.stage + L.csum + L.lists + L.cz;
  return L;
}

// FP32: registers capped for six blocks of four warps per SM (the shared
// memory allows six); FP64: no cap (it would spill)
template <typename T, typename SH>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 6 : 1)
k_b2_forward(B2Args a, const int *__restrict__ offset,
             const dvec4 *__restrict__ rel, const float4 *__restrict__ rel32, const NbGeom *geom,
             const int *__restrict__ nbr_s, const int *__restrict__ species,
             const int *__restrict__ row_of_atom, const int *__restrict__ pair_tab,
             T *__restrict__ c_out, T *__restrict__ p_out,
             double *__restrict__ norm_out, double *__restrict__ phat64,
             __half *__restrict__ phat_hi, __half *__restrict__ phat_lo, int ldp,
             const float *__restrict__ pbar) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int atom = blockIdx.x * nwarps + warp;
  const FwdLayout<T> Lay = fwd_layout<T>(a);
  const int N = SH::N(a), LMAX = SH::lmax(a), H = (LMAX + 1) * (LMAX + 1), NS = SH::NS(a);
  const int W = Lay.W, GP = Lay.GP;
  const int WS = W + 1;
  const int sb = NS * N * H;
  const int HP = (H + 3) & ~3, sbp = NS * N * HP;     // padded c row stride
  unsigned char *base = smem_raw + Lay.total * warp;
  T *g_s = reinterpret_cast<T *>(base);               // [W][GP]
  T *y_s = g_s + (size_t)W * GP;                      // [H][WS]
  T *p_s = reinterpret_cast<T *>(base);               // [n_d] (after staging)
  T *c_s = reinterpret_cast<T *>(base + Lay.stage);   // [NS N][HP] running sums
  T *cc_s = c_s + sbp;  // FP64 only: [NS N][HP] compensation
  int *list = reinterpret_cast<int *>(base + Lay.stage + Lay.csum);  // [NS][W]
  int *cnt_s = list + NS * W;                         // [NS]
  if (atom >= a.noa) return;

  for (int k = lane; k < sbp; k += 32) {
    c_s[k] = T(0);
    if (sizeof(T) == 8) cc_s[k] = T(0);
  }
  const int si = species[atom];
  const int beg = offset[atom], end = offset[atom + 1];
  __syncwarp();
  for (int w0 = beg; w0 < end; w0 += W) {
    const int cnt = min(W, end - w0);
    // ---- 1. stage bases and species lists ----
    if (lane < NS) cnt_s[lane] = 0;
    __syncwarp();
    for (int b0 = 0; b0 < cnt; b0 += 32) {
      const int b = b0 + lane;
      int sj = -1;
      if (b < cnt) {
        const int p = w0 + b;
        const int sp = nbr_s[p];
        const int kc = si * NS + sp;
        T r, x, y, z, r1t, rct;
        bool keep;
        if (sizeof(T) == 8) {
          const dvec4 rd = rel[p];
          const double rcut = a.cutoffs[kc];
          keep = a.strict ? (rsq_exact(rd) < dmul(rcut, rcut)) : (rd.x <= rcut);
          r = T(rd.x);
          x = T(rd.y);
          y = T(rd.z);
          z = T(rd.w);
          r1t = T(a.r1);
          rct = T(rcut);
        } else {
          const float4 rf = rel32[p];
          x = T(rf.x);
          y = T(rf.y);
          z = T(rf.z);
          r = T(rf.w);
          if (a.strict)
            keep = strict_keep(rel, p, a.cutoffs[kc]);
          else
            keep = keep_pair32(a, kc, rf.w, rel, geom, atom, p);
          r1t = T(a.r1f);
          rct = T(a.cutoffs32[kc]);
        }
        if (keep) {
          sj = sp;
          // FP32: hi/lo reciprocal of (rc - r1); FP64: the division
          radial_basis<T>(r, r1t, rct, N, a.cutoff_kind, g_s + (size_t)b * GP,
                          nullptr, 1, sizeof(T) == 4 ? T(a.cinv_hi[kc]) : T(0),
                          sizeof(T) == 4 ? T(a.cinv_lo[kc]) : T(0));
          real_harmonics<T>(x, y, z, LMAX, y_s + b, nullptr, WS);
        }
      }
      for (int sp = 0; sp < NS; sp++) {
        const unsigned m = __ballot_sync(0xffffffffu, sj == sp);
        if (sj == sp) list[sp * W + cnt_s[sp] + __popc(m & ((1u << lane) - 1u))] = b;
        __syncwarp();
        if (lane == 0) cnt_s[sp] += __popc(m);
        __syncwarp();
      }
    }
    __syncwarp();
    // ---- 2. accumulate: lane owns column lm ----
    for (int sp = 0; sp < NS; sp++) {
      const int ns_ = cnt_s[sp];
      if (ns_ == 0) continue;
      const int *ls = list + sp * W;
      for (int lm0 = 0; lm0 < H; lm0 += 32) {
        const int lm = lm0 + lane;
        const bool act = lm < H;
        const int lmc = act ? lm : 0;
        T sum[kMaxN], comp[kMaxN];
#pragma unroll
        for (int n = 0; n < kMaxN; n++)
          if (n < N) {
            sum[n] = c_s[(sp * N + n) * HP + lmc];
            // FP32: compensated within the window and folded at its end
            comp[n] = sizeof(T) == 8 ? cc_s[(sp * N + n) * HP + lmc] : T(0);
          }
        for (int k0 = 0; k0 < ns_; k0 += 16) {
          T chunk[kMaxN];
#pragma unroll
          for (int n = 0; n < kMaxN; n++) chunk[n] = T(0);
          const int k1 = min(ns_, k0 + 16);
          if constexpr (SH::kN > 0 && sizeof(T) == 4) {
            // radial row of the neighbor in 16-byte loads (GP = N rounded up
            // to 4), channels accumulated in pairs with paired multiply-adds
            // (pad channels past N are computed and discarded)
            constexpr int G4 = (SH::kN + 3) / 4;
            float2 c2[2 * G4];
#pragma unroll
            for (int j = 0; j < 2 * G4; j++) c2[j] = make_float2(0.f, 0.f);
            auto accum = [&](int b) {
              const float yv = y_s[lmc * WS + b];
              const float2 y2 = make_float2(yv, yv);
              const float4 *gb4 = reinterpret_cast<const float4 *>(g_s + (size_t)b * (4 * G4));
#pragma unroll
              for (int j = 0; j < G4; j++) {
                const float4 gv = gb4[j];
                c2[2 * j] = ffma2(make_float2(gv.x, gv.y), y2, c2[2 * j]);
                c2[2 * j + 1] = ffma2(make_float2(gv.z, gv.w), y2, c2[2 * j + 1]);
              }
            };
            // two neighbors per iteration (same summation order)
            int k = k0;
            for (; k + 1 < k1; k += 2) {
              const int b0 = ls[k], b1 = ls[k + 1];
              accum(b0);
              accum(b1);
            }
            if (k < k1) accum(ls[k]);
#pragma unroll
            for (int j = 0; j < 2 * G4; j++) {
              if (2 * j < SH::kN) chunk[2 * j] = c2[j].x;
              if (2 * j + 1 < SH::kN) chunk[2 * j + 1] = c2[j].y;
            }
          } else {
            for (int k = k0; k < k1; k++) {
              const int b = ls[k];
              const T yv = y_s[lmc * WS + b];
              const T *gb = g_s + (size_t)b * GP;
#pragma unroll
              for (int n = 0; n < kMaxN; n++)
                if (n < N) chunk[n] += gb[n] * yv;
            }
          }
#pragma unroll
          for (int n = 0; n < kMaxN; n++)
            if (n < N) {  // Kahan fold of the chunk
              const T yk = chunk[n] - comp[n];
              const T t = sum[n] + yk;
              comp[n] = (t - sum[n]) - yk;
              sum[n] = t;
            }
        }
        if (act) {
#pragma unroll
          for (int n = 0; n < kMaxN; n++)
            if (n < N) {
              if (sizeof(T) == 8) {
                c_s[(sp * N + n) * HP + lm] = sum[n];
                cc_s[(sp * N + n) * HP + lm] = comp[n];
              } else {
                c_s[(sp * N + n) * HP + lm] = sum[n] - comp[n];
              }
            }
        }
      }
    }
    __syncwarp();
  }
  // (FP64: fold the compensation) publish c (unpadded rows in global memory)
  for (int k = lane; k < sb; k += 32) {
    const int r = k / H, lm = k - r * H;
    T v = c_s[r * HP + lm];
    if (sizeof(T) == 8) {
      v -= cc_s[r * HP + lm];
      c_s[r * HP + lm] = v;
    }
    c_out[(size_t)atom * sb + k] = v;
  }
  __syncwarp();
  // ---- 3. B2 contraction per radial pair q, all l (B3: per radial triple) ----
  const int L1 = LMAX + 1;
  const int nd = a.n_d;
  const int npair = a.kind == kB3 ? 0 : nd / L1;
  Acc<T> nacc;
  if (a.kind == kB3) {
    V2<T> *z = reinterpret_cast<V2<T> *>(base + Lay.stage + Lay.csum + Lay.lists);
    b3_to_complex2<T>(c_s, NS * N, H, z, lane, HP);
    __syncwarp();
    // FP32 at lmax 3 (the B3 workload shape): the contraction unrolled
    constexpr int kB3L = (sizeof(T) == 4 && SH::kL1 == 4) ? 3 : -1;
    b3_contract<T, kB3L>(a.lmax, a.n_ls, a.n_tri, H, pair_tab, z, p_s, lane);
    __syncwarp();
    for (int d = lane; d < nd; d += 32) nacc.add(p_s[d] * p_s[d]);
  }
  if constexpr (SH::kL1 > 0 && SH::kNR >= 16 && (SH::kNR % 2) == 0 && sizeof(T) == 4) {
    // shape known, FP32, at least 16 radial channels: 2 x 2 blocks of c rows
    // (2a, 2a + 1) x (2b, 2b + 1), a <= b, one block per lane, so that four
    // rows read through 16-byte loads give four pairs (three on the diagonal
    // blocks); each entry m feeds the chain of its l, every p value the same
    // chain of fmaf as for one pair at a time
    constexpr int LL = SH::kL1, HH = LL * LL, H4 = (HH + 3) / 4, NR = SH::kNR;
    constexpr int NB = NR / 2, NBLK = NB * (NB + 1) / 2;
    auto l_of = [](int m) { int l = 0; while ((l + 1) * (l + 1) <= m) l++; return l; };
    auto q_of = [](int n1, int n2) { return n1 * NR - (n1 * (n1 - 1)) / 2 + (n2 - n1); };
    for (int j = lane; j < NBLK; j += 32) {
      int ba = 0, rem = j;
      while (rem >= NB - ba) {
        rem -= NB - ba;
        ba++;
      }
      const int bb = ba + rem;
      const float4 *x0 = reinterpret_cast<const float4 *>(c_s + (2 * ba) * HP);
      const float4 *x1 = reinterpret_cast<const float4 *>(c_s + (2 * ba + 1) * HP);
      const float4 *y0 = reinterpret_cast<const float4 *>(c_s + (2 * bb) * HP);
      const float4 *y1 = reinterpret_cast<const float4 *>(c_s + (2 * bb + 1) * HP);
      float v00[LL], v01[LL], v10[LL], v11[LL];
#pragma unroll
      for (int l = 0; l < LL; l++) v00[l] = v01[l] = v10[l] = v11[l] = 0.0f;
#pragma unroll
      for (int k = 0; k < H4; k++) {
        const float4 a0 = x0[k], a1 = x1[k], b0 = y0[k], b1 = y1[k];
        const float u0[4] = {a0.x, a0.y, a0.z, a0.w}, u1[4] = {a1.x, a1.y, a1.z, a1.w};
        const float w0[4] = {b0.x, b0.y, b0.z, b0.w}, w1[4] = {b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
          const int m = 4 * k + jj;
          if (m < HH) {
            const int l = l_of(m);
            v00[l] = fmaf(u0[jj], w0[jj], v00[l]);
            v01[l] = fmaf(u0[jj], w1[jj], v01[l]);
            v10[l] = fmaf(u1[jj], w0[jj], v10[l]);
            v11[l] = fmaf(u1[jj], w1[jj], v11[l]);
          }
        }
      }
      // (2a+1, 2b) is a pair only off the diagonal (n1 <= n2)
      auto put = [&](const float (&v)[LL], int n1, int n2) {
        const int q = q_of(n1, n2);
        float sq = 0.0f;
#pragma unroll
        for (int l = 0; l < LL; l++) {
          p_s[q * LL + l] = v[l];
          sq = fmaf(v[l], v[l], sq);
        }
        nacc.add(sq);
      };
      put(v00, 2 * ba, 2 * bb);
      put(v01, 2 * ba, 2 * bb + 1);
      if (bb != ba) put(v10, 2 * ba + 1, 2 * bb);
      put(v11, 2 * ba + 1, 2 * bb + 1);
    }
  } else if constexpr (SH::kL1 > 0 && sizeof(T) == 4) {
    // shape known, FP32: the lane's pairs q and q + 32 advance together with
    // paired multiply-adds; the c rows stream through 16-byte loads and each
    // entry m feeds the chain of its l, so every p value is the same chain of
    // fmaf as for one pair at a time
    constexpr int LL = SH::kL1, HH = LL * LL, H4 = (HH + 3) / 4;
    auto l_of = [](int m) { int l = 0; while ((l + 1) * (l + 1) <= m) l++; return l; };
    for (int q = lane; q < npair; q += 64) {
      const int qb = q + 32;
      const bool has_b = qb < npair;
      const int pa = pair_tab[q], pb = has_b ? pair_tab[qb] : pa;
      const float4 *xa = reinterpret_cast<const float4 *>(c_s + (pa & 0xffff) * HP);
      const float4 *ya = reinterpret_cast<const float4 *>(c_s + (pa >> 16) * HP);
      const float4 *xb = reinterpret_cast<const float4 *>(c_s + (pb & 0xffff) * HP);
      const float4 *yb = reinterpret_cast<const float4 *>(c_s + (pb >> 16) * HP);
      float2 v[LL];
#pragma unroll
      for (int l = 0; l < LL; l++) v[l] = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < H4; k++) {
        const float4 ua = xa[k], wa = ya[k], ub = xb[k], wb = yb[k];
        const float au[4] = {ua.x, ua.y, ua.z, ua.w}, aw[4] = {wa.x, wa.y, wa.z, wa.w};
        const float bu[4] = {ub.x, ub.y, ub.z, ub.w}, bw[4] = {wb.x, wb.y, wb.z, wb.w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int m = 4 * k + j;
          if (m < HH) {
            const int l = l_of(m);
            v[l] = ffma2(make_float2(au[j], bu[j]), make_float2(aw[j], bw[j]), v[l]);
          }
        }
      }
      float2 sq = make_float2(0.f, 0.f);
#pragma unroll
      for (int l = 0; l < LL; l++) {
        p_s[q * LL + l] = v[l].x;
        if (has_b) p_s[qb * LL + l] = v[l].y;
        sq = ffma2(v[l], v[l], sq);
      }
      nacc.add(sq.x);
      if (has_b) nacc.add(sq.y);
    }
  } else if constexpr (SH::kL1 > 0) {
    // shape known: both c rows in registers through 16-byte loads
    constexpr int LL = SH::kL1, HH = LL * LL, H4 = (HH + 3) / 4;
    for (int q = lane; q < npair; q += 32) {
      const int pr = pair_tab[q];
      const int n1 = pr & 0xffff, n2 = pr >> 16;
      T x[4 * H4], y[4 * H4];
#pragma unroll
      for (int k = 0; k < H4; k++) {
        if constexpr (sizeof(T) == 4) {
          const float4 u = reinterpret_cast<const float4 *>(c_s + n1 * HP)[k];
          const float4 w = reinterpret_cast<const float4 *>(c_s + n2 * HP)[k];
          x[4 * k + 0] = u.x;
          x[4 * k + 1] = u.y;
          x[4 * k + 2] = u.z;
          x[4 * k + 3] = u.w;
          y[4 * k + 0] = w.x;
          y[4 * k + 1] = w.y;
          y[4 * k + 2] = w.z;
          y[4 * k + 3] = w.w;
        } else {
#pragma unroll
          for (int j = 0; j < 4; j++) {
            x[4 * k + j] = c_s[n1 * HP + 4 * k + j];
            y[4 * k + j] = c_s[n2 * HP + 4 * k + j];
          }
        }
      }
      // p per l as a chain of multiply-adds; the pair's squared entries are
      // summed first and enter the compensated norm sum once per pair
      T sq = T(0);
#pragma unroll
      for (int l = 0; l < LL; l++) {
        T v = x[l * l] * y[l * l];
#pragma unroll
        for (int m = l * l + 1; m < (l + 1) * (l + 1); m++) v = fma_t(x[m], y[m], v);
        p_s[q * LL + l] = v;
        sq = fma_t(v, v, sq);
      }
      nacc.add(sq);
    }
  } else {
    for (int q = lane; q < npair; q += 32) {
      const int pr = pair_tab[q];
      const int n1 = pr & 0xffff, n2 = pr >> 16;
      const T *c1 = c_s + n1 * HP, *c2 = c_s + n2 * HP;
      for (int l = 0; l < L1; l++) {
        T v = T(0);
        for (int m = l * l; m < (l + 1) * (l + 1); m++) v += c1[m] * c2[m];
        p_s[q * L1 + l] = v;
        nacc.add(v * v);
      }
    }
  }
  double nrm = 0.0, inv = 0.0;
  float invf, nrm_hi = 0.0f, nrm_lo = 0.0f;
  if (sizeof(T) == 8) {
    const double nsq = warp_sum(double(nacc.s) + double(nacc.c));
    nrm = sqrt(nsq);
    inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
    invf = float(inv);
  } else {
    // |p|^2 as float-float; sqrt and 1/sqrt by one correction step of the
    // FP32 values (relative error ~1 ulp of FP32), no FP64 arithmetic
    float hi = float(nacc.s), lo = float(nacc.c);
    ff_warp_sum(hi, lo);
    const float r0 = sqrtf(hi);
    const float rc = r0 > 0.0f ? (fmaf(-r0, r0, hi) + lo) / (2.0f * r0) : 0.0f;
    const float y0 = r0 > 0.0f ? 1.0f / r0 : 0.0f;
    invf = fmaf(-y0 * y0, rc, y0);
    nrm_hi = r0;
    nrm_lo = rc;
  }
  if (lane == 0) {
    if (sizeof(T) == 4)  // FP32 kernels: |p| as a float-float pair in the 8-byte slot
      reinterpret_cast<float2 *>(norm_out)[atom] = make_float2(nrm_hi, nrm_lo);
    else
      norm_out[atom] = nrm;
  }
  __syncwarp();
  const int row = row_of_atom[atom];
  if (sizeof(T) == 4 && phat_hi && !p_out && !phat64 && (nd & 3) == 0) {
    // split operand only: four entries per lane, 16-byte reads, 8-byte writes
    const float4 *P4 = reinterpret_cast<const float4 *>(p_s);
    const float4 *B4 = reinterpret_cast<const float4 *>(pbar + (size_t)si * nd);
    uint2 *H4 = reinterpret_cast<uint2 *>(phat_hi + (size_t)row * ldp);
    uint2 *L4 = reinterpret_cast<uint2 *>(phat_lo + (size_t)row * ldp);
    for (int q = lane; q < (nd >> 2); q += 32) {
      const float4 v = P4[q], b = B4[q];
      const float2 x01 = make_float2((v.x * invf - b.x) * 8192.0f, (v.y * invf - b.y) * 8192.0f);
      const float2 x23 = make_float2((v.z * invf - b.z) * 8192.0f, (v.w * invf - b.w) * 8192.0f);
      // paired conversions (round to nearest); the residual of each entry
      // scaled by 2^11 is the lo plane
      const __half2 h01 = __float22half2_rn(x01), h23 = __float22half2_rn(x23);
      const float2 g01 = __half22float2(h01), g23 = __half22float2(h23);
      const __half2 r01 = __float22half2_rn(
          make_float2((x01.x - g01.x) * 2048.0f, (x01.y - g01.y) * 2048.0f));
      const __half2 r23 = __float22half2_rn(
          make_float2((x23.x - g23.x) * 2048.0f, (x23.y - g23.y) * 2048.0f));
      H4[q] = make_uint2(*reinterpret_cast<const unsigned *>(&h01),
                         *reinterpret_cast<const unsigned *>(&h23));
      L4[q] = make_uint2(*reinterpret_cast<const unsigned *>(&r01),
                         *reinterpret_cast<const unsigned *>(&r23));
    }
    return;
  }
  for (int d = lane; d < nd; d += 32) {
    const T v = p_s[d];
    if (p_out) p_out[(size_t)atom * nd + d] = v;
    if (phat64) phat64[(size_t)row * ldp + d] = double(v) * (sizeof(T) == 8 ? inv : double(invf));
    if (phat_hi) {
      // centred operand: delta = phat - pbar, scaled by 2^13 (|delta| <= 2)
      const float x = (float(v) * invf - pbar[(size_t)si * nd + d]) * 8192.0f;
      const __half h = __float2half_rn(x);
      const float rem = (x - __half2float(h)) * 2048.0f;
      phat_hi[(size_t)row * ldp + d] = h;
      phat_lo[(size_t)row * ldp + d] = __float2half_rn(rem);
    }
  }
}

// The mixed power-2 w = dE/dp and energy of one atom from its rows of V and of
// the split operand (global or shared memory): four consecutive entries per
// lane, 16-byte (8-byte for the fp16 planes) loads, |p| and E as float-float.
// Every entry is stored by the lane that read it, so store may overwrite V4
// in place.
template <typename T, typename Store>
__device__ __forceinline__ double w_mixed2(const AdjArgs &g, int si, int nd, float2 nrm32,
                                           const float4 *V4, const uint2 *H4,
                                           const uint2 *L4, Store store, int lane) {
  double e;
  const bool empty = nrm32.x * nrm32.x < g.empty_thresh_f;
  const int nq = nd >> 2;
  const float4 *G4 = reinterpret_cast<const float4 *>(g.gvec + (size_t)si * nd);
  const float4 *B4 = reinterpret_cast<const float4 *>(g.pbar + (size_t)si * nd);
  auto deltas = [&](uint2 h, uint2 l, float (&dl)[4]) {
    const float2 h01 = __half22float2(*reinterpret_cast<const __half2 *>(&h.x));
    const float2 h23 = __half22float2(*reinterpret_cast<const __half2 *>(&h.y));
    const float2 l01 = __half22float2(*reinterpret_cast<const __half2 *>(&l.x));
    const float2 l23 = __half22float2(*reinterpret_cast<const __half2 *>(&l.y));
    dl[0] = (h01.x + l01.x * (1.0f / 2048.0f)) * (1.0f / 8192.0f);
    dl[1] = (h01.y + l01.y * (1.0f / 2048.0f)) * (1.0f / 8192.0f);
    dl[2] = (h23.x + l23.x * (1.0f / 2048.0f)) * (1.0f / 8192.0f);
    dl[3] = (h23.y + l23.y * (1.0f / 2048.0f)) * (1.0f / 8192.0f);
  };
  // loads of kU iterations are issued before any of them is used (one atom's
  // rows are a few KB: the loop is latency-bound without this)
  constexpr int kU = 4;
  Acc<float> acc;
  for (int q0 = lane; q0 < nq; q0 += 32 * kU) {
    uint2 h[kU], l[kU];
    float4 v[kU], gg[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int q = q0 + 32 * u;
      if (q < nq) {
        h[u] = H4[q];
        l[u] = L4[q];
        v[u] = V4[q];
        gg[u] = G4[q];
      }
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      if (q0 + 32 * u < nq) {
        float dl[4];
        deltas(h[u], l[u], dl);
        acc.add((2.0f * gg[u].x + v[u].x) * dl[0]);
        acc.add((2.0f * gg[u].y + v[u].y) * dl[1]);
        acc.add((2.0f * gg[u].z + v[u].z) * dl[2]);
        acc.add((2.0f * gg[u].w + v[u].w) * dl[3]);
      }
    }
  }
  float hi = acc.s, lo = acc.c;
  ff_warp_sum(hi, lo);
  const ff et = ff_add(ff_norm(hi, lo), ff{g.c0_hi[si], g.c0_lo[si]});
  const float ef = empty ? 0.0f : et.hi + et.lo;
  const float inv = empty ? 0.0f : 1.0f / nrm32.x;
  e = empty ? 0.0 : double(et.hi) + double(et.lo);
  for (int q0 = lane; q0 < nq; q0 += 32 * kU) {
    uint2 h[kU], l[kU];
    float4 v[kU], gg[kU], pb[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int q = q0 + 32 * u;
      if (q < nq) {
        h[u] = H4[q];
        l[u] = L4[q];
        v[u] = V4[q];
        gg[u] = G4[q];
        pb[u] = B4[q];
      }
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int q = q0 + 32 * u;
      if (q < nq) {
        float dl[4];
        deltas(h[u], l[u], dl);
        store(4 * q + 0, T(2.0f * ((gg[u].x + v[u].x) - ef * (pb[u].x + dl[0])) * inv));
        store(4 * q + 1, T(2.0f * ((gg[u].y + v[u].y) - ef * (pb[u].y + dl[1])) * inv));
        store(4 * q + 2, T(2.0f * ((gg[u].z + v[u].z) - ef * (pb[u].z + dl[2])) * inv));
        store(4 * q + 3, T(2.0f * ((gg[u].w + v[u].w) - ef * (pb[u].w + dl[3])) * inv));
      }
    }
  }
  return e;
}

// w = dE/dp of one atom into w_s[nd] (all lanes), returning the atom energy:
// from the contraction V (mapped power 2), the beta vector (power 1), or
// given per operand row (kernel form).
template <typename T, typename Store>
__device__ __forceinline__ double adjoint_w(const B2Args &a, const AdjArgs &g, int si,
                                            int row, double nrm, float2 nrm32, Store store,
                                            int lane) {
  const int nd = a.n_d;
  double e = 0.0;
  if ((g.mode == kWFromV2 || g.mode == kWFromV1) && g.phat64) {
    const bool empty = nrm * nrm < g.empty_thresh;
    double dot = 0.0;
    for (int d = lane; d < nd; d += 32) {
      const double ph = g.phat64[(size_t)row * g.ldp + d];
      const double v = g.mode == kWFromV2 ? g.V64[(size_t)row * g.ldv + d]
                                          : g.beta1[(size_t)si * nd + d];
      dot += ph * v;
    }
    dot = warp_sum(dot);
    e = empty ? 0.0 : dot;
    const double inv = empty ? 0.0 : 1.0 / nrm;
    for (int d = lane; d < nd; d += 32) {
      const double ph = g.phat64[(size_t)row * g.ldp + d];
      if (g.mode == kWFromV2)
        store(d, T(2.0 * (g.V64[(size_t)row * g.ldv + d] - e * ph) * inv));
      else
        store(d, T((g.beta1[(size_t)si * nd + d] - e * ph) * inv));
    }
  } else if (g.mode == kWFromV2 && (nd & 3) == 0) {
    // the mixed power-2 form, rows read from global memory
    e = w_mixed2<T>(g, si, nd, nrm32,
                    reinterpret_cast<const float4 *>(g.V32 + (size_t)row * g.ldv),
                    reinterpret_cast<const uint2 *>(g.phat_hi + (size_t)row * g.ldp),
                    reinterpret_cast<const uint2 *>(g.phat_lo + (size_t)row * g.ldp), store,
                    lane);
  } else if (g.mode == kWFromV2 || g.mode == kWFromV1) {
    // mixed form on the centred operand delta = phat - pbar (float):
    //   power 2: E = c0 + sum_d (2 g_d + V_d) delta_d,  V = beta delta,
    //            g = beta pbar, c0 = pbar^T beta pbar;  dE/dp = 2 (g + V - E phat)/|p|
    //   power 1: E = phat . beta1,                      dE/dp = (beta1 - E phat)/|p|
    const bool empty = nrm32.x * nrm32.x < g.empty_thresh_f;
    Acc<float> acc;
    for (int d = lane; d < nd; d += 32) {
      const size_t o = (size_t)row * g.ldp + d;
      const float dl = (__half2float(g.phat_hi[o]) + __half2float(g.phat_lo[o]) * (1.0f / 2048.0f)) *
                       (1.0f / 8192.0f);
      if (g.mode == kWFromV2)
        acc.add((2.0f * g.gvec[(size_t)si * nd + d] + g.V32[(size_t)row * g.ldv + d]) * dl);
      else
        acc.add(float(g.beta1[(size_t)si * nd + d]) * (g.pbar[(size_t)si * nd + d] + dl));
    }
    float hi = acc.s, lo = acc.c;
    ff_warp_sum(hi, lo);
    const ff et = g.mode == kWFromV2 ? ff_add(ff_norm(hi, lo), ff{g.c0_hi[si], g.c0_lo[si]})
                                     : ff_norm(hi, lo);
    const float ef = empty ? 0.0f : et.hi + et.lo;
    const float inv = empty ? 0.0f : 1.0f / nrm32.x;
    e = empty ? 0.0 : double(et.hi) + double(et.lo);
    for (int d = lane; d < nd; d += 32) {
      const size_t o = (size_t)row * g.ldp + d;
      const float dl = (__half2float(g.phat_hi[o]) + __half2float(g.phat_lo[o]) * (1.0f / 2048.0f)) *
                       (1.0f / 8192.0f);
      const float ph = g.pbar[(size_t)si * nd + d] + dl;
      if (g.mode == kWFromV2)
        store(d, T(2.0f * ((g.gvec[(size_t)si * nd + d] + g.V32[(size_t)row * g.ldv + d]) -
                           ef * ph) * inv));
      else
        store(d, T((float(g.beta1[(size_t)si * nd + d]) - ef * ph) * inv));
    }
  } else {  // kWGiven: dE/dp supplied per operand row (kernel form)
    for (int d = lane; d < nd; d += 32) store(d, T(g.w_given[(size_t)row * g.ldp + d]));
    e = g.e_given ? g.e_given[row] : 0.0;
  }
  return e;
}

// u[n1, lm] = sum_n2 (W + W^T)[n1, n2, l] c[n2, lm] of one atom from its
// packed w (n1 <= n2, l fastest) and c rows in shared memory; lane owns lm.
template <typename T, typename SH>
__device__ __forceinline__ void b2_u_columns(const B2Args &a, const T *w_s, const T *c_s,
                                             T *u_row, int lane) {
  const int N = SH::N(a), LMAX = SH::lmax(a), H = (LMAX + 1) * (LMAX + 1), NS = SH::NS(a);
  const int nr = NS * N;
  const int L1 = LMAX + 1;
  for (int lm0 = 0; lm0 < H; lm0 += 32) {
    const int lm = lm0 + lane;
    if (lm >= H) continue;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) l++;
    if constexpr (SH::kNR > 0 && SH::kL1 > 0) {
      // shape known: the lane's c column in registers, every w index a constant
      // each packed w (n1 <= n2) is read once and feeds both u[n1] and u[n2]
      constexpr int NR = SH::kNR, LL = SH::kL1;
      T creg[NR], acc[NR];
#pragma unroll
      for (int n = 0; n < NR; n++) {
        creg[n] = c_s[n * H + lm];
        acc[n] = T(0);
      }
      const T *wl = w_s + l;
      auto wq = [&](int n1, int n2) {  // packed w of the pair n1 <= n2
        return wl[(n1 * NR - (n1 * (n1 - 1)) / 2 + (n2 - n1)) * LL];
      };
      if constexpr (sizeof(T) == 4 && (NR % 2) == 0) {
        // 2 x 2 blocks of (n1, n2) with paired multiply-adds: rows 2a, 2a+1
        // of u advance together
        float2 a2[NR / 2], c2[NR / 2];
#pragma unroll
        for (int a = 0; a < NR / 2; a++) {
          a2[a] = make_float2(0.f, 0.f);
          c2[a] = make_float2(creg[2 * a], creg[2 * a + 1]);
        }
#pragma unroll
        for (int a = 0; a < NR / 2; a++) {
          {  // diagonal block: (2a, 2a), (2a, 2a+1), (2a+1, 2a+1)
            const float w00 = wq(2 * a, 2 * a), w01 = wq(2 * a, 2 * a + 1);
            const float w11 = wq(2 * a + 1, 2 * a + 1);
            a2[a] = ffma2(make_float2(2.0f * w00, w01), make_float2(c2[a].x, c2[a].x), a2[a]);
            a2[a] = ffma2(make_float2(w01, 2.0f * w11), make_float2(c2[a].y, c2[a].y), a2[a]);
          }
#pragma unroll
          for (int b = a + 1; b < NR / 2; b++) {
            const float w00 = wq(2 * a, 2 * b), w01 = wq(2 * a, 2 * b + 1);
            const float w10 = wq(2 * a + 1, 2 * b), w11 = wq(2 * a + 1, 2 * b + 1);
            a2[a] = ffma2(make_float2(w00, w10), make_float2(c2[b].x, c2[b].x), a2[a]);
            a2[a] = ffma2(make_float2(w01, w11), make_float2(c2[b].y, c2[b].y), a2[a]);
            a2[b] = ffma2(make_float2(w00, w01), make_float2(c2[a].x, c2[a].x), a2[b]);
            a2[b] = ffma2(make_float2(w10, w11), make_float2(c2[a].y, c2[a].y), a2[b]);
          }
        }
#pragma unroll
        for (int a = 0; a < NR / 2; a++) {
          acc[2 * a] = a2[a].x;
          acc[2 * a + 1] = a2[a].y;
        }
      } else {
#pragma unroll
        for (int n1 = 0; n1 < NR; n1++)
#pragma unroll
          for (int n2 = n1; n2 < NR; n2++) {
            const T w = wq(n1, n2);
            if (n1 == n2) {
              acc[n1] += T(2) * w * creg[n1];
            } else {
              acc[n1] += w * creg[n2];
              acc[n2] += w * creg[n1];
            }
          }
      }
#pragma unroll
      for (int n1 = 0; n1 < NR; n1++) u_row[n1 * H + lm] = acc[n1];
    } else {
      for (int n1 = 0; n1 < nr; n1++) {
        T acc = T(0);
        // n2 < n1: pair (n2, n1), index q = n2 nr - n2 (n2 - 1)/2 + (n1 - n2)
        int q = n1;  // n2 = 0
        for (int n2 = 0; n2 < n1; n2++) {
          acc += w_s[q * L1 + l] * c_s[n2 * H + lm];
          q += nr - n2 - 1;
        }
        // n2 >= n1: pair (n1, n2)
        q = n1 * nr - (n1 * (n1 - 1)) / 2;
        acc += T(2) * w_s[q * L1 + l] * c_s[n1 * H + lm];
        for (int n2 = n1 + 1; n2 < nr; n2++)
          acc += w_s[(q + n2 - n1) * L1 + l] * c_s[n2 * H + lm];
        u_row[n1 * H + lm] = acc;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Adjoint, part 1 (one warp per atom): w = dE/dp and the atom energy, then
// u = dE/dc = (W + W^T) c per l, written to global memory.
// ---------------------------------------------------------------------------
template <typename T, typename SH>
__global__ void __launch_bounds__(128)
k_b2_wu(B2Args a, AdjArgs g, const int *__restrict__ species,
        const int *__restrict__ row_of_atom, const int *__restrict__ pair_tab,
        const T *__restrict__ c_in, const double *__restrict__ norm_in,
        double *__restrict__ atom_e, T *__restrict__ u_out) {
  (void)pair_tab;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int atom = blockIdx.x * nwarps + warp;
  const int N = SH::N(a), LMAX = SH::lmax(a), H = (LMAX + 1) * (LMAX + 1), NS = SH::NS(a);
  const int nd = a.n_d;
  const int sb = NS * N * H;
  unsigned char *base = smem_raw + a.smem_per_warp_adj * warp;
  T *w_s = reinterpret_cast<T *>(base);  // [nd]
  T *c_s = w_s + nd;                     // [sb]
  if (atom >= a.noa) return;
  const int si = species[atom];
  const int row = row_of_atom[atom];
  // FP32 kernels: the forward stored |p| as a float-float pair
  const double nrm = sizeof(T) == 8 ? norm_in[atom] : 0.0;
  const float2 nrm32 = sizeof(T) == 4 ? reinterpret_cast<const float2 *>(norm_in)[atom]
                                      : make_float2(0.0f, 0.0f);
#pragma unroll 4
  for (int k = lane; k < sb; k += 32) c_s[k] = c_in[(size_t)atom * sb + k];
  const double e =
      adjoint_w<T>(a, g, si, row, nrm, nrm32, [&](int d, T v) { w_s[d] = v; }, lane);
  if (lane == 0) atom_e[atom] = e;
  __syncwarp();
  b2_u_columns<T, SH>(a, w_s, c_s, u_out + (size_t)atom * sb, lane);
}

// Per-warp shared memory of the staged adjoint (byte offsets, 16-byte
// aligned): the atom's V row (overwritten in place by w), the hi and lo rows of
// its split operand (nd fp16 each, copied rounded up to 16 bytes), its c row,
// and the mbarrier the copies complete on.
struct WuStaged {
  uint32_t hi, lo, c, bar, total, hbytes;
};

__host__ __device__ inline WuStaged wu_staged_layout(int nd, int sb) {
  WuStaged L;
  L.hbytes = ((uint32_t)nd * 2u + 15u) & ~15u;
  L.hi = (uint32_t)nd * 4u;
  L.lo = L.hi + L.hbytes;
  L.c = L.lo + L.hbytes;
  L.bar = L.c + (uint32_t)sb * 4u;
  L.total = (L.bar + 8u + 15u) & ~15u;
  return L;
}

// The mixed power-2 adjoint, part 1, with the atom's rows staged: one lane
// starts bulk asynchronous copies of the V row, both split-operand rows and
// the c row (about 14 KB for n_d = 1500) into the warp's shared memory, all
// completing on one mbarrier, so every warp keeps its whole row in flight at
// once; then the same arithmetic as k_b2_wu from shared memory.  The wait is
// bounded: when it runs out the warp records FPP_ERR_TIMEOUT, waits (bounded)
// once more for its copies and returns without outputs.
template <typename SH>
__global__ void __launch_bounds__(128)
k_b2_wu_staged(B2Args a, AdjArgs g, const int *__restrict__ species,
               const int *__restrict__ row_of_atom, const float *__restrict__ c_in,
               const double *__restrict__ norm_in, double *__restrict__ atom_e,
               float *__restrict__ u_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int atom = blockIdx.x * (blockDim.x >> 5) + warp;
  if (atom >= a.noa) return;
  const int nd = a.n_d;
  const int sb = SH::kNR * SH::kL1 * SH::kL1;
  const WuStaged Ly = wu_staged_layout(nd, sb);
  unsigned char *base = smem_raw + (size_t)Ly.total * warp;
  float *v_s = reinterpret_cast<float *>(base);
  const uint32_t bar = smem_u32(base + Ly.bar);
  const int si = species[atom];
  const int row = row_of_atom[atom];
  if (lane == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_expect_tx(bar, (uint32_t)nd * 4u + 2u * Ly.hbytes + (uint32_t)sb * 4u);
    bulk_load(smem_u32(v_s), g.V32 + (size_t)row * g.ldv, (uint32_t)nd * 4u, bar);
    bulk_load(smem_u32(base + Ly.hi), g.phat_hi + (size_t)row * g.ldp, Ly.hbytes, bar);
    bulk_load(smem_u32(base + Ly.lo), g.phat_lo + (size_t)row * g.ldp, Ly.hbytes, bar);
    bulk_load(smem_u32(base + Ly.c), c_in + (size_t)atom * sb, (uint32_t)sb * 4u, bar);
  }
  __syncwarp();
  const float2 nrm32 = reinterpret_cast<const float2 *>(norm_in)[atom];
  bool ok = mbar_wait(bar, 0);
  ok = __all_sync(0xffffffffu, ok) != 0;
  if (!ok) {
    if (lane == 0) set_status(g.status, FPP_ERR_TIMEOUT, 221, atom);
    mbar_wait(bar, 0);
    return;
  }
  const double e = w_mixed2<float>(
      g, si, nd, nrm32, reinterpret_cast<const float4 *>(v_s),
      reinterpret_cast<const uint2 *>(base + Ly.hi), reinterpret_cast<const uint2 *>(base + Ly.lo),
      [&](int d, float v) { v_s[d] = v; }, lane);
  if (lane == 0) atom_e[atom] = e;
  __syncwarp();
  b2_u_columns<float, SH>(a, v_s, reinterpret_cast<const float *>(base + Ly.c),
                          u_out + (size_t)atom * sb, lane);
  if (lane == 0) mbar_inval(bar);
}

// ---------------------------------------------------------------------------
// B3 adjoint, part 1 (one warp per atom): w = dE/dp, then the holomorphic
// derivative u = dE/dc of the complex coefficients,
//   u[n1, l1m1] += w_q W c[n2,l2m2] c[n3,l3m3]   (and the two permutations),
// accumulated by each lane into its own column of shared memory (no atomics;
// the 32 columns are summed in a fixed order), and mapped back to dE/dc_real
// (the inverse of b3_to_complex's linear map), written to global memory.
// ---------------------------------------------------------------------------
template <typename T>
__host__ __device__ inline size_t b3_adjoint_smem_per_warp(const B2Args &a, bool fixed = false) {
  const size_t nr = (size_t)a.n_species * a.N;
  // fixed: the private rows of positions 2 and 3 (position 1 is in
  // registers); otherwise all three
  const size_t priv = (fixed ? 4 : 6) * (size_t)a.H * 32;
  size_t b;
  if (fixed) {
    // the private rows share memory with the w rows of the first round
    const size_t rows_a = (size_t)(a.n_tri < 32 ? a.n_tri : 32) * a.n_ls;
    const size_t rows_b = (size_t)(a.n_tri > 32 ? a.n_tri - 32 : 0) * a.n_ls;
    b = sizeof(T) * ((priv > rows_a ? priv : rows_a) + ((rows_b + 3) & ~(size_t)3) +
                     2 * nr * (a.H + 1) + 2 * nr * a.H);
  } else {
    // w (padded to 4 entries), complex c, summed u, and per-lane private rows
    // of the lane's triple (complex entries interleaved)
    b = sizeof(T) * ((size_t)((a.n_d + 3) & ~3) + 2 * nr * (a.H + 1) + 2 * nr * a.H + priv);
  }
  return (b + 15) & ~(size_t)15;
}

// LM >= 0: the adjoint's terms unrolled for lmax = LM (a.lmax must equal it)
template <typename T, int LM = -1>
__global__ void __launch_bounds__(128)
k_b3_wu(B2Args a, AdjArgs g, const int *__restrict__ species,
        const int *__restrict__ row_of_atom, const int *__restrict__ tri,
        const T *__restrict__ c_in, const double *__restrict__ norm_in,
        double *__restrict__ atom_e, T *__restrict__ u_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int atom = blockIdx.x * nwarps + warp;
  const int H = a.H, H1 = a.H + 1, nd = a.n_d;
  const int nr = a.n_species * a.N, sb = nr * H;
  unsigned char *base = smem_raw + a.smem_per_warp_adj * warp;
  T *w_s = reinterpret_cast<T *>(base);  // [nd] (fixed: rows of triples < 32)
  T *w_b = nullptr;                      // fixed: rows of triples >= 32
  V2<T> *z, *u2, *up;                    // [nr][H+1] complex c, [sb] summed u,
                                         // [3 H][32] private rows
  const int rows_a = a.n_tri < 32 ? a.n_tri : 32;
  if constexpr (LM >= 0) {
    const size_t priv = 4 * (size_t)H * 32, wa = (size_t)rows_a * a.n_ls;
    const size_t wbn = (size_t)(a.n_tri - rows_a) * a.n_ls;
    w_b = w_s + (priv > wa ? priv : wa);
    z = reinterpret_cast<V2<T> *>(w_b + ((wbn + 3) & ~(size_t)3));
    u2 = z + (size_t)nr * H1;
    up = reinterpret_cast<V2<T> *>(w_s);
  } else {
    z = reinterpret_cast<V2<T> *>(w_s + ((nd + 3) & ~3));
    u2 = z + (size_t)nr * H1;
    up = u2 + sb;
  }
  if (atom >= a.noa) return;
  const int si = species[atom];
  const int row = row_of_atom[atom];
  // FP32 kernels: the forward stored |p| as a float-float pair
  const double nrm = sizeof(T) == 8 ? norm_in[atom] : 0.0;
  const float2 nrm32 = sizeof(T) == 4 ? reinterpret_cast<const float2 *>(norm_in)[atom]
                                      : make_float2(0.0f, 0.0f);
  // real c staged through u2 (free until the accumulation below)
  T *cst = reinterpret_cast<T *>(u2);
  for (int k = lane; k < sb; k += 32) cst[k] = c_in[(size_t)atom * sb + k];
  const int split = rows_a * a.n_ls;
  const double e = adjoint_w<T>(
      a, g, si, row, nrm, nrm32,
      [&](int d, T v) {
        if (LM >= 0 && d >= split)
          w_b[d - split] = v;
        else
          w_s[d] = v;
      },
      lane);
  if (lane == 0) atom_e[atom] = e;
  __syncwarp();
  b3_to_complex2<T>(cst, nr, H, z, lane);
  __syncwarp();
  for (int k = lane; k < sb; k += 32) u2[k] = V2<T>{T(0), T(0)};
  __syncwarp();
  if constexpr (LM >= 0)
    b3_contract_adjoint_fixed<T, LM>(a.n_tri, H, nr, tri, z, w_s, w_b, up, u2, lane);
  else
    b3_contract_adjoint<T>(a.lmax, a.n_ls, a.n_tri, H, nr, tri, z, w_s, up, u2, lane);
  // dE/dc_real: for m > 0 with u+ = u[l, m], u- = u[l, -m], s = (-1)^m:
  //   dE/dR = (s Re u+ + Re u-) / sqrt 2,  dE/dS = (Im u- - s Im u+) / sqrt 2
  const T is2 = T(0.70710678118654752440);
  for (int k = lane; k < sb; k += 32) {
    const int n = k / H, lm = k - n * H;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) l++;
    const int m = lm - l * l - l;
    const int am = m < 0 ? -m : m;
    const int kp = n * H + l * l + l + am, km = n * H + l * l + l - am;
    const T sg = (am & 1) ? T(-1) : T(1);
    T v;
    if (m == 0)
      v = u2[k].x;
    else if (m > 0)
      v = (sg * u2[kp].x + u2[km].x) * is2;
    else
      v = (u2[km].y - sg * u2[kp].y) * is2;
    u_out[(size_t)atom * sb + k] = v;
  }
}

// Stored B3 derivatives (FP64) for a list of structure pairs, as b3.cpp:
// 206-240: rows 3*idx + comp of dB3_i / dr_ij and force_dots = dp . p_i.
// One warp per pair; lanes take radial triples.
__host__ __device__ inline size_t b3_dp_smem_per_warp(const B2Args &a) {
  const size_t nr = (size_t)a.n_species * a.N;
  return sizeof(double) * (2 * nr * (a.H + 1) + 3 * (size_t)a.N * a.H +
                           6 * (size_t)a.N * (a.H + 1) + nr * a.H + 2 * a.N + 4 * a.H);
}

__global__ void __launch_bounds__(128)
k_b3_dp(B2Args a, int npl, const int *__restrict__ plist, const int *__restrict__ nbr_i,
        const int *__restrict__ nbr_s, const dvec4 *__restrict__ rel,
        const int *__restrict__ tri, const double *__restrict__ c_in,
        const double *__restrict__ p_in, double *__restrict__ dp, int ldd,
        double *__restrict__ force_dots) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int idx = blockIdx.x * nwarps + warp;
  const int N = a.N, H = a.H, H1 = a.H + 1, nd = a.n_d;
  const int nr = a.n_species * N;
  double *base = reinterpret_cast<double *>(smem_raw) + (size_t)warp * (b3_dp_smem_per_warp(a) / 8);
  double *zr = base;                    // [nr][H+1] complex c of atom i
  double *zi = zr + (size_t)nr * H1;
  double *dcr = zi + (size_t)nr * H1;   // [3][N][H] real derivative (s_j block)
  double *dzr = dcr + 3 * N * H;        // [3][N][H+1] complex derivative
  double *dzi = dzr + 3 * N * H1;
  double *c_s = dzi + 3 * N * H1;       // [nr][H] real c
  double *gb = c_s + (size_t)nr * H;    // [N] g, [N] dg
  double *yb = gb + 2 * N;              // [H] Y, [3H] dY
  if (idx >= npl) return;
  const int p = plist[idx];
  const int i = nbr_i[p], sj = nbr_s[p];
  const dvec4 rd = rel[p];
  const double rcut = a.cutoffs[0];
  for (int k = lane; k < nr * H; k += 32) c_s[k] = c_in[(size_t)i * nr * H + k];
  if (lane == 0) {
    radial_basis<double>(rd.x, a.r1, rcut, N, a.cutoff_kind, gb, gb + N, 1);
    real_harmonics<double>(rd.y, rd.z, rd.w, a.lmax, yb, yb + H, 1);
  }
  __syncwarp();
  const double uv[3] = {rd.y / rd.x, rd.z / rd.x, rd.w / rd.x};
  for (int k = lane; k < 3 * N * H; k += 32) {
    const int comp = k / (N * H), rem = k - comp * N * H, n = rem / H, lm = rem - n * H;
    dcr[k] = gb[N + n] * uv[comp] * yb[lm] + gb[n] * yb[H + 3 * lm + comp];
  }
  __syncwarp();
  b3_to_complex<double>(c_s, nr, H, zr, zi, lane);
  for (int comp = 0; comp < 3; comp++)
    b3_to_complex<double>(dcr + comp * N * H, N, H, dzr + comp * N * H1,
                          dzi + comp * N * H1, lane);
  __syncwarp();
  const int *beg = c_b3.beg + c_b3.ls_off[a.lmax];
  const int n_ls = a.n_ls;
  double fdot[3] = {0, 0, 0};
  for (int t = 0; t < n_ls; t++) {
    const int e0 = beg[t], e1 = beg[t + 1];
    for (int r = lane; r < a.n_tri; r += 32) {
      const int tr = tri[r];
      const int n1 = tr & 0xff, n2 = (tr >> 8) & 0xff, n3 = tr >> 16;
      const bool in1 = n1 / N == sj, in2 = n2 / N == sj, in3 = n3 / N == sj;
      const int d1 = n1 % N, d2 = n2 % N, d3 = n3 % N;
      double v[3] = {0, 0, 0};
      for (int q = e0; q < e1; q++) {
        const unsigned ix = c_b3.idx[q];
        const int i1 = ix & 0xff, i2 = (ix >> 8) & 0xff, i3 = ix >> 16;
        const double w = c_b3.w[q];
        const double ar = zr[n1 * H1 + i1], ai = zi[n1 * H1 + i1];
        const double br = zr[n2 * H1 + i2], bi = zi[n2 * H1 + i2];
        const double cr = zr[n3 * H1 + i3], ci = zi[n3 * H1 + i3];
        for (int comp = 0; comp < 3; comp++) {
          const double *Dr = dzr + comp * N * H1, *Di = dzi + comp * N * H1;
          double acc = 0.0;
          if (in1) {  // Re(d1 b c)
            const double xr = Dr[d1 * H1 + i1] * br - Di[d1 * H1 + i1] * bi;
            const double xi = Dr[d1 * H1 + i1] * bi + Di[d1 * H1 + i1] * br;
            acc += xr * cr - xi * ci;
          }
          if (in2) {  // Re(a d2 c)
            const double xr = ar * Dr[d2 * H1 + i2] - ai * Di[d2 * H1 + i2];
            const double xi = ar * Di[d2 * H1 + i2] + ai * Dr[d2 * H1 + i2];
            acc += xr * cr - xi * ci;
          }
          if (in3) {  // Re(a b d3)
            const double xr = ar * br - ai * bi, xi = ar * bi + ai * br;
            acc += xr * Dr[d3 * H1 + i3] - xi * Di[d3 * H1 + i3];
          }
          v[comp] += w * acc;
        }
      }
      const int d = r * n_ls + t;
      const double pv = p_in[(size_t)i * nd + d];
      for (int comp = 0; comp < 3; comp++) {
        dp[(size_t)(3 * idx + comp) * ldd + d] = v[comp];
        fdot[comp] += v[comp] * pv;
      }
    }
  }
  for (int comp = 0; comp < 3; comp++) {
    const double v = warp_sum(fdot[comp]);
    if (lane == 0) force_dots[3 * idx + comp] = v;
  }
}

// ---------------------------------------------------------------------------
// Adjoint, part 2 (one thread per pair):
//   f_ij = sum_{n, lm} u_i[s_j N + n, lm] (g'_n Y_lm r_hat + g_n grad Y_lm)
// with g, g' in registers and the harmonics generated in order and consumed
// immediately.
// ---------------------------------------------------------------------------
template <typename T, typename SH>
__global__ void __launch_bounds__(128)
k_pair_force(B2Args a, int strict, long long n_pairs, const int *__restrict__ nbr_i,
             const dvec4 *__restrict__ rel, const float4 *__restrict__ rel32, const NbGeom *geom,
             const int *__restrict__ nbr_s, const int *__restrict__ species,
             const T *__restrict__ u, T *__restrict__ pair_f) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const int N = SH::N(a), LMAX = SH::lmax(a), H = (LMAX + 1) * (LMAX + 1), NS = SH::NS(a);
  const int sb = NS * N * H;
  const int i = nbr_i[p], sj = nbr_s[p], si = species[i];
  const int kc = si * NS + sj;
  T r, x, y, z, r1t, rct;
  bool keep;
  if (sizeof(T) == 8) {
    const dvec4 rd = rel[p];
    const double rcut = a.cutoffs[kc];
    keep = strict ? (rsq_exact(rd) < dmul(rcut, rcut)) : (rd.x <= rcut);
    r = T(rd.x);
    x = T(rd.y);
    y = T(rd.z);
    z = T(rd.w);
    r1t = T(a.r1);
    rct = T(rcut);
  } else {
    const float4 rf = rel32[p];
    x = T(rf.x);
    y = T(rf.y);
    z = T(rf.z);
    r = T(rf.w);
    if (strict)
      keep = strict_keep(rel, p, a.cutoffs[kc]);
    else
      keep = keep_pair32(a, kc, rf.w, rel, geom, i, p);
    r1t = T(a.r1f);
    rct = T(a.cutoffs32[kc]);
  }
  T f[3] = {T(0), T(0), T(0)};
  if (keep) {
    T gr[kMaxN], dg[kMaxN];
    radial_basis_reg<T>(r, r1t, rct, N, a.cutoff_kind, gr, dg,
                        sizeof(T) == 4 ? T(a.cinv_hi[kc]) : T(0),
                        sizeof(T) == 4 ? T(a.cinv_lo[kc]) : T(0));
    const T *ur = u + (size_t)i * sb + (size_t)sj * N * H;
    T fr = T(0);
    if constexpr (sizeof(T) == 4) {
      // paired FP32 multiply-adds: (ag, bd) and (f0, f1), (f2, fr) advance
      // together (each component is the same chain of fmaf as unpaired)
      float2 gd[kMaxN];
#pragma unroll
      for (int n = 0; n < kMaxN; n++) gd[n] = make_float2(gr[n], dg[n]);
      float2 f01 = make_float2(0.f, 0.f), f2r = make_float2(0.f, 0.f);
      harmonics_visit_f2(x, y, z, LMAX, [&](int lm, float Yv, float2 Yxy, float Yz) {
        float2 ab = make_float2(0.f, 0.f);
#pragma unroll
        for (int n = 0; n < kMaxN; n++)
          if (n < N) {
            const float uv = ur[n * H + lm];
            ab = ffma2(make_float2(uv, uv), gd[n], ab);
          }
        f01 = ffma2(make_float2(ab.x, ab.x), Yxy, f01);
        f2r = ffma2(ab, make_float2(Yz, Yv), f2r);
      });
      f[0] = f01.x;
      f[1] = f01.y;
      f[2] = f2r.x;
      fr = f2r.y;
    } else {
      harmonics_visit<T>(x, y, z, LMAX, [&](int lm, T Yv, T Yx, T Yy, T Yz) {
        T ag = T(0), bd = T(0);
#pragma unroll
        for (int n = 0; n < kMaxN; n++)
          if (n < N) {
            const T uv = ur[n * H + lm];
            ag += uv * gr[n];
            bd += uv * dg[n];
          }
        fr += bd * Yv;
        f[0] += ag * Yx;
        f[1] += ag * Yy;
        f[2] += ag * Yz;
      });
    }
    const T ir = T(1) / r;
    f[0] += fr * x * ir;
    f[1] += fr * y * ir;
    f[2] += fr * z * ir;
  }
  if (sizeof(T) == 4) {
    reinterpret_cast<float4 *>(pair_f)[p] =
        make_float4(float(f[0]), float(f[1]), float(f[2]), 0.0f);
  } else {
    pair_f[(size_t)p * 4 + 0] = f[0];
    pair_f[(size_t)p * 4 + 1] = f[1];
    pair_f[(size_t)p * 4 + 2] = f[2];
    pair_f[(size_t)p * 4 + 3] = T(0);
  }
}

// Stored derivatives of b2.cpp:181-242 for a list of structure pairs (FP64):
// rows 3*idx + comp of dp = d p_i / d r_ij and force_dots = dp . p_i.
// One warp per pair.
__global__ void __launch_bounds__(128)
k_b2_dp(B2Args a, int npl, const int *__restrict__ plist,
        const int *__restrict__ nbr_i, const int *__restrict__ nbr_s,
        const dvec4 *__restrict__ rel, const int *__restrict__ species,
        const int *__restrict__ pair_tab, const double *__restrict__ c_in,
        const double *__restrict__ p_in, double *__restrict__ dp, int ldd,
        double *__restrict__ force_dots) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int idx = blockIdx.x * nwarps + warp;
  const int N = a.N, H = a.H, NS = a.n_species, nd = a.n_d;
  const int sb = NS * N * H;
  double *base = reinterpret_cast<double *>(smem_raw) + (size_t)warp * (sb + 3 * N * H + 2 * N + 4 * H);
  double *c_s = base;                 // [sb]
  double *dc = c_s + sb;              // [3][N][H]
  double *gb = dc + 3 * N * H;        // [N] g, [N] dg
  double *yb = gb + 2 * N;            // [H] Y, [3H] dY
  if (idx >= npl) return;
  const int p = plist[idx];
  const int i = nbr_i[p], sj = nbr_s[p];
  const int si = species[i];
  const dvec4 rd = rel[p];
  const double rcut = a.cutoffs[si * NS + sj];
  for (int k = lane; k < sb; k += 32) c_s[k] = c_in[(size_t)i * sb + k];
  if (lane == 0) {
    radial_basis<double>(rd.x, a.r1, rcut, N, a.cutoff_kind, gb, gb + N, 1);
    real_harmonics<double>(rd.y, rd.z, rd.w, a.lmax, yb, yb + H, 1);
  }
  __syncwarp();
  const double u[3] = {rd.y / rd.x, rd.z / rd.x, rd.w / rd.x};
  for (int k = lane; k < 3 * N * H; k += 32) {
    const int comp = k / (N * H), rem = k - comp * N * H, n = rem / H, lm = rem - n * H;
    dc[k] = gb[N + n] * u[comp] * yb[lm] + gb[n] * yb[H + 3 * lm + comp];
  }
  __syncwarp();
  const int L1 = a.lmax + 1;
  double fdot[3] = {0, 0, 0};
  for (int d = lane; d < nd; d += 32) {
    const int q = d / L1, l = d - q * L1;
    const int pr = pair_tab[q];
    const int n1 = pr & 0xffff, n2 = pr >> 16;
    const bool in1 = (n1 / N) == sj, in2 = (n2 / N) == sj;
    const double pv = p_in[(size_t)i * nd + d];
    for (int comp = 0; comp < 3; comp++) {
      double v = 0.0;
      for (int m = 0; m < 2 * l + 1; m++) {
        const int lm = l * l + m;
        if (in2) v += c_s[n1 * H + lm] * dc[comp * N * H + (n2 % N) * H + lm];
        if (in1) v += dc[comp * N * H + (n1 % N) * H + lm] * c_s[n2 * H + lm];
      }
      dp[(size_t)(3 * idx + comp) * ldd + d] = v;
      fdot[comp] += v * pv;
    }
  }
  for (int comp = 0; comp < 3; comp++) {
    double v = warp_sum(fdot[comp]);
    if (lane == 0) force_dots[3 * idx + comp] = v;
  }
}

int launch_b2_dp(const B2Args &a, int npl, const int *plist, const int *nbr_i,
                 const int *nbr_s, const dvec4 *rel, const int *species,
                 const int *pair_tab, const double *c_in, const double *p_in,
                 double *dp, int ldd, double *force_dots, cudaStream_t stream) {
  if (npl == 0) return 0;
  if (a.kind == kB3) {
    const size_t per3 = b3_dp_smem_per_warp(a);
    int w3 = 4;
    while (w3 > 1 && per3 * w3 > 200 * 1024) w3 >>= 1;
    const size_t sm3 = per3 * w3;
    if (sm3 > 227 * 1024) return -1;
    if (cudaFuncSetAttribute(k_b3_dp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm3) != cudaSuccess)
      return -1;
    k_b3_dp<<<ceil_div(npl, w3), 32 * w3, sm3, stream>>>(a, npl, plist, nbr_i, nbr_s, rel,
                                                         pair_tab, c_in, p_in, dp, ldd,
                                                         force_dots);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  }
  const int sb = a.n_species * a.N * a.H;
  size_t per = sizeof(double) * (sb + 3 * a.N * a.H + 2 * a.N + 4 * a.H);
  int wpb = 4;
  while (wpb > 1 && per * wpb > 200 * 1024) wpb >>= 1;
  size_t smem = per * wpb;
  if (smem > 227 * 1024) return -1;
  if (cudaFuncSetAttribute(k_b2_dp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  k_b2_dp<<<ceil_div(npl, wpb), 32 * wpb, smem, stream>>>(
      a, npl, plist, nbr_i, nbr_s, rel, species, pair_tab, c_in, p_in, dp, ldd,
      force_dots);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// FP32 pair forces, one warp per atom: lanes take the atom's pairs (f_ij
// coalesced, f_ji gathered through the reverse index), the warp sums the force
// and the virial f_ij (x) r_ij as float-float.  Warps walk atoms with a grid
// stride and keep their atoms' energy and virial as float-float sums; each
// block writes one partial row for k_reduce (fixed order: deterministic).
constexpr int kGatherWarps = 8;

// Float-float sum over the kGatherLanes lanes of a group (xor offsets stay
// inside the group), every lane of the group ends with the total.
constexpr int kGatherLanes = 4;  // lanes per atom (eight atoms per warp)
__device__ __forceinline__ void ff_group_sum(float &hi, float &lo) {
#pragma unroll
  for (int o = kGatherLanes / 2; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    float s, e;
    two_sum(hi, h2, s, e);
    e += lo + l2;
    hi = s + e;
    lo = e - (hi - s);
  }
}

// four resident blocks per SM (64 registers): the kernel waits on its
// dependent loads, and 32 warps hide more of that than 24
__global__ void __launch_bounds__(32 * kGatherWarps, 4)
k_gather_warp(int noa, const int *__restrict__ offset, const int *__restrict__ rev,
              const float4 *__restrict__ rel32, const float4 *__restrict__ pair_f,
              const double *__restrict__ atom_e, double *__restrict__ forces,
              double *__restrict__ partial) {
  __shared__ double sm_e[kGatherWarps];
  __shared__ float2 sm_v[kGatherWarps][9];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / kGatherLanes, gl = lane % kGatherLanes;  // group, lane in group
  constexpr int kGroups = 32 / kGatherLanes;
  float th[9], tl[9];  // this lane's share of the virial, float-float
#pragma unroll
  for (int k = 0; k < 9; k++) th[k] = tl[k] = 0.0f;
  double esum = 0.0;  // group leaders: their atoms' energies
  // atoms in rounds of kGroups per warp; all lanes run the same number of
  // rounds (the group shuffles need the whole warp)
  const int stride = gridDim.x * kGatherWarps * kGroups;
  for (int i0 = (blockIdx.x * kGatherWarps + warp) * kGroups; i0 < noa; i0 += stride) {
    const int i = i0 + g;
    const bool live = i < noa;
    float hi[12], lo[12];
#pragma unroll
    for (int k = 0; k < 12; k++) hi[k] = lo[k] = 0.0f;
    const int beg = live ? offset[i] : 0, end = live ? offset[i + 1] : 0;
    for (int p = beg + gl; p < end; p += kGatherLanes) {
      const int q = rev[p];
      const float4 fp = pair_f[p];
      const float4 fq = q >= 0 ? pair_f[q] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 r = rel32[p];
      const float f[3] = {fp.x, fp.y, fp.z}, gq[3] = {fq.x, fq.y, fq.z};
      const float rr[3] = {r.x, r.y, r.z};
#pragma unroll
      for (int a = 0; a < 3; a++) {
        float t, e;
        two_sum(hi[a], f[a], t, e);
        lo[a] += e;
        two_sum(t, -gq[a], hi[a], e);
        lo[a] += e;
#pragma unroll
        for (int b = 0; b < 3; b++) {
          const int k = 3 + 3 * a + b;
          two_sum(hi[k], f[a] * rr[b], t, e);
          hi[k] = t;
          lo[k] += e;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 12; k++) ff_group_sum(hi[k], lo[k]);
    if (live) {
      // lanes 0..2 of the group convert one force component each
      const float fh = gl == 0 ? hi[0] : (gl == 1 ? hi[1] : hi[2]);
      const float fl = gl == 0 ? lo[0] : (gl == 1 ? lo[1] : lo[2]);
      if (gl < 3) forces[3 * i + gl] = double(fh) + double(fl);
      if (gl == 0) esum += atom_e[i];
      if (gl == 0) {
#pragma unroll
        for (int k = 0; k < 9; k++) {
          float t, e;
          two_sum(th[k], hi[3 + k], t, e);
          th[k] = t;
          tl[k] += e + lo[3 + k];
        }
      }
    }
  }
  // the group leaders' virial (other lanes hold zeros) and energies, summed
  // over the warp and then the block in a fixed order; the virial stays
  // float-float until one conversion per block (FP64 instructions are scarce)
#pragma unroll
  for (int k = 0; k < 9; k++) ff_warp_sum(th[k], tl[k]);
  esum = warp_sum(esum);
  if (lane == 0) {
    sm_e[warp] = esum;
#pragma unroll
    for (int k = 0; k < 9; k++) sm_v[warp][k] = make_float2(th[k], tl[k]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kGatherWarps; w++) v += sm_e[w];
    partial[(size_t)blockIdx.x * 10] = v;
  } else if (threadIdx.x < 10) {
    const int k = threadIdx.x - 1;
    ff t = ff{sm_v[0][k].x, sm_v[0][k].y};
#pragma unroll
    for (int w = 1; w < kGatherWarps; w++) t = ff_add(t, ff{sm_v[w][k].x, sm_v[w][k].y});
    partial[(size_t)blockIdx.x * 10 + threadIdx.x] = double(t.hi) + double(t.lo);
  }
}

// ---------------------------------------------------------------------------
// Kuf of a batch of training structures by the adjoint route (FP64), the
// envs_struc columns of normalized_dot_product.cpp:115-210 without the stored
// descriptor derivatives.  One persistent launch: each block takes work items
// (structure, atom i) and, for the sparse environments k of the atom's
// species in passes of KS:
//   z_k = dhat_k . phat_i, the energy column += sig^2 z_k^power;
//   w_k = dk/dp_i = sig^2 power z_k^(power-1) (dhat_k - z_k phat_i) / |p_i|;
//   u_k = dk/dc_i through the B2 contraction (u[n1,lm] = sum_n2 (W+W^T) c);
//   per pair (i, j) the bases g, dg, Y, dY are recomputed once and
//   f = dk/dr_ij = u_k . dc_i/dr_ij goes to the columns of the labels:
//   F_i += f, F_j -= f, stress(a <= b) -= f_a r_b / V.
// Contributions to other atoms' columns are FP64 atomic adds (the order of
// those additions varies between runs, at the level of FP64 rounding).
// ---------------------------------------------------------------------------
struct KufLayout {
  size_t ph, c, w, u, zz, aa, acc, pg, py, prel, prh, ints, total;
};

__host__ __device__ inline KufLayout kuf_layout(const B2Args &a, int ks) {
  const size_t nd = a.n_d, sb = (size_t)a.n_species * a.N * a.H;
  KufLayout L;
  size_t o = 0;
  L.ph = o; o += nd;
  L.c = o; o += sb;
  L.w = o; o += (size_t)ks * nd;
  L.u = o; o += (size_t)ks * sb;
  L.zz = o; o += ks;
  L.aa = o; o += ks;
  L.acc = o; o += (size_t)ks * 9;
  L.pg = o; o += 32 * 2 * (size_t)a.N;
  L.py = o; o += 32 * 4 * (size_t)a.H;
  L.prel = o; o += 32 * 4;
  L.prh = o; o += 32 * 3;                    // unit vectors r / |r| of the window
  L.ints = o; o += (3 * 32 + 1) / 2 + 1;   // pj, psj, pkeep as ints
  L.total = o * sizeof(double);
  return L;
}

__device__ __forceinline__ double kuf_pow(double z, double p) {
  if (p == 2.0) return z * z;
  if (p == 1.0) return z;
  return pow(z, p);
}

__global__ void __launch_bounds__(256)
k_kuf_adjoint(const KufArgs k, int ks, int n_items, int item0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *sm = reinterpret_cast<double *>(smem_raw);
  const B2Args &a = k.a;
  const KufLayout L = kuf_layout(a, ks);
  double *ph = sm + L.ph, *c = sm + L.c, *w = sm + L.w, *u = sm + L.u;
  double *zz = sm + L.zz, *aa = sm + L.aa, *acc = sm + L.acc;
  double *pg = sm + L.pg, *py = sm + L.py, *prel = sm + L.prel, *prh = sm + L.prh;
  int *pj = reinterpret_cast<int *>(sm + L.ints), *psj = pj + 32, *pkeep = psj + 32;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarp = nth >> 5;
  const int N = a.N, H = a.H, NS = a.n_species, nd = a.n_d, L1 = a.lmax + 1;
  const int nr = NS * N, sb = nr * H;
  for (int it = item0 + blockIdx.x; it < item0 + n_items; it += gridDim.x) {
    const int2 item = k.items[it];
    const KufStruc S = k.strucs[item.x];
    const int i = item.y;
    const int si = S.species[i];
    const double nrm = S.norm64[i];
    if (nrm < 1e-8) continue;  // empty environment: no energy, no forces
    const KufSpecies SP = k.sp[si];
    if (SP.n_sparse == 0) continue;
    const int row = S.row_of_atom[i];
    __syncthreads();  // the previous item's shared memory is free
    for (int d = tid; d < nd; d += nth) ph[d] = S.phat64[(size_t)row * k.ldp + d];
    for (int q = tid; q < sb; q += nth) c[q] = S.c64[(size_t)i * sb + q];
    const int beg = S.offset[i], end = S.offset[i + 1];
    const int col_i = S.force_col[i];
    __syncthreads();
    for (int k0 = 0; k0 < SP.n_sparse; k0 += ks) {
      const int kc = min(ks, SP.n_sparse - k0);
      // z_k = dhat_k . phat_i (a warp per k)
      for (int kk = warp; kk < kc; kk += nwarp) {
        const double *dk = SP.dhat + (size_t)(k0 + kk) * nd;
        double v = 0.0;
        for (int d = lane; d < nd; d += 32) v = fma(dk[d], ph[d], v);
        v = warp_sum(v);
        if (lane == 0) zz[kk] = v;
      }
      __syncthreads();
      for (int kk = tid; kk < kc; kk += nth) {
        const bool live = SP.norms[k0 + kk] >= 1e-8;
        const double z = zz[kk];
        if (live && S.col_e >= 0)
          atomicAdd(k.kuf + (size_t)(SP.row0 + k0 + kk) * k.n_labels + S.col_e,
                    k.sig2 * kuf_pow(z, k.power));
        aa[kk] = live ? k.sig2 * k.power * kuf_pow(z, k.power - 1.0) / nrm : 0.0;
        for (int q = 0; q < 9; q++) acc[kk * 9 + q] = 0.0;
      }
      __syncthreads();
      // w_k = a_k (dhat_k - z_k phat_i)
      for (int idx = tid; idx < kc * nd; idx += nth) {
        const int kk = idx / nd, d = idx - kk * nd;
        w[idx] = aa[kk] * (SP.dhat[(size_t)(k0 + kk) * nd + d] - zz[kk] * ph[d]);
      }
      __syncthreads();
      // u_k[n1, lm] = sum_n2 w_k[(n1, n2), l] c[n2, lm] (the diagonal twice)
      for (int idx = tid; idx < kc * sb; idx += nth) {
        const int kk = idx / sb, rem = idx - kk * sb;
        const int n1 = rem / H, lm = rem - n1 * H;
        int l = 0;
        while ((l + 1) * (l + 1) <= lm) l++;
        const double *wk = w + (size_t)kk * nd;
        double v = 0.0;
        for (int n2 = 0; n2 < nr; n2++) {
          const int lo = n1 < n2 ? n1 : n2, hi = n1 < n2 ? n2 : n1;
          const int q = lo * nr - lo * (lo - 1) / 2 + (hi - lo);
          const double f = n1 == n2 ? 2.0 : 1.0;
          v = fma(f * wk[q * L1 + l], c[n2 * H + lm], v);
        }
        u[idx] = v;
      }
      __syncthreads();
      for (int w0 = beg; w0 < end; w0 += 32) {
        const int np = min(32, end - w0);
        // stage the bases of up to 32 pairs (a thread per pair)
        if (tid < np) {
          const int p = w0 + tid;
          const dvec4 rd = S.rel[p];
          const int sj = S.nbr_s[p];
          const double rcut = a.cutoffs[si * NS + sj];
          const bool keep = rd.x <= rcut;  // the B2 filter (b2.cpp:277)
          pj[tid] = S.nbr_j[p];
          psj[tid] = sj;
          pkeep[tid] = keep ? 1 : 0;
          prel[4 * tid + 0] = rd.x;
          prel[4 * tid + 1] = rd.y;
          prel[4 * tid + 2] = rd.z;
          prel[4 * tid + 3] = rd.w;
          // the unit vector once per pair (FP64 divisions are costly here)
          const double ir = keep ? 1.0 / rd.x : 0.0;
          prh[3 * tid + 0] = rd.y * ir;
          prh[3 * tid + 1] = rd.z * ir;
          prh[3 * tid + 2] = rd.w * ir;
          // bases lane-fastest (stride 32): the warp's lanes read one
          // coefficient of 32 different pairs from 32 consecutive doubles,
          // free of shared-memory bank conflicts
          if (keep) {
            radial_basis<double>(rd.x, a.r1, rcut, N, a.cutoff_kind, pg + tid,
                                 pg + 32 * N + tid, 32);
            real_harmonics<double>(rd.y, rd.z, rd.w, a.lmax, py + tid, py + 32 * H + tid, 32);
          }
        }
        __syncthreads();
        // f for (sparse k, pair): a warp per k, a lane per pair
        for (int kk = warp; kk < kc; kk += nwarp) {
          double f[3] = {0.0, 0.0, 0.0};
          if (lane < np && pkeep[lane]) {
            const double *g = pg + lane, *dg = pg + 32 * N + lane;      // stride 32
            const double *Y = py + lane, *dY = py + 32 * H + lane;      // stride 32
            const double *ur = u + (size_t)kk * sb + (size_t)psj[lane] * N * H;
            double fr = 0.0;
            for (int lm = 0; lm < H; lm++) {
              double A = 0.0, B = 0.0;
              for (int n = 0; n < N; n++) {
                const double uv = ur[n * H + lm];
                A = fma(uv, g[32 * n], A);
                B = fma(uv, dg[32 * n], B);
              }
              fr = fma(B, Y[32 * lm], fr);
              f[0] = fma(A, dY[32 * (3 * lm + 0)], f[0]);
              f[1] = fma(A, dY[32 * (3 * lm + 1)], f[1]);
              f[2] = fma(A, dY[32 * (3 * lm + 2)], f[2]);
            }
            f[0] = fma(fr, prh[3 * lane + 0], f[0]);
            f[1] = fma(fr, prh[3 * lane + 1], f[1]);
            f[2] = fma(fr, prh[3 * lane + 2], f[2]);
            const int cj = S.force_col[pj[lane]];
            double *krow = k.kuf + (size_t)(SP.row0 + k0 + kk) * k.n_labels;
            if (cj >= 0) {
              atomicAdd(krow + cj + 0, -f[0]);
              atomicAdd(krow + cj + 1, -f[1]);
              atomicAdd(krow + cj + 2, -f[2]);
            }
          }
          // own force column and the stress, summed over the warp's pairs
          const double rx = lane < np ? prel[4 * lane + 1] : 0.0;
          const double ry = lane < np ? prel[4 * lane + 2] : 0.0;
          const double rz = lane < np ? prel[4 * lane + 3] : 0.0;
          double t[9] = {f[0], f[1], f[2], f[0] * rx, f[0] * ry, f[0] * rz,
                         f[1] * ry, f[1] * rz, f[2] * rz};
#pragma unroll
          for (int q = 0; q < 9; q++) t[q] = warp_sum(t[q]);
          if (lane == 0)
            for (int q = 0; q < 9; q++) acc[kk * 9 + q] += t[q];
        }
        __syncthreads();
      }
      // the atom's own force column and the stress columns
      for (int kk = tid; kk < kc; kk += nth) {
        double *krow = k.kuf + (size_t)(SP.row0 + k0 + kk) * k.n_labels;
        if (col_i >= 0)
          for (int q = 0; q < 3; q++) atomicAdd(krow + col_i + q, acc[kk * 9 + q]);
        if (S.col_s >= 0)
          for (int q = 0; q < 6; q++)
            atomicAdd(krow + S.col_s + q, -acc[kk * 9 + 3 + q] * S.vol_inv);
      }
      __syncthreads();
    }
  }
}

size_t kuf_adjoint_smem(const B2Args &a, int ks, int threads) {
  if (threads < 64 || threads > 256 || (threads & 31)) return 0;
  const size_t b = kuf_layout(a, ks).total;
  return b <= 227 * 1024 ? b : 0;
}

int launch_kuf_adjoint(const KufArgs &k, int ks, int threads, int n_items, int item0,
                       cudaStream_t stream) {
  if (n_items <= 0) return 0;
  const size_t smem = kuf_adjoint_smem(k.a, ks, threads);
  if (smem == 0) return -1;
  if (cudaFuncSetAttribute(k_kuf_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_kuf_adjoint, threads, smem) !=
          cudaSuccess)
    return -1;
  const int grid = std::min(n_items, sms * std::max(per_sm, 1));
  k_kuf_adjoint<<<grid, threads, smem, stream>>>(k, ks, n_items, item0);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// F_i = sum over pairs of i (f_ij - f_ji); each block also reduces its atoms'
// energies and virials (sum f_ij (x) r_ij) into one partial row (fixed tree
// order, so the result is deterministic).  128 threads per block.
template <typename T>
__global__ void __launch_bounds__(128)
k_gather(int noa, const int *__restrict__ offset, const int *__restrict__ rev,
         const float4 *__restrict__ rel32, const dvec4 *__restrict__ rel,
         const T *__restrict__ pair_f, const double *__restrict__ atom_e,
         double *__restrict__ forces, double *__restrict__ partial) {
  __shared__ double sm[10][128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (sizeof(T) == 4 && i < noa) {
    // FP32 pair forces: per-atom sums kept as float-float (exact to ~2^-48)
    // and the virial compensated, so no FP64 instruction runs per pair
    float Fh[3] = {0, 0, 0}, Fl[3] = {0, 0, 0};
    float Vs[9], Vc[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Vs[k] = Vc[k] = 0.0f;
    for (int p = offset[i]; p < offset[i + 1]; p++) {
      const int q = rev[p];
      const float4 fp = reinterpret_cast<const float4 *>(pair_f)[p];
      const float4 fq = q >= 0 ? reinterpret_cast<const float4 *>(pair_f)[q]
                               : make_float4(0.f, 0.f, 0.f, 0.f);
      const float fv[3] = {fp.x, fp.y, fp.z}, gv[3] = {fq.x, fq.y, fq.z};
#pragma unroll
      for (int a = 0; a < 3; a++) {
        float s, e;
        two_sum(Fh[a], fv[a], s, e);
        Fl[a] += e;
        two_sum(s, -gv[a], Fh[a], e);
        Fl[a] += e;
      }
      const float4 r = rel32[p];
      const float rr[3] = {r.x, r.y, r.z};
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
          const int k = a * 3 + b;
          const float x = fv[a] * rr[b];
          const float t = Vs[k] + x;
          Vc[k] += fabsf(Vs[k]) >= fabsf(x) ? (Vs[k] - t) + x : (x - t) + Vs[k];
          Vs[k] = t;
        }
    }
#pragma unroll
    for (int a = 0; a < 3; a++) forces[3 * i + a] = double(Fh[a]) + double(Fl[a]);
#pragma unroll
    for (int k = 0; k < 9; k++) acc[1 + k] = double(Vs[k]) + double(Vc[k]);
    acc[0] = atom_e[i];
  } else if (i < noa) {
    double F[3] = {0, 0, 0};
    for (int p = offset[i]; p < offset[i + 1]; p++) {
      const int q = rev[p];
      const double f0 = double(pair_f[(size_t)p * 4 + 0]);
      const double f1 = double(pair_f[(size_t)p * 4 + 1]);
      const double f2 = double(pair_f[(size_t)p * 4 + 2]);
      F[0] += f0;
      F[1] += f1;
      F[2] += f2;
      if (q >= 0) {  // always present for a periodic list; -1 is reported upstream
        F[0] -= double(pair_f[(size_t)q * 4 + 0]);
        F[1] -= double(pair_f[(size_t)q * 4 + 1]);
        F[2] -= double(pair_f[(size_t)q * 4 + 2]);
      }
      double rr[3];
      if (sizeof(T) == 8) {
        const dvec4 r = rel[p];
        rr[0] = r.y;
        rr[1] = r.z;
        rr[2] = r.w;
      } else {
        const float4 r = rel32[p];
        rr[0] = r.x;
        rr[1] = r.y;
        rr[2] = r.z;
      }
      const double ff[3] = {f0, f1, f2};
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) acc[1 + a * 3 + b] += ff[a] * rr[b];
    }
    forces[3 * i + 0] = F[0];
    forces[3 * i + 1] = F[1];
    forces[3 * i + 2] = F[2];
    acc[0] = atom_e[i];
  }
#pragma unroll
  for (int k = 0; k < 10; k++) sm[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int st = 64; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
#pragma unroll
      for (int k = 0; k < 10; k++) sm[k][threadIdx.x] += sm[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 10) partial[(size_t)blockIdx.x * 10 + threadIdx.x] = sm[threadIdx.x][0];
}

// Sum of the per-block partial rows: out[0] = E, out[1..9] = sum f (x) r.
// Block k sums column k (ten blocks on ten SMs: FP64 adds are scarce on one
// SM): strided per-thread sums, then a fixed shared-memory tree.
__global__ void __launch_bounds__(128)
k_reduce(int nblocks, const double *__restrict__ partial, double *__restrict__ out) {
  __shared__ double sm[128];
  const int k = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partial[(size_t)b * 10 + k];
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int st = 64; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) sm[threadIdx.x] += sm[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[k] = sm[0];
}

// ---------------------------------------------------------------------------
// Host launchers.
// ---------------------------------------------------------------------------
size_t forward_smem_per_warp(const B2Args &a, size_t elem) {
  return elem == sizeof(float) ? fwd_layout<float>(a).total : fwd_layout<double>(a).total;
}

size_t adjoint_smem_per_warp(const B2Args &a, size_t elem) {
  const int sb = a.n_species * a.N * a.H;
  size_t b = elem * ((size_t)a.n_d + (size_t)sb);
  return (b + 15) & ~(size_t)15;
}

// Warps per block (4, 2 or 1) for a warp-per-atom kernel with `per` bytes of
// shared memory per warp: the most resident warps per SM (228 KB of shared
// memory per SM, 1 KB reserved per block, at most 32 blocks), ties to the
// larger block.  0 if one warp does not fit in a block.
static int warps_per_block(size_t per) {
  int best = 0, best_warps = 0;
  for (int wpb = 4; wpb >= 1; wpb >>= 1) {
    const size_t blk = per * wpb;
    if (blk > 227 * 1024) continue;
    int blocks = (int)((228 * 1024) / (blk + 1024));
    if (blocks > 32) blocks = 32;
    if (blocks * wpb > best_warps) {
      best_warps = blocks * wpb;
      best = wpb;
    }
  }
  return best;
}

template <typename T>
int launch_b2_forward(B2Args a, const Neigh &nb, const int *species,
                      const int *row_of_atom, const int *pair_tab, T *c_out,
                      T *p_out, double *norm_out, double *phat64, __half *phat_hi,
                      __half *phat_lo, int ldp, const float *pbar, cudaStream_t stream) {
  if (a.noa == 0) return 0;
  a.window = 32;
  const size_t per = fwd_layout<T>(a).total;
  const int wpb = warps_per_block(per);
  if (wpb == 0) return -1;
  size_t smem = per * wpb;
  return with_shape<T>(a, [&](auto sh) {
    auto kern = k_b2_forward<T, decltype(sh)>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return -1;
    kern<<<ceil_div(a.noa, wpb), 32 * wpb, smem, stream>>>(
        a, nb.offset, nb.rel, nb.rel32, nb.geom, nb.nbr_s, species, row_of_atom, pair_tab,
        c_out, p_out, norm_out, phat64, phat_hi, phat_lo, ldp, pbar);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  });
}

template <typename T>
int launch_b2_adjoint(B2Args a, const AdjArgs &g, const Neigh &nb,
                      const int *species, const int *row_of_atom,
                      const int *pair_tab, const T *c_in, const double *norm_in,
                      double *atom_e, T *pair_f, double *forces, double *atom_vir,
                      double *reduce_out, bool gather, T *u_buf, long long n_pairs,
                      const int *nbr_i, cudaStream_t stream) {
  if (a.noa == 0) return 0;
  // FP32 at lmax 3 (the B3 workload shape): the unrolled adjoint
  const bool b3_fixed = a.kind == kB3 && sizeof(T) == 4 && a.lmax == 3;
  a.smem_per_warp_adj = a.kind == kB3 ? b3_adjoint_smem_per_warp<T>(a, b3_fixed)
                                      : adjoint_smem_per_warp(a, sizeof(T));
  const int wpb = warps_per_block(a.smem_per_warp_adj);
  if (wpb == 0) return -1;
  size_t smem = a.smem_per_warp_adj * wpb;
  if (a.kind == kB3) {
    auto kern3 = k_b3_wu<T, -1>;
    if constexpr (sizeof(T) == 4)
      if (b3_fixed) kern3 = k_b3_wu<T, 3>;
    if (cudaFuncSetAttribute(kern3, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return -1;
    kern3<<<ceil_div(a.noa, wpb), 32 * wpb, smem, stream>>>(a, g, species, row_of_atom,
                                                            pair_tab, c_in, norm_in, atom_e,
                                                            u_buf);
  } else {
    const int rc = with_shape<T>(a, [&](auto sh) {
      using SH = decltype(sh);
      if constexpr (sizeof(T) == 4 && SH::kNR > 0 && SH::kL1 > 0) {
        // the mixed power-2 form with every row a whole number of 16-byte
        // units at 16-byte aligned addresses: the staged kernel
        const int sb = SH::kNR * SH::kL1 * SH::kL1;
        auto al16 = [](const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
        if (g.mode == kWFromV2 && !g.phat64 && g.V32 && g.phat_hi && g.phat_lo &&
            (a.n_d & 3) == 0 && (g.ldv & 3) == 0 && (g.ldp & 7) == 0 &&
            2 * g.ldp >= (int)wu_staged_layout(a.n_d, sb).hbytes && (sb & 3) == 0 &&
            al16(g.V32) && al16(g.phat_hi) && al16(g.phat_lo) && al16(c_in)) {
          const size_t per = wu_staged_layout(a.n_d, sb).total;
          const int w = warps_per_block(per);
          if (w == 0) return -1;
          auto ks = k_b2_wu_staged<SH>;
          if (cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(per * w)) != cudaSuccess)
            return -1;
          ks<<<ceil_div(a.noa, w), 32 * w, per * w, stream>>>(
              a, g, species, row_of_atom, reinterpret_cast<const float *>(c_in), norm_in,
              atom_e, reinterpret_cast<float *>(u_buf));
          return 0;
        }
      }
      auto kern = k_b2_wu<T, SH>;
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem) != cudaSuccess)
        return -1;
      kern<<<ceil_div(a.noa, wpb), 32 * wpb, smem, stream>>>(a, g, species, row_of_atom,
                                                             pair_tab, c_in, norm_in,
                                                             atom_e, u_buf);
      return 0;
    });
    if (rc != 0) return -1;
  }
  if (cudaGetLastError() != cudaSuccess) return -1;
  if (n_pairs > 0) {
    with_shape<T>(a, [&](auto sh) {
      k_pair_force<T, decltype(sh)><<<(unsigned)((n_pairs + 127) / 128), 128, 0, stream>>>(
          a, g.strict, n_pairs, nbr_i, nb.rel, nb.rel32, nb.geom, nb.nbr_s, species, u_buf,
          pair_f);
      return 0;
    });
    if (cudaGetLastError() != cudaSuccess) return -1;
  }
  if (!gather) return 0;
  int nblk;
  if constexpr (sizeof(T) == 4) {
    // a few resident blocks per SM, each walking many atoms
    nblk = std::min(ceil_div(a.noa, kGatherWarps * (32 / kGatherLanes)), 152 * 8);
    k_gather_warp<<<nblk, 32 * kGatherWarps, 0, stream>>>(
        a.noa, nb.offset, nb.rev, nb.rel32, reinterpret_cast<const float4 *>(pair_f), atom_e,
        forces, atom_vir);
  } else {
    nblk = ceil_div(a.noa, 128);
    k_gather<T><<<nblk, 128, 0, stream>>>(a.noa, nb.offset, nb.rev, nb.rel32, nb.rel, pair_f,
                                          atom_e, forces, atom_vir);
  }
  if (cudaGetLastError() != cudaSuccess) return -1;
  k_reduce<<<10, 128, 0, stream>>>(nblk, atom_vir, reduce_out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template int launch_b2_forward<float>(B2Args, const Neigh &, const int *, const int *,
                                      const int *, float *, float *, double *,
                                      double *, __half *, __half *, int, const float *,
                                      cudaStream_t);
template int launch_b2_forward<double>(B2Args, const Neigh &, const int *, const int *,
                                       const int *, double *, double *, double *,
                                       double *, __half *, __half *, int, const float *,
                                       cudaStream_t);
template int launch_b2_adjoint<float>(B2Args, const AdjArgs &, const Neigh &,
                                      const int *, const int *, const int *,
                                      const float *, const double *, double *,
                                      float *, double *, double *, double *,
                                      bool, float *, long long, const int *, cudaStream_t);
template int launch_b2_adjoint<double>(B2Args, const AdjArgs &, const Neigh &,
                                       const int *, const int *, const int *,
                                       const double *, const double *, double *,
                                       double *, double *, double *, double *,
                                       bool, double *, long long, const int *,
                                       cudaStream_t);

}  // namespace fpp
