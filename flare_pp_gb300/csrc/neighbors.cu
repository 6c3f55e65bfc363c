// Periodic neighbor list on the GPU with the reference's exact semantics.
//
// The reference (src/flare_pp/structure.cpp:52-118) scans every pair (i, j)
// and every image shift s in [-sweep, sweep]^3, keeps dist < cutoff &&
// dist != 0, and orders each atom's list by j, then s1, s2, s3.  Here the
// same (j, s) pairs are found through bins in fractional coordinates:
//   1. wrap_bin    wrapped positions (reference formula, exact FP64 order),
//                  their float-float split, fractional coordinates, a bin
//                  (bins are about half the cutoff wide)
//   2. bin sort    counting sort of atoms into bins
//   3. enum        warp per atom: the bin ranges reachable for each shift
//                  (looked up across the lanes), candidates tested in FP32
//                  with a safety margin, the ones near the cutoff decided in
//                  float-float and, within ~1e-6 A of it, by the reference's
//                  FP64 distance; accepted keys (j << 20 | shift) sorted into
//                  reference order (warp bitonic sort) in a per-atom slab
//   4. compact     CSR arrays from the slabs; the FP32 pair vector of the
//                  canonical half from the float-float image, written to the
//                  pair and (negated) to its reverse (j, i, -s), whose index
//                  it finds and links for the deterministic force gather
// An atom with more than 256 neighbors sends the build through the two-pass
// path (count, fill, sort_geom with FP64 geometry, reverse).  All FP64
// arithmetic that decides membership or is returned uses explicitly rounded
// operations, so results equal the oracle bit for bit; the FP64 pair table is
// filled on demand (ensure_rel64) for the callers that return or consume FP64
// geometry.
#include <cub/cub.cuh>
#include <algorithm>
#include <cstring>

#include <cmath>
#include <cstdio>

#include "common.cuh"
#include "geom.cuh"
#include "internal.h"

namespace fpp {

struct CellDev {
  double cell[9], ct[9], ct_inv[9], cdot[9], cdot_inv[9];
  float cell32[9];
  CellFF cff;               // lattice vectors as float-float
  float cut2_hi, cut2_lo;   // cutoff^2 as float-float
  float ff_eps;             // |r^2_ff - cutoff^2| above this decides without FP64
  double cutoff;
  float in2, out2, zero2;  // FP32 squared-distance bands: surely inside below
                           // in2, surely outside above out2, and distances
                           // below sqrt(zero2) re-checked for dist == 0;
                           // everything between is decided in exact FP64
  float delta32[3];        // fractional reach per lattice direction
  int sweep, ns, n_shift;
  int nb[3];
};

static CellDev make_dev(const CellInfo &ci) {
  CellDev d;
  for (int k = 0; k < 9; k++) {
    d.cell[k] = ci.cell[k];
    d.ct[k] = ci.ct[k];
    d.ct_inv[k] = ci.ct_inv[k];
    d.cdot[k] = ci.cdot[k];
    d.cdot_inv[k] = ci.cdot_inv[k];
    d.cell32[k] = (float)ci.cell[k];
    d.cff.hi[k] = (float)ci.cell[k];
    d.cff.lo[k] = (float)(ci.cell[k] - (double)d.cff.hi[k]);
  }
  d.cutoff = ci.cutoff;
  {
    const double c2 = ci.cutoff * ci.cutoff;
    d.cut2_hi = (float)c2;
    d.cut2_lo = (float)(c2 - (double)d.cut2_hi);
  }
  double cmax = 0;
  for (int k = 0; k < 9; k++) cmax = fmax(cmax, fabs(ci.cell[k]));
  // FP32 positions are within 2^-24 |x| of the FP64 ones; an FP32 image
  // component then errs by at most ~2^-24 (18 + 12 sweep) cmax, which the
  // margin covers about five times over
  double margin = 2e-4 + 4e-6 * (cmax * (2 * ci.sweep + 2) + ci.cutoff);
  d.in2 = (float)((ci.cutoff - margin) * (ci.cutoff - margin));
  if (ci.cutoff <= margin) d.in2 = 0.f;
  d.out2 = (float)((ci.cutoff + margin) * (ci.cutoff + margin));
  d.zero2 = (float)(margin * margin);
  for (int k = 0; k < 3; k++)
    d.delta32[k] = (float)((ci.cutoff + 2 * margin) / ci.height[k] + 1e-6);
  d.sweep = ci.sweep;
  d.ns = 2 * ci.sweep + 1;
  d.n_shift = d.ns * d.ns * d.ns;
  for (int k = 0; k < 3; k++) d.nb[k] = ci.nb[k];
  // float-float image error: positions split hi + lo carry ~2^-48 |x|, and
  // each float-float operation errs by ~2^-44 of its operands' magnitude;
  // with about ten operations on magnitudes below scale = cmax (2 sweep + 2)
  // + rc, a component errs by < 2^-40 scale and r^2 by 2 r times that.  The
  // margin is 2^-30 scale (2 rc + 1): a thousand times more, and still far
  // below the FP32 rounding of any distance.
  {
    const double scale = cmax * (2 * ci.sweep + 2) + ci.cutoff;
    d.ff_eps = (float)(std::ldexp(1.0, -30) * scale * (2.0 * ci.cutoff + 1.0) + 1e-30);
  }
  return d;
}

NbGeom nb_geom(const StructureState &st) {
  NbGeom g;
  g.wp = st.wrapped.as<dvec4>();
  g.keys = st.nbr_key.as<long long>();
  for (int k = 0; k < 9; k++) g.cell[k] = st.ci.cell[k];
  g.sweep = st.ci.sweep;
  g.ns = 2 * st.ci.sweep + 1;
  return g;
}

// (n,3) x (3,3) row with the sum order ((a0 b0 + a1 b1) + a2 b2).
__device__ __forceinline__ void mm3(const double a[3], const double *m,
                                    double out[3]) {
#pragma unroll
  for (int j = 0; j < 3; j++)
    out[j] = dadd(dadd(dmul(a[0], m[0 * 3 + j]), dmul(a[1], m[1 * 3 + j])),
                  dmul(a[2], m[2 * 3 + j]));
}

// Structure::wrap_positions (structure.cpp:120-133) plus binning.
__global__ void k_wrap_bin(int noa, const double *__restrict__ pos, CellDev cd,
                           dvec4 *__restrict__ wp, float4 *__restrict__ wp32,
                           float4 *__restrict__ wp_lo,
                           float4 *__restrict__ frac, int *__restrict__ atom_bin,
                           int *__restrict__ bin_count, DeviceStatus *st) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= noa) return;
  double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
  if (!isfinite(p[0]) || !isfinite(p[1]) || !isfinite(p[2])) {
    set_status(st, FPP_ERR_NUMERIC, 1, i);
    p[0] = p[1] = p[2] = 0.0;
  }
  double t[3], rel[3], rw[3], w[3];
  mm3(p, cd.ct, t);
  mm3(t, cd.cdot_inv, rel);
#pragma unroll
  for (int k = 0; k < 3; k++) rw[k] = dsub(rel[k], floor(rel[k]));
  mm3(rw, cd.cdot, t);
  mm3(t, cd.ct_inv, w);
  wp[i] = dvec4{w[0], w[1], w[2], 0.0};
  const float4 h = make_float4((float)w[0], (float)w[1], (float)w[2], 0.f);
  wp32[i] = h;
  wp_lo[i] = make_float4((float)(w[0] - (double)h.x), (float)(w[1] - (double)h.y),
                         (float)(w[2] - (double)h.z), 0.f);
  frac[i] = make_float4((float)rw[0], (float)rw[1], (float)rw[2], 0.f);
  int b[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    int v = (int)floor(rw[k] * cd.nb[k]);
    b[k] = min(max(v, 0), cd.nb[k] - 1);
  }
  int bin = (b[0] * cd.nb[1] + b[1]) * cd.nb[2] + b[2];
  atom_bin[i] = bin;
  atomicAdd(&bin_count[bin], 1);
}

__global__ void k_bin_scatter(int noa, const int *__restrict__ atom_bin,
                              const int *__restrict__ bin_start,
                              int *__restrict__ bin_cursor,
                              int *__restrict__ bin_atoms,
                              const float4 *__restrict__ wp32,
                              float4 *__restrict__ binned) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= noa) return;
  int b = atom_bin[i];
  int slot = atomicAdd(&bin_cursor[b], 1);
  bin_atoms[bin_start[b] + slot] = i;
  float4 q = wp32[i];
  q.w = __int_as_float(i);  // FP32 position and atom index in one 16-byte load
  binned[bin_start[b] + slot] = q;
}

// Exact FP64 image distance of the reference (structure.cpp:69-77):
// im = ((diff + s1 c0) + s2 c1) + s3 c2, dist = sqrt((x^2 + y^2) + z^2).
// dadd(v, dmul(s, c)) bit for bit, with the products by 0 and +-1 (exact)
// formed without FP64 instructions, which are scarce on this GPU.
__device__ __forceinline__ double exact_image(const dvec4 &wi, const dvec4 &wj,
                                              const CellDev &cd, int s1, int s2,
                                              int s3, double im[3]) {
  return exact_image_cell(wi, wj, cd.cell, s1, s2, s3, im);
}

// The exact FP64 decision, out of line: it is rarely reached, and kept out
// of the callers' instruction stream and registers.
static __device__ __noinline__ bool member_fp64(const dvec4 *__restrict__ wp, int i, int j,
                                         const CellDev &cd, int s1, int s2, int s3) {
  double imd[3];
  const double dist = exact_image(wp[i], wp[j], cd, s1, s2, s3, imd);
  return (dist < cd.cutoff) && (dist != 0.0);
}

// Membership of a candidate whose FP32 distance fell in the band around the
// cutoff (or near zero): float-float first, the exact FP64 distance only if
// that is within ff_eps of the cutoff or of zero.
__device__ __forceinline__ bool band_member(int i, int j, const CellDev &cd,
                                            const dvec4 *__restrict__ wp,
                                            const float4 *__restrict__ wp32,
                                            const float4 *__restrict__ wp_lo, int s1,
                                            int s2, int s3) {
  ff im[3], r2;
  image_ff(wp32[i], wp_lo[i], wp32[j], wp_lo[j], cd.cff, s1, s2, s3, im, r2);
  const ff d = ff_add(r2, ff{-cd.cut2_hi, -cd.cut2_lo});
  const float dv = d.hi + d.lo;
  if (r2.hi > cd.ff_eps) {
    if (dv < -cd.ff_eps) return true;
    if (dv > cd.ff_eps) return false;
  }
  return member_fp64(wp, i, j, cd, s1, s2, s3);
}

// Enumerate the candidate (j, s) pairs of atom i; `emit` is called by each
// lane for each accepted pair.  All lanes of the warp call this together.
// Candidates are screened in FP32; only pairs whose FP32 distance lies within
// the margin band around the cutoff (or near zero) are decided by the
// reference's exact FP64 distance, so the accepted set is the reference's.
template <typename Emit>
__device__ __forceinline__ void enumerate_pairs(int i, const CellDev &cd,
                                                const dvec4 *__restrict__ wp,
                                                const float4 *__restrict__ wp32,
                                                const float4 *__restrict__ frac,
                                                const int *__restrict__ bin_start,
                                                const int *__restrict__ bin_atoms,
                                                Emit emit) {
  const int lane = threadIdx.x & 31;
  const float4 pi = wp32[i];
  const float4 fi = frac[i];
  const float fik[3] = {fi.x, fi.y, fi.z};
  for (int s1 = -cd.sweep; s1 <= cd.sweep; s1++) {
    for (int s2 = -cd.sweep; s2 <= cd.sweep; s2++) {
      for (int s3 = -cd.sweep; s3 <= cd.sweep; s3++) {
        const int sv[3] = {s1, s2, s3};
        int lo[3], hi[3];
        bool empty = false;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const float c = fik[k] - (float)sv[k];
          int l = (int)floorf((c - cd.delta32[k]) * cd.nb[k]);
          int h = (int)floorf((c + cd.delta32[k]) * cd.nb[k]);
          l = max(l, 0);
          h = min(h, cd.nb[k] - 1);
          if (l > h) empty = true;
          lo[k] = l;
          hi[k] = h;
        }
        if (empty) continue;
        const int sidx = ((s1 + cd.sweep) * cd.ns + (s2 + cd.sweep)) * cd.ns +
                         (s3 + cd.sweep);
        const float sx = s1 * cd.cell32[0] + s2 * cd.cell32[3] + s3 * cd.cell32[6];
        const float sy = s1 * cd.cell32[1] + s2 * cd.cell32[4] + s3 * cd.cell32[7];
        const float sz = s1 * cd.cell32[2] + s2 * cd.cell32[5] + s3 * cd.cell32[8];
        for (int b0 = lo[0]; b0 <= hi[0]; b0++)
          for (int b1 = lo[1]; b1 <= hi[1]; b1++)
            for (int b2 = lo[2]; b2 <= hi[2]; b2++) {
              int bin = (b0 * cd.nb[1] + b1) * cd.nb[2] + b2;
              int beg = bin_start[bin], end = bin_start[bin + 1];
              for (int base = beg; base < end; base += 32) {
                int t = base + lane;
                bool ok = false;
                int j = -1;
                if (t < end) {
                  j = bin_atoms[t];
                  float4 pj = wp32[j];
                  float dx = (pj.x - pi.x) + sx;
                  float dy = (pj.y - pi.y) + sy;
                  float dz = (pj.z - pi.z) + sz;
                  const float d2 = dx * dx + dy * dy + dz * dz;
                  if (d2 < cd.in2 && d2 > cd.zero2) {
                    ok = true;
                  } else if (d2 <= cd.out2) {
                    double im[3];
                    double dist = exact_image(wp[i], wp[j], cd, s1, s2, s3, im);
                    ok = (dist < cd.cutoff) && (dist != 0.0);
                  }
                }
                emit(ok, j, sidx);
              }
            }
      }
    }
  }
}

// Single-pass enumeration (one warp per atom): the candidate bin ranges of
// all shifts are listed in shared memory, candidates are then tested 32 at a
// time across ranges (FP32, exact FP64 only in the band around the cutoff),
// accepted keys are collected and rank-sorted in shared memory and written to
// a per-atom slab of kSlabCap keys.  An atom with more neighbors sets
// *overflow and the caller rebuilds with the two-pass kernels below.
constexpr int kSlabCap = 256;
constexpr int kMaxRanges = 64;
constexpr int kEnumWarps = 4;

__global__ void __launch_bounds__(32 * kEnumWarps)
k_enum(int noa, CellDev cd, const dvec4 *__restrict__ wp, const float4 *__restrict__ wp32,
       const float4 *__restrict__ wp_lo,
       const float4 *__restrict__ frac, const int *__restrict__ bin_start,
       const float4 *__restrict__ binned, int *__restrict__ count,
       long long *__restrict__ slab, int *__restrict__ overflow) {
  __shared__ long long s_keys[kEnumWarps][kSlabCap];
  __shared__ int s_rstart[kEnumWarps][kMaxRanges];
  __shared__ int s_rpre[kEnumWarps][kMaxRanges + 1];
  __shared__ int s_rsidx[kEnumWarps][kMaxRanges];
  __shared__ float4 s_rshift[kEnumWarps][kMaxRanges];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kEnumWarps + w;
  if (i >= noa) return;
  const float4 pi = wp32[i];
  const float4 fi = frac[i];
  const float fik[3] = {fi.x, fi.y, fi.z};
  const int center = (cd.sweep * cd.ns + cd.sweep) * cd.ns + cd.sweep;
  int nacc = 0, nr = 0, tot = 0;
  if (lane == 0) s_rpre[w][0] = 0;
  __syncwarp();
  auto flush = [&]() {
    for (int base = 0; base < tot; base += 32) {
      const int t = base + lane;
      bool ok = false;
      long long key = 0;
      if (t < tot) {
        int lo = 0, hi = nr - 1;  // last range with rpre <= t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_rpre[w][mid] <= t)
            lo = mid;
          else
            hi = mid - 1;
        }
        const float4 q = binned[s_rstart[w][lo] + (t - s_rpre[w][lo])];
        const float4 sh = s_rshift[w][lo];
        const float dx = (q.x - pi.x) + sh.x;
        const float dy = (q.y - pi.y) + sh.y;
        const float dz = (q.z - pi.z) + sh.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const int j = __float_as_int(q.w);
        const int sidx = s_rsidx[w][lo];
        if (d2 < cd.in2 && d2 > cd.zero2) {
          ok = true;
        } else if (j == i && sidx == center) {
          ok = false;  // the atom itself: its exact distance is 0
        } else if (d2 <= cd.out2) {
          int s1, s2, s3;
          decode_shift(sidx, cd.ns, cd.sweep, s1, s2, s3);
          ok = band_member(i, j, cd, wp, wp32, wp_lo, s1, s2, s3);
        }
        key = ((long long)j << kKeyBits) | sidx;
      }
      const unsigned m = __ballot_sync(0xffffffffu, ok);
      if (ok) {
        const int pos = nacc + __popc(m & ((1u << lane) - 1u));
        if (pos < kSlabCap) s_keys[w][pos] = key;
      }
      nacc += __popc(m);
    }
    nr = 0;
    tot = 0;
    __syncwarp();
  };
  // the shifts' bin ranges are evaluated one shift per lane; the warp then
  // walks the non-empty ones
  const unsigned full = 0xffffffffu;
  for (int s0 = 0; s0 < cd.n_shift; s0 += 32) {
    const int sidx = s0 + lane;
    int lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1};
    float4 sh = make_float4(0.f, 0.f, 0.f, 0.f);
    bool nonempty = false;
    if (sidx < cd.n_shift) {
      const int s3 = sidx % cd.ns - cd.sweep;
      const int s2 = (sidx / cd.ns) % cd.ns - cd.sweep;
      const int s1 = sidx / (cd.ns * cd.ns) - cd.sweep;
      const int sv[3] = {s1, s2, s3};
      nonempty = true;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float c = fik[k] - (float)sv[k];
        const int l = (int)floorf((c - cd.delta32[k]) * cd.nb[k]);
        const int h = (int)floorf((c + cd.delta32[k]) * cd.nb[k]);
        lo[k] = max(l, 0);
        hi[k] = min(h, cd.nb[k] - 1);
        if (lo[k] > hi[k]) nonempty = false;
      }
      sh = make_float4(s1 * cd.cell32[0] + s2 * cd.cell32[3] + s3 * cd.cell32[6],
                       s1 * cd.cell32[1] + s2 * cd.cell32[4] + s3 * cd.cell32[7],
                       s1 * cd.cell32[2] + s2 * cd.cell32[5] + s3 * cd.cell32[8], 0.f);
    }
    unsigned todo = __ballot_sync(full, nonempty);
    while (todo) {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1;
      const int ssrc = __shfl_sync(full, sidx, src);
      const int l0 = __shfl_sync(full, lo[0], src), h0 = __shfl_sync(full, hi[0], src);
      const int l1 = __shfl_sync(full, lo[1], src), h1 = __shfl_sync(full, hi[1], src);
      const int l2 = __shfl_sync(full, lo[2], src), h2 = __shfl_sync(full, hi[2], src);
      const float4 shs = make_float4(__shfl_sync(full, sh.x, src), __shfl_sync(full, sh.y, src),
                                     __shfl_sync(full, sh.z, src), 0.f);
      // bins along the last direction are contiguous: one range per (b0, b1),
      // looked up by the lanes in parallel, appended in (b0, b1) order
      const int w1 = h1 - l1 + 1, ncomb = (h0 - l0 + 1) * w1;
      for (int c0 = 0; c0 < ncomb; c0 += 32) {
        const int c = c0 + lane;
        int st = 0, cn = 0;
        if (c < ncomb) {
          const int b0 = l0 + c / w1, b1 = l1 + c % w1;
          const int bin_lo = (b0 * cd.nb[1] + b1) * cd.nb[2] + l2;
          const int bin_hi = (b0 * cd.nb[1] + b1) * cd.nb[2] + h2;
          st = bin_start[bin_lo];
          cn = bin_start[bin_hi + 1] - st;
        }
        const unsigned nz = __ballot_sync(full, cn > 0);
        const int k = __popc(nz);
        if (k == 0) continue;
        if (nr + k > kMaxRanges) flush();
        int incl = cn;  // inclusive scan of the counts in lane order
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(full, incl, o);
          if (lane >= o) incl += v;
        }
        if (cn > 0) {
          const int idx = nr + __popc(nz & ((1u << lane) - 1u));
          s_rstart[w][idx] = st;
          s_rsidx[w][idx] = ssrc;
          s_rshift[w][idx] = shs;
          s_rpre[w][idx + 1] = tot + incl;
        }
        __syncwarp();
        tot += __shfl_sync(full, incl, 31);
        nr += k;
      }
    }
  }
  flush();
  if (lane == 0) count[i] = nacc;
  if (nacc > kSlabCap) {
    if (lane == 0) atomicExch(overflow, 1);
    return;
  }
  if (nacc <= 64) {
    // bitonic sort across the warp, key e in lane e % 32, register e / 32
    // (the keys are unique; the padding sorts last)
    const long long pad = 0x7fffffffffffffffLL;
    long long k0 = lane < nacc ? s_keys[w][lane] : pad;
    long long k1 = lane + 32 < nacc ? s_keys[w][lane + 32] : pad;
    auto step = [&](long long v, int e, int stride, int size) {
      const long long o = __shfl_xor_sync(0xffffffffu, v, stride);
      const bool keep_min = ((e & stride) == 0) == ((e & size) == 0);
      return keep_min ? (v < o ? v : o) : (v < o ? o : v);
    };
    for (int size = 2; size <= 64; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        if (stride == 32) {  // partners in the same lane; size 64 ascends everywhere
          const long long lo = k0 < k1 ? k0 : k1, hi = k0 < k1 ? k1 : k0;
          k0 = lo;
          k1 = hi;
        } else {
          k0 = step(k0, lane, stride, size);
          k1 = step(k1, lane + 32, stride, size);
        }
      }
    if (lane < nacc) slab[(size_t)i * kSlabCap + lane] = k0;
    if (lane + 32 < nacc) slab[(size_t)i * kSlabCap + lane + 32] = k1;
    return;
  }
  for (int e = lane; e < nacc; e += 32) {
    const long long key = s_keys[w][e];
    int rank = 0;
    for (int f = 0; f < nacc; f++) rank += (s_keys[w][f] < key) ? 1 : 0;
    slab[(size_t)i * kSlabCap + rank] = key;
  }
}

// Slab -> CSR in reference order, with the FP64 geometry of every pair.
__global__ void k_compact_geom(int noa, CellDev cd, const float4 *__restrict__ wp32,
                               const float4 *__restrict__ wp_lo,
                               const int *__restrict__ species,
                               const int *__restrict__ offset,
                               const long long *__restrict__ slab,
                               long long *__restrict__ keys, int *__restrict__ nbr_i,
                               int *__restrict__ nbr_j, int *__restrict__ nbr_s,
                               float4 *__restrict__ rel32, int *__restrict__ rev,
                               DeviceStatus *st, long long cap,
                               const int *__restrict__ flags) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= noa) return;
  // launched before the host has read the pair total: nothing is written
  // when the slab overflowed or the pair buffers hold fewer than the total
  if (flags[0] != 0 || (long long)offset[noa] > cap) return;
  const int lane = threadIdx.x & 31;
  const int beg = offset[i], n = offset[i + 1] - beg;
  const float4 hi_i = wp32[i], lo_i = wp_lo[i];
  // the pair (i, j, s) and its reverse (j, i, -s) have exactly negated
  // images, so the geometry is computed for the canonical half only -- keys
  // above (i, centre shift), a suffix of the sorted list -- and written to
  // both; the canonical pair also finds its reverse (binary search in j's
  // sorted slab row) and links the two.  FP32 vectors come from the
  // float-float image (no FP64 here).
  const long long thr = ((long long)i << kKeyBits) |
                        ((cd.sweep * cd.ns + cd.sweep) * cd.ns + cd.sweep);
  int c0 = 0;
  for (int e0 = 0; e0 < n; e0 += 32) {
    const int e = e0 + lane;
    long long key = 0;
    if (e < n) {
      key = slab[(size_t)i * kSlabCap + e];
      const int out = beg + e;
      const int j = (int)(key >> kKeyBits);
      keys[out] = key;
      nbr_i[out] = i;
      nbr_j[out] = j;
      nbr_s[out] = species[j];
    }
    c0 += __popc(__ballot_sync(0xffffffffu, e < n && key <= thr));
  }
  for (int e = c0 + lane; e < n; e += 32) {
    const long long key = slab[(size_t)i * kSlabCap + e];
    const int j = (int)(key >> kKeyBits);
    const int sidx = (int)(key & kKeyMask);
    int s1, s2, s3;
    decode_shift(sidx, cd.ns, cd.sweep, s1, s2, s3);
    ff im[3], r2;
    image_ff(hi_i, lo_i, wp32[j], wp_lo[j], cd.cff, s1, s2, s3, im, r2);
    const float4 v = make_float4(im[0].hi + im[0].lo, im[1].hi + im[1].lo,
                                 im[2].hi + im[2].lo, ff_sqrt_f(r2));
    const int out = beg + e;
    rel32[out] = v;
    // reverse pair (j, i, -s) in j's sorted row
    const long long want = ((long long)i << kKeyBits) | (cd.n_shift - 1 - sidx);
    const long long *row = slab + (size_t)j * kSlabCap;
    int lo = 0, hi = offset[j + 1] - offset[j] - 1, found = -1;
    while (lo <= hi) {
      const int mid = (lo + hi) >> 1;
      const long long k = row[mid];
      if (k == want) {
        found = mid;
        break;
      }
      if (k < want)
        lo = mid + 1;
      else
        hi = mid - 1;
    }
    if (found < 0) {
      set_status(st, FPP_ERR_NUMERIC, 7, out);
      rev[out] = -1;
      continue;
    }
    const int orev = offset[j] + found;
    rev[out] = orev;
    rev[orev] = out;
    rel32[orev] = make_float4(-v.x, -v.y, -v.z, v.w);
  }
}

// The FP64 pair table (r, x, y, z) of every pair, by the reference's formula.
__global__ void k_rel64(long long n_pairs, CellDev cd, const dvec4 *__restrict__ wp,
                        const long long *__restrict__ keys, const int *__restrict__ nbr_i,
                        dvec4 *__restrict__ rel) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const long long key = keys[p];
  int s1, s2, s3;
  decode_shift((int)(key & kKeyMask), cd.ns, cd.sweep, s1, s2, s3);
  double im[3];
  const double dist = exact_image(wp[nbr_i[p]], wp[(int)(key >> kKeyBits)], cd, s1, s2, s3, im);
  rel[p] = dvec4{dist, im[0], im[1], im[2]};
}

__global__ void k_count(int noa, CellDev cd, const dvec4 *__restrict__ wp,
                        const float4 *__restrict__ wp32,
                        const float4 *__restrict__ frac,
                        const int *__restrict__ bin_start,
                        const int *__restrict__ bin_atoms,
                        int *__restrict__ count) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= noa) return;
  int lane = threadIdx.x & 31;
  int n = 0;
  enumerate_pairs(i, cd, wp, wp32, frac, bin_start, bin_atoms,
                  [&](bool ok, int, int) { n += ok ? 1 : 0; });
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if (lane == 0) count[i] = n;
}

__global__ void k_fill(int noa, CellDev cd, const dvec4 *__restrict__ wp,
                       const float4 *__restrict__ wp32,
                       const float4 *__restrict__ frac,
                       const int *__restrict__ bin_start,
                       const int *__restrict__ bin_atoms,
                       const int *__restrict__ offset,
                       long long *__restrict__ keys) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= noa) return;
  int lane = threadIdx.x & 31;
  int pos = offset[i];
  enumerate_pairs(i, cd, wp, wp32, frac, bin_start, bin_atoms,
                  [&](bool ok, int j, int sidx) {
                    unsigned m = __ballot_sync(0xffffffffu, ok);
                    if (ok) {
                      int r = __popc(m & ((1u << lane) - 1u));
                      keys[pos + r] = ((long long)j << kKeyBits) | sidx;
                    }
                    pos += __popc(m);
                  });
}

// Rank the unique keys of each atom's segment and write the pair geometry in
// reference order.
__global__ void k_sort_geom(int noa, CellDev cd, const dvec4 *__restrict__ wp,
                            const int *__restrict__ species,
                            const int *__restrict__ offset,
                            const long long *__restrict__ keys_tmp,
                            long long *__restrict__ keys, int *__restrict__ nbr_i,
                            int *__restrict__ nbr_j, int *__restrict__ nbr_s,
                            dvec4 *__restrict__ rel, float4 *__restrict__ rel32) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= noa) return;
  int lane = threadIdx.x & 31;
  int beg = offset[i], end = offset[i + 1];
  const dvec4 wi = wp[i];
  for (int e = beg + lane; e < end; e += 32) {
    long long key = keys_tmp[e];
    int rank = 0;
    for (int f = beg; f < end; f++) rank += (keys_tmp[f] < key) ? 1 : 0;
    int out = beg + rank;
    int j = (int)(key >> kKeyBits);
    int sidx = (int)(key & kKeyMask);
    int s3 = sidx % cd.ns - cd.sweep;
    int s2 = (sidx / cd.ns) % cd.ns - cd.sweep;
    int s1 = sidx / (cd.ns * cd.ns) - cd.sweep;
    double im[3];
    double dist = exact_image(wi, wp[j], cd, s1, s2, s3, im);
    keys[out] = key;
    nbr_i[out] = i;
    nbr_j[out] = j;
    nbr_s[out] = species[j];
    rel[out] = dvec4{dist, im[0], im[1], im[2]};
    rel32[out] = make_float4((float)im[0], (float)im[1], (float)im[2], (float)dist);
  }
}

// Reverse pair: (i, j, s) -> (j, i, -s), found by binary search in j's list
// (the two-pass build; the one-pass build links pairs in k_compact_geom).
__global__ void k_reverse(long long n_pairs, CellDev cd,
                          const int *__restrict__ offset,
                          const long long *__restrict__ keys,
                          const int *__restrict__ nbr_i,
                          const int *__restrict__ nbr_j, int *__restrict__ rev,
                          DeviceStatus *st) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  int i = nbr_i[p], j = nbr_j[p];
  int sidx = (int)(keys[p] & kKeyMask);
  long long want = ((long long)i << kKeyBits) | (cd.n_shift - 1 - sidx);
  int lo = offset[j], hi = offset[j + 1] - 1, found = -1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    long long k = keys[mid];
    if (k == want) {
      found = mid;
      break;
    }
    if (k < want)
      lo = mid + 1;
    else
      hi = mid - 1;
  }
  if (found < 0) set_status(st, FPP_ERR_NUMERIC, 6, (int)p);
  rev[p] = found;
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
static void inv3(const double a[9], double out[9], double *det_out) {
  double c00 = a[4] * a[8] - a[5] * a[7];
  double c01 = a[5] * a[6] - a[3] * a[8];
  double c02 = a[3] * a[7] - a[4] * a[6];
  double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  out[0] = c00 / det;
  out[3] = c01 / det;
  out[6] = c02 / det;
  out[1] = (a[2] * a[7] - a[1] * a[8]) / det;
  out[4] = (a[0] * a[8] - a[2] * a[6]) / det;
  out[7] = (a[1] * a[6] - a[0] * a[7]) / det;
  out[2] = (a[1] * a[5] - a[2] * a[4]) / det;
  out[5] = (a[2] * a[3] - a[0] * a[5]) / det;
  out[8] = (a[0] * a[4] - a[1] * a[3]) / det;
  if (det_out) *det_out = det;
}

static double dot3(const double *a, const double *b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

int make_cell_info(const double *cell, double cutoff, CellInfo *ci) {
  for (int k = 0; k < 9; k++) {
    if (!std::isfinite(cell[k])) return fail(FPP_ERR_NUMERIC, "cell is not finite");
    ci->cell[k] = cell[k];
  }
  if (!(cutoff > 0) || !std::isfinite(cutoff))
    return fail(FPP_ERR_INVALID, "cutoff must be positive and finite");
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) ci->ct[i * 3 + j] = cell[j * 3 + i];
  double det_ct, det;
  inv3(ci->ct, ci->ct_inv, &det_ct);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      ci->cdot[i * 3 + j] = (cell[i * 3 + 0] * ci->ct[0 * 3 + j] +
                             cell[i * 3 + 1] * ci->ct[1 * 3 + j]) +
                            cell[i * 3 + 2] * ci->ct[2 * 3 + j];
  inv3(ci->cdot, ci->cdot_inv, nullptr);
  double tmp[9];
  inv3(cell, tmp, &det);
  if (!(std::fabs(det) > 0) || !std::isfinite(det))
    return fail(FPP_ERR_INVALID, "cell is singular");
  ci->volume = std::fabs(det);
  // get_single_sweep_cutoff (structure.cpp:135-165)
  const double *v1 = cell, *v2 = cell + 3, *v3 = cell + 6;
  double ab = dot3(v1, v2), ac = dot3(v1, v3), bc = dot3(v2, v3);
  double a = std::sqrt(dot3(v1, v1)), b = std::sqrt(dot3(v2, v2)),
         c = std::sqrt(dot3(v3, v3));
  auto h = [](double x, double cs) { return x * std::sqrt(1 - cs * cs); };
  double cand[6] = {h(a, ab / (a * b)), h(b, ab / (a * b)), h(a, ac / (a * c)),
                    h(c, ac / (a * c)), h(b, bc / (b * c)), h(c, bc / (b * c))};
  double ssc = cand[0];
  for (int k = 0; k < 6; k++)
    if (cand[k] < ssc) ssc = cand[k];
  ci->single_sweep_cutoff = ssc;
  ci->cutoff = cutoff;
  double sw = std::ceil(cutoff / ssc);
  if (!(sw >= 1) || sw > 16)
    return fail(FPP_ERR_CAPACITY, "cutoff needs more than 16 periodic sweeps");
  ci->sweep = (int)sw;
  // face-to-face heights: volume / |a_j x a_k|
  for (int k = 0; k < 3; k++) {
    const double *p = cell + 3 * ((k + 1) % 3), *q = cell + 3 * ((k + 2) % 3);
    double cx = p[1] * q[2] - p[2] * q[1];
    double cy = p[2] * q[0] - p[0] * q[2];
    double cz = p[0] * q[1] - p[1] * q[0];
    ci->height[k] = ci->volume / std::sqrt(cx * cx + cy * cy + cz * cz);
    // bins of about half the cutoff: an atom's reach then spans ~5 bins per
    // direction instead of 3 whole-cutoff bins, ~40% fewer candidates
    int nb = (int)std::floor(ci->height[k] / (0.5 * cutoff * (1 + 1e-6) + 1e-6));
    ci->nb[k] = std::min(std::max(nb, 1), 1024);
  }
  long long nbins = (long long)ci->nb[0] * ci->nb[1] * ci->nb[2];
  while (nbins > (1ll << 22)) {
    for (int k = 0; k < 3; k++) ci->nb[k] = std::max(1, ci->nb[k] / 2);
    nbins = (long long)ci->nb[0] * ci->nb[1] * ci->nb[2];
  }
  return FPP_OK;
}

int ensure_readback(StructureState &st) {
  if (st.rb) return FPP_OK;
  void *h = nullptr, *d = nullptr;
  FPP_CUDA(cudaHostAlloc(&h, sizeof(HostReadback), cudaHostAllocMapped));
  const cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
  if (e != cudaSuccess) {
    cudaFreeHost(h);
    return cuda_fail(e, "cudaHostGetDevicePointer");
  }
  std::memset(h, 0, sizeof(HostReadback));
  st.rb = static_cast<HostReadback *>(h);
  st.rb_dev = static_cast<HostReadback *>(d);
  return FPP_OK;
}

int status_from_readback(StructureState &st, cudaStream_t stream, const char *what) {
  const DeviceStatus h = *reinterpret_cast<const DeviceStatus *>(st.rb->status);
  if (h.code != 0) {
    // cleared once reported (an asynchronous call leaves its errors here for
    // the next synchronizing call)
    FPP_CUDA(cudaMemsetAsync(st.status.ptr, 0, sizeof(DeviceStatus), stream));
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: device status %d at %d (index %d)", what,
             h.code, h.where, h.info);
    return fail(h.code, buf);
  }
  return FPP_OK;
}

int check_status(StructureState &st, cudaStream_t stream, const char *what) {
  FPP_TRY(ensure_readback(st));
  FPP_CUDA(cudaMemcpyAsync(st.rb->status, st.status.ptr, sizeof(DeviceStatus),
                           cudaMemcpyDeviceToHost, stream));
  FPP_CUDA(cudaStreamSynchronize(stream));
  return status_from_readback(st, stream, what);
}

// The pair total, the slab overflow flag and the status word into the
// host-visible readback block (one thread).
__global__ void k_nb_readback(const int *__restrict__ total, const int *__restrict__ flags,
                              const DeviceStatus *__restrict__ status,
                              HostReadback *__restrict__ rb) {
  if (threadIdx.x != 0) return;
  rb->total_pairs = *total;
  rb->overflow = flags[0];
  rb->status[0] = status->code;
  rb->status[1] = status->where;
  rb->status[2] = status->info;
  rb->status[3] = status->pad;
}

// Pairs the pair buffers hold (0 before the first build; the FP64 table,
// filled on demand, counts too).
static long long pair_capacity(const StructureState &st) {
  if (!st.nbr_key.ptr || !st.nbr_i.ptr || !st.nbr_j.ptr || !st.nbr_s.ptr ||
      !st.nbr_rel.ptr || !st.nbr_rel32.ptr || !st.nbr_rev.ptr)
    return 0;
  size_t c = st.nbr_key.bytes / sizeof(long long);
  c = std::min(c, st.nbr_rel.bytes / sizeof(dvec4));
  c = std::min(c, st.nbr_i.bytes / sizeof(int));
  c = std::min(c, st.nbr_j.bytes / sizeof(int));
  c = std::min(c, st.nbr_s.bytes / sizeof(int));
  c = std::min(c, st.nbr_rel32.bytes / sizeof(float4));
  c = std::min(c, st.nbr_rev.bytes / sizeof(int));
  return (long long)c;
}

int build_neighbors(StructureState &st, cudaStream_t stream) {
  const int noa = st.noa;
  CellDev cd = make_dev(st.ci);
  const int nbins = st.ci.nb[0] * st.ci.nb[1] * st.ci.nb[2];
  if (!st.status.ptr) {
    FPP_TRY(st.status.reserve(sizeof(DeviceStatus)));
    FPP_CUDA(cudaMemsetAsync(st.status.ptr, 0, sizeof(DeviceStatus), stream));
  }
  FPP_TRY(st.nbr_count.reserve(sizeof(int) * (noa + 1)));
  FPP_TRY(st.nbr_offset.reserve(sizeof(int) * (noa + 1)));
  if (noa == 0) {
    st.n_pairs = 0;
    FPP_CUDA(cudaMemsetAsync(st.nbr_offset.ptr, 0, sizeof(int), stream));
    return FPP_OK;
  }
  FPP_TRY(st.wrapped.reserve(sizeof(dvec4) * noa));
  FPP_TRY(st.wrapped32.reserve(sizeof(float4) * noa));
  FPP_TRY(st.wrapped_lo.reserve(sizeof(float4) * noa));
  st.rel64_valid = false;
  FPP_TRY(st.frac.reserve(sizeof(float4) * noa));
  FPP_TRY(st.atom_bin.reserve(sizeof(int) * noa));
  FPP_TRY(st.bin_atoms.reserve(sizeof(int) * noa));
  FPP_TRY(st.bin_count.reserve(sizeof(int) * (nbins + 1)));
  FPP_TRY(st.bin_start.reserve(sizeof(int) * (nbins + 1)));
  FPP_TRY(st.bin_cursor.reserve(sizeof(int) * nbins));
  FPP_CUDA(cudaMemsetAsync(st.bin_count.ptr, 0, sizeof(int) * (nbins + 1), stream));
  FPP_CUDA(cudaMemsetAsync(st.bin_cursor.ptr, 0, sizeof(int) * nbins, stream));
  DeviceStatus *dst = st.status.as<DeviceStatus>();

  const int tb = 256;
  k_wrap_bin<<<ceil_div(noa, tb), tb, 0, stream>>>(
      noa, st.positions.as<double>(), cd, st.wrapped.as<dvec4>(),
      st.wrapped32.as<float4>(), st.wrapped_lo.as<float4>(), st.frac.as<float4>(),
      st.atom_bin.as<int>(),
      st.bin_count.as<int>(), dst);
  FPP_CUDA(cudaGetLastError());

  size_t tmp_bytes = 0, t2 = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, st.bin_count.as<int>(),
                                st.bin_start.as<int>(), nbins + 1, stream);
  cub::DeviceScan::ExclusiveSum(nullptr, t2, st.nbr_count.as<int>(),
                                st.nbr_offset.as<int>(), noa + 1, stream);
  FPP_TRY(st.scan_tmp.reserve(std::max(tmp_bytes, t2)));
  tmp_bytes = st.scan_tmp.bytes;
  FPP_CUDA(cub::DeviceScan::ExclusiveSum(st.scan_tmp.ptr, tmp_bytes,
                                         st.bin_count.as<int>(),
                                         st.bin_start.as<int>(), nbins + 1, stream));
  FPP_TRY(st.binned.reserve(sizeof(float4) * noa));
  k_bin_scatter<<<ceil_div(noa, tb), tb, 0, stream>>>(
      noa, st.atom_bin.as<int>(), st.bin_start.as<int>(), st.bin_cursor.as<int>(),
      st.bin_atoms.as<int>(), st.wrapped32.as<float4>(), st.binned.as<float4>());
  FPP_CUDA(cudaGetLastError());

  const int wpb = 4;  // warps per block, one atom per warp
  dim3 grid(ceil_div(noa, wpb)), block(32 * wpb);
  FPP_CUDA(cudaMemsetAsync(st.nbr_count.as<int>() + noa, 0, sizeof(int), stream));
  // single pass into the per-atom slab
  FPP_TRY(st.slab.reserve(sizeof(long long) * (size_t)noa * kSlabCap));
  FPP_TRY(st.flags.reserve(sizeof(int) * 4));
  FPP_CUDA(cudaMemsetAsync(st.flags.ptr, 0, sizeof(int) * 4, stream));
  k_enum<<<ceil_div(noa, kEnumWarps), 32 * kEnumWarps, 0, stream>>>(
      noa, cd, st.wrapped.as<dvec4>(), st.wrapped32.as<float4>(), st.wrapped_lo.as<float4>(),
      st.frac.as<float4>(), st.bin_start.as<int>(), st.binned.as<float4>(),
      st.nbr_count.as<int>(),
      st.slab.as<long long>(), st.flags.as<int>());
  FPP_CUDA(cudaGetLastError());
  tmp_bytes = st.scan_tmp.bytes;
  FPP_CUDA(cub::DeviceScan::ExclusiveSum(st.scan_tmp.ptr, tmp_bytes,
                                         st.nbr_count.as<int>(),
                                         st.nbr_offset.as<int>(), noa + 1, stream));
  FPP_TRY(ensure_readback(st));
  k_nb_readback<<<1, 32, 0, stream>>>(st.nbr_offset.as<int>() + noa, st.flags.as<int>(),
                                      st.status.as<DeviceStatus>(), st.rb_dev);
  FPP_CUDA(cudaGetLastError());
  if (!st.nb_ready) FPP_CUDA(cudaEventCreateWithFlags(&st.nb_ready, cudaEventDisableTiming));
  FPP_CUDA(cudaEventRecord(st.nb_ready, stream));
  // the compaction into the pair buffers of an earlier build, queued before
  // the host waits for the pair total so that the GPU has work meanwhile; it
  // writes nothing (and is launched again below) when the slab overflowed or
  // the buffers are too small
  const long long cap = pair_capacity(st);
  if (cap > 0) {
    k_compact_geom<<<grid, block, 0, stream>>>(
        noa, cd, st.wrapped32.as<float4>(), st.wrapped_lo.as<float4>(), st.species.as<int>(),
        st.nbr_offset.as<int>(), st.slab.as<long long>(), st.nbr_key.as<long long>(),
        st.nbr_i.as<int>(), st.nbr_j.as<int>(), st.nbr_s.as<int>(),
        st.nbr_rel32.as<float4>(), st.nbr_rev.as<int>(), dst, cap, st.flags.as<int>());
    FPP_CUDA(cudaGetLastError());
  }
  FPP_CUDA(cudaEventSynchronize(st.nb_ready));
  FPP_TRY(status_from_readback(st, stream, "neighbor build or an earlier asynchronous call"));
  const bool overflow = st.rb->overflow != 0;
  int total = st.rb->total_pairs;
  if (overflow) {
    // some atom has more than kSlabCap neighbors: two-pass count / fill
    k_count<<<grid, block, 0, stream>>>(noa, cd, st.wrapped.as<dvec4>(),
                                        st.wrapped32.as<float4>(), st.frac.as<float4>(),
                                        st.bin_start.as<int>(), st.bin_atoms.as<int>(),
                                        st.nbr_count.as<int>());
    FPP_CUDA(cudaGetLastError());
    tmp_bytes = st.scan_tmp.bytes;
    FPP_CUDA(cub::DeviceScan::ExclusiveSum(st.scan_tmp.ptr, tmp_bytes,
                                           st.nbr_count.as<int>(),
                                           st.nbr_offset.as<int>(), noa + 1, stream));
    FPP_CUDA(cudaMemcpyAsync(&total, st.nbr_offset.as<int>() + noa, sizeof(int),
                             cudaMemcpyDeviceToHost, stream));
    FPP_CUDA(cudaStreamSynchronize(stream));
  }
  if (total < 0) return fail(FPP_ERR_CAPACITY, "more than 2^31 neighbor pairs");
  st.n_pairs = total;
  const bool compacted = !overflow && (long long)total <= cap;
  // an eighth of headroom, so that a pair total that grows a little from one
  // build to the next stays within the buffers
  const size_t np = (size_t)std::max(total, 1) + (size_t)total / 8;
  if (!compacted) {
    // the queued compaction (which wrote nothing) may still hold the buffers
    if (cap > 0) FPP_CUDA(cudaStreamSynchronize(stream));
    FPP_TRY(st.nbr_key.reserve(sizeof(long long) * np));
    FPP_TRY(st.nbr_i.reserve(sizeof(int) * np));
    FPP_TRY(st.nbr_j.reserve(sizeof(int) * np));
    FPP_TRY(st.nbr_s.reserve(sizeof(int) * np));
    FPP_TRY(st.nbr_rel.reserve(sizeof(dvec4) * np));
    FPP_TRY(st.nbr_rel32.reserve(sizeof(float4) * np));
    FPP_TRY(st.nbr_rev.reserve(sizeof(int) * np));
  }
  // read by later kernels through mapped memory; no kernel in flight reads it
  // (the queued compaction does not)
  st.rb->geom = nb_geom(st);
  if (total == 0) return FPP_OK;
  if (!overflow) {
    if (!compacted) {
      k_compact_geom<<<grid, block, 0, stream>>>(
          noa, cd, st.wrapped32.as<float4>(), st.wrapped_lo.as<float4>(), st.species.as<int>(),
          st.nbr_offset.as<int>(), st.slab.as<long long>(), st.nbr_key.as<long long>(),
          st.nbr_i.as<int>(), st.nbr_j.as<int>(), st.nbr_s.as<int>(),
          st.nbr_rel32.as<float4>(), st.nbr_rev.as<int>(), dst, (long long)total,
          st.flags.as<int>());
      FPP_CUDA(cudaGetLastError());
    }
    return FPP_OK;  // reverse links and mirrored geometry written above
  } else {
    FPP_TRY(st.nbr_key_tmp.reserve(sizeof(long long) * np));
    k_fill<<<grid, block, 0, stream>>>(noa, cd, st.wrapped.as<dvec4>(),
                                       st.wrapped32.as<float4>(), st.frac.as<float4>(),
                                       st.bin_start.as<int>(), st.bin_atoms.as<int>(),
                                       st.nbr_offset.as<int>(),
                                       st.nbr_key_tmp.as<long long>());
    FPP_CUDA(cudaGetLastError());
    k_sort_geom<<<grid, block, 0, stream>>>(
        noa, cd, st.wrapped.as<dvec4>(), st.species.as<int>(),
        st.nbr_offset.as<int>(), st.nbr_key_tmp.as<long long>(),
        st.nbr_key.as<long long>(), st.nbr_i.as<int>(), st.nbr_j.as<int>(),
        st.nbr_s.as<int>(), st.nbr_rel.as<dvec4>(), st.nbr_rel32.as<float4>());
    FPP_CUDA(cudaGetLastError());
    st.rel64_valid = true;  // this build computes the FP64 table for every pair
  }
  k_reverse<<<ceil_div(total, tb), tb, 0, stream>>>(
      total, cd, st.nbr_offset.as<int>(), st.nbr_key.as<long long>(),
      st.nbr_i.as<int>(), st.nbr_j.as<int>(), st.nbr_rev.as<int>(), dst);
  FPP_CUDA(cudaGetLastError());
  return FPP_OK;
}

int ensure_rel64(StructureState &st, cudaStream_t stream) {
  if (st.rel64_valid || st.n_pairs == 0) {
    st.rel64_valid = true;
    return FPP_OK;
  }
  const CellDev cd = make_dev(st.ci);
  k_rel64<<<ceil_div((int)st.n_pairs, 256), 256, 0, stream>>>(
      st.n_pairs, cd, st.wrapped.as<dvec4>(), st.nbr_key.as<long long>(),
      st.nbr_i.as<int>(), st.nbr_rel.as<dvec4>());
  FPP_CUDA(cudaGetLastError());
  st.rel64_valid = true;
  return FPP_OK;
}

// ---------------------------------------------------------------------------
// Neighbor reuse within a skin.  The list was built at cutoff + skin from the
// positions x_b (wrapped w_b); for new positions x with max |x - x_b| <= skin/2
// every pair within the cutoff is still in it.  The pair keys (j, shift) stay
// valid when the positions are not re-wrapped, so the wrapped positions become
// w = w_b + (x - x_b) and every pair vector is recomputed from them with the
// build's float-float image formula; the FP64 table follows on demand
// (ensure_rel64, the reference's image formula on w).
// ---------------------------------------------------------------------------
__global__ void k_max_disp2(int noa, const double *__restrict__ pos,
                            const double *__restrict__ pos_b,
                            unsigned long long *__restrict__ out) {
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < noa; i += gridDim.x * blockDim.x) {
    const double dx = pos[3 * i] - pos_b[3 * i], dy = pos[3 * i + 1] - pos_b[3 * i + 1],
                 dz = pos[3 * i + 2] - pos_b[3 * i + 2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    m = (d2 > m || d2 != d2) ? d2 : m;  // a NaN propagates (forces a rebuild)
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, m, o);
    m = (v > m || v != v) ? v : m;
  }
  // non-negative doubles (and NaN) order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_refresh_wrapped(int noa, const double *__restrict__ pos,
                                  const double *__restrict__ pos_b,
                                  const dvec4 *__restrict__ wp_b, dvec4 *__restrict__ wp,
                                  float4 *__restrict__ wp32, float4 *__restrict__ wp_lo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= noa) return;
  const dvec4 b = wp_b[i];
  const double w[3] = {dadd(b.x, dsub(pos[3 * i], pos_b[3 * i])),
                       dadd(b.y, dsub(pos[3 * i + 1], pos_b[3 * i + 1])),
                       dadd(b.z, dsub(pos[3 * i + 2], pos_b[3 * i + 2]))};
  wp[i] = dvec4{w[0], w[1], w[2], 0.0};
  const float4 h = make_float4((float)w[0], (float)w[1], (float)w[2], 0.f);
  wp32[i] = h;
  wp_lo[i] = make_float4((float)(w[0] - (double)h.x), (float)(w[1] - (double)h.y),
                         (float)(w[2] - (double)h.z), 0.f);
}

// The canonical half of the pairs (key above (i, centre shift)) computes its
// float-float vector and writes it, negated, to its reverse pair as well, as
// the build does.
__global__ void k_refresh_rel32(long long n_pairs, CellDev cd, const float4 *__restrict__ wp32,
                                const float4 *__restrict__ wp_lo,
                                const long long *__restrict__ keys,
                                const int *__restrict__ nbr_i, const int *__restrict__ rev,
                                float4 *__restrict__ rel32) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const int i = nbr_i[p];
  const long long key = keys[p];
  const long long thr = ((long long)i << kKeyBits) |
                        ((cd.sweep * cd.ns + cd.sweep) * cd.ns + cd.sweep);
  if (key <= thr) return;
  const int j = (int)(key >> kKeyBits);
  int s1, s2, s3;
  decode_shift((int)(key & kKeyMask), cd.ns, cd.sweep, s1, s2, s3);
  ff im[3], r2;
  image_ff(wp32[i], wp_lo[i], wp32[j], wp_lo[j], cd.cff, s1, s2, s3, im, r2);
  const float4 v = make_float4(im[0].hi + im[0].lo, im[1].hi + im[1].lo, im[2].hi + im[2].lo,
                               ff_sqrt_f(r2));
  rel32[p] = v;
  const int q = rev[p];
  if (q >= 0) rel32[q] = make_float4(-v.x, -v.y, -v.z, v.w);
}

// New positions (already in st.positions): refresh the geometry of the list
// when no atom has moved more than skin / 2 since its build, else rebuild.
// Sets *reused.
int update_neighbors(StructureState &st, cudaStream_t stream, bool *reused) {
  *reused = false;
  const int noa = st.noa;
  if (st.skin > 0 && st.have_build && noa > 0) {
    FPP_TRY(st.disp_max.reserve(sizeof(unsigned long long)));
    FPP_CUDA(cudaMemsetAsync(st.disp_max.ptr, 0, sizeof(unsigned long long), stream));
    const int tb = 256, blocks = std::min(ceil_div(noa, tb), 4 * 152);
    k_max_disp2<<<blocks, tb, 0, stream>>>(noa, st.positions.as<double>(),
                                            st.pos_build.as<double>(),
                                            st.disp_max.as<unsigned long long>());
    FPP_CUDA(cudaGetLastError());
    unsigned long long bits = 0;
    FPP_CUDA(cudaMemcpyAsync(&bits, st.disp_max.ptr, sizeof(bits), cudaMemcpyDeviceToHost,
                             stream));
    FPP_CUDA(cudaStreamSynchronize(stream));
    double d2;
    std::memcpy(&d2, &bits, sizeof(d2));
    if (d2 == d2 && 4.0 * d2 <= st.skin * st.skin) {
      const CellDev cd = make_dev(st.ci);
      k_refresh_wrapped<<<ceil_div(noa, tb), tb, 0, stream>>>(
          noa, st.positions.as<double>(), st.pos_build.as<double>(),
          st.wrapped_build.as<dvec4>(), st.wrapped.as<dvec4>(), st.wrapped32.as<float4>(),
          st.wrapped_lo.as<float4>());
      FPP_CUDA(cudaGetLastError());
      if (st.n_pairs > 0) {
        k_refresh_rel32<<<(int)((st.n_pairs + tb - 1) / tb), tb, 0, stream>>>(
            st.n_pairs, cd, st.wrapped32.as<float4>(), st.wrapped_lo.as<float4>(),
            st.nbr_key.as<long long>(), st.nbr_i.as<int>(), st.nbr_rev.as<int>(),
            st.nbr_rel32.as<float4>());
        FPP_CUDA(cudaGetLastError());
      }
      st.rel64_valid = false;
      st.n_reuses++;
      *reused = true;
      return FPP_OK;
    }
  }
  FPP_TRY(build_neighbors(st, stream));
  st.n_builds++;
  st.have_build = false;
  if (st.skin > 0 && noa > 0) {
    FPP_TRY(st.pos_build.reserve(sizeof(double) * 3 * noa));
    FPP_TRY(st.wrapped_build.reserve(sizeof(dvec4) * noa));
    FPP_CUDA(cudaMemcpyAsync(st.pos_build.ptr, st.positions.ptr, sizeof(double) * 3 * noa,
                             cudaMemcpyDeviceToDevice, stream));
    FPP_CUDA(cudaMemcpyAsync(st.wrapped_build.ptr, st.wrapped.ptr, sizeof(dvec4) * noa,
                             cudaMemcpyDeviceToDevice, stream));
    st.have_build = true;
  }
  return FPP_OK;
}

}  // namespace fpp
