// FP64-accurate C = A B^T on the fp16 tensor cores (tcgen05), by exact
// integer slices (the splitting scheme of Ozaki, Ogita, Oishi and Rump,
// "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applications", Numer. Algorithms 59, 2012).
//
// Each row of A (and of B) is scaled by a power of two 2^e so that its
// entries lie in (-1, 1), then cut into kOzakiDigits signed digits of
// kOzakiBits bits:  a = 2^e sum_s d_s 2^(-5 (s + 1)),  |d_s| <= 31,
// which fp16 holds exactly.  For one pair of digit planes (s, t) the products
// d_s d_t are integers of at most 961 and a K-sum of them stays an integer; all
// the pairs of one level L = s + t summed over at most kOzakiChunkK columns
// stay below 11 * 1536 * 961 < 2^24, so the FP32 TMEM accumulator holds them
// EXACTLY whatever order or truncation the tensor cores use.  The epilogue
// adds each level into C in FP64:
//   C = 2^(e_a + e_b) sum_{L <= 10} 2^(-5 (L + 2)) (sum_{s + t = L} A_s B_t^T),
// which keeps about 55 bits of every operand relative to its row's largest
// entry (the pairs of levels 11 and above, dropped, weigh below 2^-55 of it).
//
// Kernel layout (one persistent CTA per SM, 320 threads):
//   warp 0 lane 0  TMA producer: 128B-swizzled 128 x 64 tiles of the A and B
//                  digit planes into a 6-stage ring
//   warp 1 lane 0  MMA issuer: per unit (tile, level, K chunk) the pairs of
//                  the level into one 128-column TMEM accumulator; four
//                  accumulators rotate between units
//   warps 2-9      epilogue: two warps per TMEM lane quarter, each owning 64
//                  columns of its 32 rows: tcgen05.ld, then the level times
//                  2^(-5 (L + 2)) added to FP64 sums held in registers for the
//                  whole tile; after the last level the row and column powers
//                  of two are applied and the tile is stored once
// Every wait is bounded; a wait that runs out records FPP_ERR_TIMEOUT in the
// status word and the CTA skips to its exit.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "gemm_ozaki.h"
#include "tc_prims.cuh"

namespace fpp {

namespace {
constexpr int OBM = 128, OBN = 128, OBK = kTmaBoxK, OSTAGES = 6;
constexpr int OA_TILE = OBM * OBK * 2, OB_TILE = OBN * OBK * 2;
constexpr int OSTAGE_BYTES = OA_TILE + OB_TILE;
constexpr int OACC = 4;                 // TMEM accumulators (units in flight)
constexpr int OTMEM_COLS = OACC * OBN;
constexpr int OEPI = 8;                 // epilogue warps
constexpr int OTHREADS = 32 * (2 + OEPI);
constexpr int OSMEM_BYTES = OSTAGES * OSTAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int kChunkBlocks = kOzakiChunkK / OBK;
static_assert(kOzakiChunkK % OBK == 0, "K chunks are whole TMA boxes");
// exactness of one level's sum: (pairs per level) * chunk * 31^2 < 2^24
static_assert((long long)kOzakiDigits * kOzakiChunkK * 961 < (1ll << 24),
              "a level's integer sum must fit the FP32 significand");
}  // namespace

struct OzakiParams {
  CUtensorMap a, b;          // digit planes: rows s * Mp + m (s * Np + n), inner Kp
  int M, N, Mp, Np;
  int kblocks, n_chunks, tiles_n, n_tiles;
  int b_lower;               // B lower triangular: tile n0 needs K < n0 + OBN only
  const double *pa, *pb;     // 2^e of each row of A and of B
  double *C;
  long long ldc;
  DeviceStatus *status;
};

__global__ void __launch_bounds__(OTHREADS, 1)
k_ozaki_gemm(const __grid_constant__ OzakiParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *gbase = smem_raw + (base - raw);
  const uint32_t bars = base + OSTAGES * OSTAGE_BYTES;
  uint64_t *bar_ptr = reinterpret_cast<uint64_t *>(gbase + OSTAGES * OSTAGE_BYTES);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_ptr + 2 * OSTAGES + 2 * OACC);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (OSTAGES + s); };
  auto accf_bar = [&](int b) { return bars + 8u * (2 * OSTAGES + b); };
  auto acce_bar = [&](int b) { return bars + 8u * (2 * OSTAGES + OACC + b); };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cid = (int)blockIdx.x, ncta = (int)gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < OSTAGES; s++) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < OACC; b++) {
      mbar_init(accf_bar(b), 1);
      mbar_init(acce_bar(b), OEPI);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(OTMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // K blocks and chunks of a tile: all of K, or with a lower-triangular B
  // (row n of B is zero beyond column n) only the blocks below n0 + OBN
  auto tile_kb = [&](int t) {
    if (!p.b_lower) return p.kblocks;
    const int n0 = (t % p.tiles_n) * OBN;
    const int e = (n0 + OBN + OBK - 1) / OBK;
    return e < p.kblocks ? e : p.kblocks;
  };
  auto n_chunks_of = [&](int kbt) { return (kbt + kChunkBlocks - 1) / kChunkBlocks; };

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    int it = 0;
    bool stop = false;
    for (int t = cid; t < p.n_tiles && !stop; t += ncta) {
      const int mrow = (t / p.tiles_n) * OBM, n0 = (t % p.tiles_n) * OBN;
      const int kbt = tile_kb(t), nch = n_chunks_of(kbt);
      for (int L = 0; L < kOzakiDigits && !stop; L++)
        for (int c = 0; c < nch && !stop; c++) {
          const int kb1 = min((c + 1) * kChunkBlocks, kbt);
          for (int s = 0; s <= L && !stop; s++)
            for (int kb = c * kChunkBlocks; kb < kb1; kb++, it++) {
              const int st = it % OSTAGES;
              const uint32_t ph = (uint32_t)((it / OSTAGES) & 1);
              if (!mbar_wait(empty_bar(st), ph ^ 1u)) {
                set_status(p.status, FPP_ERR_TIMEOUT, 211, t);
                *abort_flag = 1;
              }
              if (*abort_flag) {
                stop = true;
                break;
              }
              const uint32_t sa = base + st * OSTAGE_BYTES;
              mbar_expect_tx(full_bar(st), OSTAGE_BYTES);
              tma_load_2d(sa, &p.a, full_bar(st), kb * OBK, s * p.Mp + mrow);
              tma_load_2d(sa + OA_TILE, &p.b, full_bar(st), kb * OBK, (L - s) * p.Np + n0);
            }
        }
    }
    // drain: every stage this CTA filled has been read before it exits
    for (int d = 0; d < OSTAGES && !*abort_flag; d++, it++) {
      if (!mbar_wait(empty_bar(it % OSTAGES), (uint32_t)(((it / OSTAGES) & 1) ^ 1))) {
        set_status(p.status, FPP_ERR_TIMEOUT, 215, d);
        *abort_flag = 1;
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    int it = 0, j = 0;
    bool stop = false;
    for (int t = cid; t < p.n_tiles && !stop; t += ncta) {
      const int kbt = tile_kb(t), nch = n_chunks_of(kbt);
      for (int L = 0; L < kOzakiDigits && !stop; L++)
        for (int c = 0; c < nch && !stop; c++, j++) {
          const int kb1 = min((c + 1) * kChunkBlocks, kbt);
          const int buf = j % OACC;
          const uint32_t acc = tmem + (uint32_t)(buf * OBN);
          if (!mbar_wait(acce_bar(buf), (uint32_t)(((j / OACC) & 1) ^ 1))) {
            set_status(p.status, FPP_ERR_TIMEOUT, 212, t);
            *abort_flag = 1;
          }
          if (*abort_flag) {
            mma_commit(accf_bar(buf));  // release the epilogue of this buffer
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          bool first = true;
          for (int s = 0; s <= L && !stop; s++)
            for (int kb = c * kChunkBlocks; kb < kb1; kb++, it++) {
              const int st = it % OSTAGES;
              const uint32_t ph = (uint32_t)((it / OSTAGES) & 1);
              if (!mbar_wait(full_bar(st), ph)) {
                set_status(p.status, FPP_ERR_TIMEOUT, 213, t);
                *abort_flag = 1;
                stop = true;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
              const uint32_t sa = base + st * OSTAGE_BYTES, sb = sa + OA_TILE;
#pragma unroll
              for (int ks = 0; ks < OBK / 16; ks++) {
                const uint32_t off = ks * 32;
                mma_f16<OBN>(acc, smem_desc(sa + off), smem_desc(sb + off),
                             (first && ks == 0) ? 0u : 1u);
              }
              first = false;
              mma_commit(empty_bar(st));  // frees the stage once these MMAs read it
            }
          mma_commit(accf_bar(buf));
        }
    }
  } else if (warp >= 2) {
    // ---------------- epilogue ----------------
    const int q = warp & 3;                 // TMEM lane quarter this warp may access
    const int half = (warp - 2) / 4;        // which 64 columns of the tile
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    int j = 0;
    bool stop = false;
    for (int t = cid; t < p.n_tiles && !stop; t += ncta) {
      const int mrow = (t / p.tiles_n) * OBM, n0 = (t % p.tiles_n) * OBN + half * 64;
      const int r = mrow + q * 32 + lane;
      const int nch = n_chunks_of(tile_kb(t));
      double acc[64];
#pragma unroll
      for (int i = 0; i < 64; i++) acc[i] = 0.0;
      for (int L = 0; L < kOzakiDigits && !stop; L++) {
        // 2^(-5 (L + 2)), exact
        const double sL = __longlong_as_double((long long)(1023 - 5 * (L + 2)) << 52);
        for (int c = 0; c < nch; c++, j++) {
          const int buf = j % OACC;
          bool have = mbar_wait(accf_bar(buf), (uint32_t)((j / OACC) & 1));
          have = __all_sync(0xffffffffu, have) != 0;
          if (!have) {
            if (lane == 0) set_status(p.status, FPP_ERR_TIMEOUT, 214, t);
            *abort_flag = 1;
            stop = true;
            break;
          }
          if (__shfl_sync(0xffffffffu, *abort_flag, 0)) {
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t tm = tmem + (uint32_t)(buf * OBN + half * 64) + lane_base;
          float v[32];
          tmem_ld32(tm, v);
#pragma unroll
          for (int i = 0; i < 32; i++) acc[i] = fma((double)v[i], sL, acc[i]);
          tmem_ld32(tm + 32, v);
#pragma unroll
          for (int i = 0; i < 32; i++) acc[32 + i] = fma((double)v[i], sL, acc[32 + i]);
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(acce_bar(buf));
        }
      }
      if (stop || r >= p.M) continue;
      const double pr = p.pa[r];
      double *crow = p.C + (size_t)r * p.ldc + n0;
#pragma unroll
      for (int i = 0; i < 64; i++)
        if (n0 + i < p.N) crow[i] = acc[i] * pr * p.pb[n0 + i];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 2) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(OTMEM_COLS)
                 : "memory");
  }
}

// Digit planes of the rows of X (rows x K, leading dimension ldx): a warp per
// row; rows >= rows and columns >= K of the padded planes are written as zeros.
__global__ void __launch_bounds__(256)
k_ozaki_split(int rows, int K, long long ldx, const double *__restrict__ X, int rows_pad,
              int k_pad, __half *__restrict__ planes, double *__restrict__ p2) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= rows_pad) return;
  const int r = warp;
  const size_t plane = (size_t)rows_pad * k_pad;
  __half *dst = planes + (size_t)r * k_pad;
  if (r >= rows) {
    for (int k = lane; k < k_pad; k += 32)
      for (int s = 0; s < kOzakiDigits; s++) dst[s * plane + k] = __float2half_rn(0.0f);
    return;
  }
  const double *x = X + (size_t)r * ldx;
  double mx = 0.0;
  for (int k = lane; k < K; k += 32) mx = fmax(mx, fabs(x[k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  // the row's power of two: max |x| < 2^e (e = 0 for an all-zero row)
  int e = 0;
  if (mx > 0.0) frexp(mx, &e);
  if (lane == 0) p2[r] = ldexp(1.0, e);
  const double inv = ldexp(1.0, -e);
  // 55-bit fixed point of |x| 2^-e (exact scaling; truncation below 2^-55)
  const double two55 = 36028797018963968.0;
  for (int k = lane; k < k_pad; k += 32) {
    const double v = k < K ? x[k] : 0.0;
    const unsigned long long X55 = __double2ull_rz(fabs(v) * inv * two55);
    const bool neg = v < 0.0;
#pragma unroll
    for (int s = 0; s < kOzakiDigits; s++) {
      const int d = (int)((X55 >> (kOzakiBits * (kOzakiDigits - 1 - s))) & 31ull);
      dst[s * plane + k] = __int2half_rn(neg ? -d : d);
    }
  }
}

static int ozaki_launch_shape(int dev, int *ctas) {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static int cached[kMaxDev] = {0};
  if (dev < 0 || dev >= kMaxDev) return -1;
  std::lock_guard<std::mutex> lock(mu);
  if (cached[dev] == 0) {
    if (cudaFuncSetAttribute(k_ozaki_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             OSMEM_BYTES) != cudaSuccess)
      return -1;
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ozaki_gemm, OTHREADS,
                                                      OSMEM_BYTES) != cudaSuccess)
      return -1;
    if (per_sm < 1) return -1;
    cached[dev] = sms * per_sm;
  }
  *ctas = cached[dev];
  return 0;
}

OzakiShape ozaki_shape(int rows, int K) {
  OzakiShape s;
  s.rows_pad = (rows + OBM - 1) / OBM * OBM;
  s.k_pad = (K + OBK - 1) / OBK * OBK;
  s.plane_bytes = (size_t)s.rows_pad * s.k_pad * sizeof(__half) * kOzakiDigits;
  return s;
}

int launch_ozaki_split(int rows, int K, const double *X, long long ldx, __half *planes,
                       double *p2, cudaStream_t stream) {
  if (rows <= 0) return 0;
  const OzakiShape sh = ozaki_shape(rows, K);
  const int threads = 256;
  const long long warps = sh.rows_pad;
  const int blocks = (int)((warps * 32 + threads - 1) / threads);
  k_ozaki_split<<<blocks, threads, 0, stream>>>(rows, K, ldx, X, sh.rows_pad, sh.k_pad,
                                                 planes, p2);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_ozaki_gemm(int M, int N, int K, const __half *a_planes, const double *pa,
                      const __half *b_planes, const double *pb, double *C, long long ldc,
                      DeviceStatus *status, cudaStream_t stream, bool b_lower) {
  if (M <= 0 || N <= 0) return 0;
  if (K <= 0) return -2;
  const OzakiShape sa = ozaki_shape(M, K), sb = ozaki_shape(N, K);
  if (((uintptr_t)a_planes | (uintptr_t)b_planes) % 16 != 0 || ldc < N) return -2;
  OzakiParams p;
  std::memset(&p, 0, sizeof(p));
  // one map over all digit planes of an operand: rows s * rows_pad + row
  if (make_map(&p.a, a_planes, sa.k_pad, sa.rows_pad * kOzakiDigits, sa.k_pad, OBM) ||
      make_map(&p.b, b_planes, sb.k_pad, sb.rows_pad * kOzakiDigits, sb.k_pad, OBN))
    return -3;
  p.M = M;
  p.N = N;
  p.Mp = sa.rows_pad;
  p.Np = sb.rows_pad;
  p.kblocks = sa.k_pad / OBK;
  p.n_chunks = (p.kblocks + kChunkBlocks - 1) / kChunkBlocks;
  p.b_lower = b_lower ? 1 : 0;
  p.tiles_n = (N + OBN - 1) / OBN;
  p.n_tiles = (sa.rows_pad / OBM) * p.tiles_n;
  p.pa = pa;
  p.pb = pb;
  p.C = C;
  p.ldc = ldc;
  p.status = status;
  int dev = 0, ctas = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || ozaki_launch_shape(dev, &ctas) != 0) return -1;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.blockDim = dim3(OTHREADS, 1, 1);
  cfg.dynamicSmemBytes = OSMEM_BYTES;
  cfg.stream = stream;
  cfg.gridDim = dim3(p.n_tiles < ctas ? p.n_tiles : ctas, 1, 1);
  if (cudaLaunchKernelEx(&cfg, k_ozaki_gemm, p) != cudaSuccess) return -1;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace fpp
