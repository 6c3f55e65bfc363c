// Split-fp16 contraction on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   V[m, n] = sum_k P[m, k] B[n, k]
// with both operands given as power-of-two-scaled fp16 pairs
//   P ~ (P_hi + P_lo / 2048) / sP,   B ~ (B_hi + B_lo / 2048) / sB,
// evaluated as three MMAs into two FP32 accumulators held in TMEM:
//   acc0 += P_hi B_hi^T,   acc1 += P_hi B_lo^T + P_lo B_hi^T,
//   V = (acc0 + acc1 / 2048) / (sP sB).
// That keeps about 22 significant bits per operand, which the mapped-beta
// energy needs (a single fp16 or bf16 term, or a bf16 hi/lo split, does not).
// The cross terms have their own accumulator: added into the leading one they
// would each round against its magnitude (measured: 1.6x the force error).
//
// One persistent CTA per SM walks the 128 x 128 tiles of all species blocks
// (each block of P rows against its own B), in one launch; every CTA loads
// all four operand planes of its own tile (no clusters):
//   warp 0 lane 0  TMA producer: 128B-swizzled K-major tiles of P_hi, P_lo,
//                  B_hi, B_lo (64 K-columns per stage) into a 3-stage ring
//   warp 1 lane 0  MMA issuer: 4 K=16 steps x 3 tcgen05.mma per stage,
//                  tcgen05.commit frees the stage; the two accumulator pairs
//                  (2 x 2 x 128 TMEM columns) alternate between tiles, so the
//                  epilogue of one tile overlaps the MMAs of the next
//   warps 2-5      epilogue: tcgen05.ld of their 32 TMEM lanes, combine,
//                  scale, store FP32 rows of V, then release the accumulators
// Every mbarrier wait is bounded; a wait that runs out records
// FPP_ERR_TIMEOUT in the status word and the CTA skips to its exit.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "gemm_tc.h"
#include "tc_prims.cuh"

namespace fpp {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 3;
static_assert(BK == kTmaBoxK, "the tensor maps load 64-column boxes");
constexpr int A_TILE = BM * BK * 2;  // bytes, one fp16 operand tile
constexpr int B_TILE = BN * BK * 2;
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr int TMEM_COLS = 512;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;

// ---------------------------------------------------------------------------
// Grouped persistent form (see the header comment).
// ---------------------------------------------------------------------------
struct GroupedParams {
  CUtensorMap a_hi, a_lo;
  CUtensorMap b_hi[kGemmMaxGroups], b_lo[kGemmMaxGroups];
  int row0[kGemmMaxGroups], M[kGemmMaxGroups];
  float scale[kGemmMaxGroups];
  int tile_start[kGemmMaxGroups + 1];  // work items (tiles) per group (prefix)
  int n_groups, tiles_n, N, K;          // tiles_n: column tiles per row tile
  float *V;
  int ldv;
  DeviceStatus *status;
};


__global__ void __launch_bounds__(192, 1)
k_split_gemm_grouped(const __grid_constant__ GroupedParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *gbase = smem_raw + (base - raw);
  const uint32_t bars = base + STAGES * STAGE_BYTES;
  uint64_t *bar_ptr = reinterpret_cast<uint64_t *>(gbase + STAGES * STAGE_BYTES);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_ptr + 2 * STAGES + 4);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (STAGES + s); };
  auto accf_bar = [&](int b) { return bars + 8u * (2 * STAGES + b); };
  auto acce_bar = [&](int b) { return bars + 8u * (2 * STAGES + 2 + b); };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tiles = p.tile_start[p.n_groups];
  const int kblocks = (p.K + BK - 1) / BK;
  const int cid = (int)blockIdx.x, ncl = (int)gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(accf_bar(b), 1);
      mbar_init(acce_bar(b), 4);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // work item (one 128 x 128 tile; consecutive items share a row tile, so the
  // CTAs running at once read each A tile from L2 rather than DRAM)
  // -> (group, row of the operand block, first column)
  auto locate = [&](int t, int &g, int &mrow, int &n0) {
    g = 0;
    while (g + 1 < p.n_groups && t >= p.tile_start[g + 1]) g++;
    const int lt = t - p.tile_start[g];
    mrow = (lt / p.tiles_n) * BM;
    n0 = (lt % p.tiles_n) * BN;
  };

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    int it = 0;
    for (int t = cid; t < n_tiles && !*abort_flag; t += ncl) {
      int g, mrow, n0;
      locate(t, g, mrow, n0);
      const int arow = p.row0[g] + mrow;
      for (int kb = 0; kb < kblocks; kb++, it++) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)((it / STAGES) & 1);
        if (!mbar_wait(empty_bar(s), ph ^ 1u)) {
          set_status(p.status, FPP_ERR_TIMEOUT, 111, t);
          *abort_flag = 1;
          break;
        }
        if (*abort_flag) break;
        const uint32_t st = base + s * STAGE_BYTES;
        mbar_expect_tx(full_bar(s), STAGE_BYTES);
        const int kc = kb * BK;
        tma_load_2d(st, &p.a_hi, full_bar(s), kc, arow);
        tma_load_2d(st + A_TILE, &p.a_lo, full_bar(s), kc, arow);
        tma_load_2d(st + 2 * A_TILE, &p.b_hi[g], full_bar(s), kc, n0);
        tma_load_2d(st + 2 * A_TILE + B_TILE, &p.b_lo[g], full_bar(s), kc, n0);
      }
    }
    // drain: every stage this CTA filled has been read (no MMA completion
    // arrival is still in flight at exit)
    for (int d = 0; d < STAGES && !*abort_flag; d++, it++) {
      if (!mbar_wait(empty_bar(it % STAGES), (uint32_t)(((it / STAGES) & 1) ^ 1))) {
        set_status(p.status, FPP_ERR_TIMEOUT, 115, d);
        *abort_flag = 1;
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    int it = 0, j = 0;
    for (int t = cid; t < n_tiles; t += ncl, j++) {
      const int buf = j & 1;
      const uint32_t acc0 = tmem + (uint32_t)(buf * 2 * BN), acc1 = acc0 + BN;
      if (!mbar_wait(acce_bar(buf), (uint32_t)(((j >> 1) & 1) ^ 1))) {
        set_status(p.status, FPP_ERR_TIMEOUT, 112, t);
        *abort_flag = 1;
      }
      if (*abort_flag) {
        mma_commit(accf_bar(buf));  // release the epilogue of this buffer
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      bool ok = true;
      for (int kb = 0; kb < kblocks; kb++, it++) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)((it / STAGES) & 1);
        if (!mbar_wait(full_bar(s), ph)) {
          set_status(p.status, FPP_ERR_TIMEOUT, 113, t);
          *abort_flag = 1;
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = base + s * STAGE_BYTES;
        const uint32_t a_hi = st, a_lo = st + A_TILE;
        const uint32_t b_hi = st + 2 * A_TILE;  // B_lo follows at + B_TILE
#pragma unroll
        for (int ks = 0; ks < BK / 16; ks++) {
          const uint32_t off = ks * 32;
          const uint32_t first = (kb > 0 || ks > 0) ? 1u : 0u;
          // B_hi and B_lo are one 256-row operand in shared memory and acc0,
          // acc1 adjacent TMEM columns: [acc0 | acc1] = A_hi [B_hi ; B_lo]^T
          // in one N = 256 MMA, then acc1 += A_lo B_hi^T.  Shared-memory
          // reads per K step fall from 24 KB to 20 KB (the operand reads and
          // the TMA writes share the SM's shared-memory bandwidth).
          mma_f16<2 * BN>(acc0, smem_desc(a_hi + off), smem_desc(b_hi + off), first);
          mma_f16<BN>(acc1, smem_desc(a_lo + off), smem_desc(b_hi + off), 1u);
        }
        mma_commit(empty_bar(s));  // frees the stage once these MMAs have read it
      }
      mma_commit(accf_bar(buf));
      if (!ok) break;
    }
  } else if (warp >= 2) {
    // ---------------- epilogue ----------------
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    int j = 0;
    for (int t = cid; t < n_tiles; t += ncl, j++) {
      const int buf = j & 1;
      bool have = mbar_wait(accf_bar(buf), (uint32_t)((j >> 1) & 1));
      have = __all_sync(0xffffffffu, have) != 0;
      if (!have) {
        if (lane == 0) set_status(p.status, FPP_ERR_TIMEOUT, 114, t);
        *abort_flag = 1;
        break;
      }
      if (__shfl_sync(0xffffffffu, *abort_flag, 0)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int g, mrow, n0;
      locate(t, g, mrow, n0);
      const int r = mrow + q * 32 + lane;  // row within the group
      const float sc = p.scale[g];
      const uint32_t acc0 = tmem + (uint32_t)(buf * 2 * BN) + lane_base, acc1 = acc0 + BN;
#pragma unroll 1
      for (int c = 0; c < BN; c += 32) {
        float v0[32], v1[32];
        tmem_ld32(acc0 + c, v0);
        tmem_ld32(acc1 + c, v1);
        if (r < p.M[g]) {
          float *dst = p.V + (size_t)(p.row0[g] + r) * p.ldv + n0 + c;
          const int ncol = p.N - (n0 + c);
          if (ncol >= 32) {
            // 32-byte stores: each lane writes whole sectors of its row
#pragma unroll
            for (int i = 0; i < 32; i += 8) {
              float o[8];
#pragma unroll
              for (int j = 0; j < 8; j++) o[j] = (v0[i + j] + v1[i + j] * (1.0f / 2048.0f)) * sc;
              asm volatile(
                  "st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst + i),
                  "f"(o[0]), "f"(o[1]), "f"(o[2]), "f"(o[3]), "f"(o[4]), "f"(o[5]), "f"(o[6]),
                  "f"(o[7])
                  : "memory");
            }
          } else {
            for (int i = 0; i < 32; i++)
              if (i < ncol) dst[i] = (v0[i] + v1[i] * (1.0f / 2048.0f)) * sc;
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(acce_bar(buf));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 2) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
int split_gemm_smem_bytes() { return SMEM_BYTES; }

// The shared-memory attribute and the resident CTA count are properties of a
// device: set and measured once per device, under a lock (host threads may
// launch on several devices).
static int launch_shape(int dev, int *ctas) {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static int cached[kMaxDev] = {0};
  if (dev < 0 || dev >= kMaxDev) return -1;
  std::lock_guard<std::mutex> lock(mu);
  if (cached[dev] == 0) {
    if (cudaFuncSetAttribute(k_split_gemm_grouped,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SMEM_BYTES) != cudaSuccess)
      return -1;
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_split_gemm_grouped, 192,
                                                      SMEM_BYTES) != cudaSuccess)
      return -1;
    if (per_sm < 1) return -1;
    cached[dev] = sms * per_sm;
  }
  *ctas = cached[dev];
  return 0;
}

int launch_split_gemm_grouped(const GroupedGemmArgs &g, cudaStream_t stream) {
  if (g.n_groups <= 0 || g.N <= 0) return 0;
  if (g.n_groups > kGemmMaxGroups) return -2;
  if ((g.lda * 2) % 16 != 0 || ((uintptr_t)g.a_hi | (uintptr_t)g.a_lo) % 16 != 0) return -2;
  // V rows take 32-byte stores: 32-byte aligned rows
  if (g.ldv % 8 != 0 || ((uintptr_t)g.V % 32) != 0 || g.K > g.lda) return -2;
  GroupedParams p;
  std::memset(&p, 0, sizeof(p));
  if (make_map(&p.a_hi, g.a_hi, g.K, g.a_rows, g.lda, BM) ||
      make_map(&p.a_lo, g.a_lo, g.K, g.a_rows, g.lda, BM))
    return -3;
  const int tiles_n = (g.N + BN - 1) / BN;
  int tiles = 0;
  for (int k = 0; k < g.n_groups; k++) {
    const GemmGroup &q = g.group[k];
    if ((q.ldb * 2) % 16 != 0 || ((uintptr_t)q.b_hi | (uintptr_t)q.b_lo) % 16 != 0 ||
        g.K > q.ldb)
      return -2;
    if (make_map(&p.b_hi[k], q.b_hi, g.K, q.b_rows, q.ldb, BN) ||
        make_map(&p.b_lo[k], q.b_lo, g.K, q.b_rows, q.ldb, BN))
      return -3;
    p.row0[k] = q.row0;
    p.M[k] = q.M;
    p.scale[k] = q.out_scale;
    p.tile_start[k] = tiles;
    tiles += ((q.M + BM - 1) / BM) * tiles_n;
  }
  p.tile_start[g.n_groups] = tiles;
  p.n_groups = g.n_groups;
  p.tiles_n = tiles_n;
  p.N = g.N;
  p.K = g.K;
  p.V = g.V;
  p.ldv = g.ldv;
  p.status = g.status;
  if (tiles == 0) return 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  int ctas = 0;
  if (launch_shape(dev, &ctas) != 0) return -1;
  // one persistent CTA per SM (the shared-memory ring admits one per SM)
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.blockDim = dim3(192, 1, 1);
  cfg.dynamicSmemBytes = SMEM_BYTES;
  cfg.stream = stream;
  cfg.gridDim = dim3(tiles < ctas ? tiles : ctas, 1, 1);
  if (cudaLaunchKernelEx(&cfg, k_split_gemm_grouped, p) != cudaSuccess) return -1;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace fpp
