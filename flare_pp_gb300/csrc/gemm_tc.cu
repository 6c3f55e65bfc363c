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
//
// One CTA computes a 128 x 256 tile of V:
//   warp 0 lane 0  TMA producer: 128B-swizzled K-major tiles of P_hi, P_lo,
//                  B_hi, B_lo (64 K-columns per stage) into a 2-stage ring
//   warp 1 lane 0  MMA issuer: 4 K=16 steps x 3 tcgen05.mma per stage,
//                  tcgen05.commit frees the stage
//   warp 2         allocates / frees the 512 TMEM columns
//   warps 0-3      epilogue: tcgen05.ld of their 32 TMEM lanes, combine,
//                  scale, store FP32 rows of V
// Every mbarrier wait is bounded; a wait that runs out records
// FPP_ERR_TIMEOUT in the status word and the CTA skips to its exit.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "common.cuh"
#include "gemm_tc.h"

namespace fpp {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 2;
constexpr int A_TILE = BM * BK * 2;  // bytes, one fp16 operand tile
constexpr int B_TILE = BN * BK * 2;
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr int TMEM_COLS = 512;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: false when about two seconds pass without the phase
// completing.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    for (int k = 0; k < 256; k++)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitBudgetNs) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map,
                                            uint32_t bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1)
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128B swizzle, 8-row core
// groups 1024 B apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)2 << 61;              // SWIZZLE_128B
  return d;
}

// Instruction descriptor: kind::f16 with fp16 A and B, FP32 accumulate,
// K-major A and B, M = 128, N = 256.
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) |
                            ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
        "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
        "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(128, 1)
k_split_gemm(const __grid_constant__ CUtensorMap map_a_hi,
             const __grid_constant__ CUtensorMap map_a_lo,
             const __grid_constant__ CUtensorMap map_b_hi,
             const __grid_constant__ CUtensorMap map_b_lo, int row0, int M, int N,
             int K, float out_scale, float *__restrict__ V, int ldv,
             DeviceStatus *status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned operand ring (required by the 128B swizzle)
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *gbase = smem_raw + (base - raw);
  const uint32_t bars = base + STAGES * STAGE_BYTES;
  uint64_t *bar_ptr = reinterpret_cast<uint64_t *>(gbase + STAGES * STAGE_BYTES);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_ptr + 2 * STAGES + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (STAGES + s); };
  const uint32_t done_bar = bars + 8u * (2 * STAGES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = blockIdx.x * BN;
  const int m0 = blockIdx.y * BM;
  const int kblocks = (K + BK - 1) / BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    mbar_init(done_bar, 1);
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
  const uint32_t acc0 = tmem, acc1 = tmem + BN;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    for (int kb = 0; kb < kblocks; kb++) {
      const int s = kb % STAGES;
      const uint32_t ph = (uint32_t)((kb / STAGES) & 1);
      if (!mbar_wait(empty_bar(s), ph ^ 1u)) {
        set_status(status, FPP_ERR_TIMEOUT, 101, kb);
        *abort_flag = 1;
        break;
      }
      if (*abort_flag) break;
      const uint32_t st = base + s * STAGE_BYTES;
      mbar_expect_tx(full_bar(s), STAGE_BYTES);
      const int kc = kb * BK;
      tma_load_2d(st, &map_a_hi, full_bar(s), kc, row0 + m0);
      tma_load_2d(st + A_TILE, &map_a_lo, full_bar(s), kc, row0 + m0);
      tma_load_2d(st + 2 * A_TILE, &map_b_hi, full_bar(s), kc, n0);
      tma_load_2d(st + 2 * A_TILE + B_TILE, &map_b_lo, full_bar(s), kc, n0);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    for (int kb = 0; kb < kblocks; kb++) {
      const int s = kb % STAGES;
      const uint32_t ph = (uint32_t)((kb / STAGES) & 1);
      if (!mbar_wait(full_bar(s), ph)) {
        set_status(status, FPP_ERR_TIMEOUT, 102, kb);
        *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = base + s * STAGE_BYTES;
      const uint32_t a_hi = st, a_lo = st + A_TILE;
      const uint32_t b_hi = st + 2 * A_TILE, b_lo = st + 2 * A_TILE + B_TILE;
#pragma unroll
      for (int ks = 0; ks < BK / 16; ks++) {
        const uint32_t off = ks * 32;  // 16 fp16 = 32 bytes along K
        const uint32_t acc = (kb > 0 || ks > 0) ? 1u : 0u;
        mma_f16(acc0, smem_desc(a_hi + off), smem_desc(b_hi + off), acc);
        mma_f16(acc1, smem_desc(a_hi + off), smem_desc(b_lo + off), acc);
        mma_f16(acc1, smem_desc(a_lo + off), smem_desc(b_hi + off), 1u);
      }
      mma_commit(empty_bar(s));
    }
    // signal the epilogue (also on the error path, so nobody waits forever)
    mma_commit(done_bar);
  }

  // ---------------- epilogue: all four warps ----------------
  __syncwarp();
  bool have = mbar_wait(done_bar, 0);
  have = __all_sync(0xffffffffu, have) != 0;
  if (!have && lane == 0) set_status(status, FPP_ERR_TIMEOUT, 103, warp);
  const int aborted = __shfl_sync(0xffffffffu, *abort_flag, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (have && !aborted) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int c = 0; c < BN; c += 32) {
      float v0[32], v1[32];
      tmem_ld32(acc0 + lane_base + c, v0);
      tmem_ld32(acc1 + lane_base + c, v1);
      if (row < M) {
        float *dst = V + (size_t)row * ldv + n0 + c;
        const int ncol = N - (n0 + c);
        if (ncol >= 32) {
#pragma unroll
          for (int i = 0; i < 32; i += 4) {
            float4 o;
            o.x = (v0[i + 0] + v1[i + 0] * (1.0f / 2048.0f)) * out_scale;
            o.y = (v0[i + 1] + v1[i + 1] * (1.0f / 2048.0f)) * out_scale;
            o.z = (v0[i + 2] + v1[i + 2] * (1.0f / 2048.0f)) * out_scale;
            o.w = (v0[i + 3] + v1[i + 3] * (1.0f / 2048.0f)) * out_scale;
            *reinterpret_cast<float4 *>(dst + i) = o;
          }
        } else {
          for (int i = 0; i < 32; i++)
            if (i < ncol) dst[i] = (v0[i] + v1[i] * (1.0f / 2048.0f)) * out_scale;
        }
      }
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
// The tensor-map encoder is a driver entry point; it is resolved through the
// runtime so that the library does not link libcuda directly.
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

static int make_map(CUtensorMap *map, const void *ptr, int inner, int rows,
                    int ld_elems, int box_rows) {
  auto cuTensorMapEncodeTiled = encode_fn();
  if (!cuTensorMapEncodeTiled) return -1;
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld_elems * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = cuTensorMapEncodeTiled(
      map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(ptr), dims, strides,
      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -1;
}

int split_gemm_smem_bytes() { return SMEM_BYTES; }

int launch_split_gemm(const SplitGemmArgs &g, cudaStream_t stream) {
  if (g.M <= 0 || g.N <= 0) return 0;
  // operand rows must start 16-byte aligned and be 16-byte multiples
  if ((g.lda * 2) % 16 != 0 || (g.ldb * 2) % 16 != 0) return -2;
  if (((uintptr_t)g.a_hi | (uintptr_t)g.a_lo | (uintptr_t)g.b_hi |
       (uintptr_t)g.b_lo) % 16 != 0)
    return -2;
  if (g.ldv % 4 != 0 || ((uintptr_t)g.V % 16) != 0) return -2;
  if (g.K > g.lda || g.K > g.ldb) return -2;
  CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo;
  if (make_map(&ma_hi, g.a_hi, g.K, g.a_rows, g.lda, BM) ||
      make_map(&ma_lo, g.a_lo, g.K, g.a_rows, g.lda, BM) ||
      make_map(&mb_hi, g.b_hi, g.K, g.b_rows, g.ldb, BN) ||
      make_map(&mb_lo, g.b_lo, g.K, g.b_rows, g.ldb, BN))
    return -3;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_split_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SMEM_BYTES) != cudaSuccess)
      return -1;
    attr = true;
  }
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
  k_split_gemm<<<grid, 128, SMEM_BYTES, stream>>>(ma_hi, ma_lo, mb_hi, mb_lo, g.row0,
                                                  g.M, g.N, g.K, g.out_scale, g.V,
                                                  g.ldv, g.status);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace fpp
