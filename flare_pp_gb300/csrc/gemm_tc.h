// Launch interface of the split-fp16 tcgen05 contraction.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "common.cuh"

namespace fpp {

struct SplitGemmArgs {
  // A operand: a_rows x K (row stride lda elements), tile rows start at row0
  const __half *a_hi, *a_lo;
  int a_rows, lda, row0;
  // B operand: b_rows x K (row stride ldb)
  const __half *b_hi, *b_lo;
  int b_rows, ldb;
  int M, N, K;          // output tile extent: M rows from row0, N columns
  float out_scale;      // 1 / (sA sB)
  float *V;             // output rows row0.. (row stride ldv), already offset
  int ldv;
  DeviceStatus *status;
};

int launch_split_gemm(const SplitGemmArgs &g, cudaStream_t stream);
int split_gemm_smem_bytes();

}  // namespace fpp
