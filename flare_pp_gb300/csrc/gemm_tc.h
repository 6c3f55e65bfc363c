// Launch interface of the split-fp16 tcgen05 contraction.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "common.cuh"

namespace fpp {

// Grouped persistent form: operand rows in species blocks (row0, M) of one
// A, each block against its own B; lo planes hold the fp16 residual scaled by
// 2048 (A ~ A_hi + A_lo / 2048), V[row0 + r, :] = (A B^T)[r, :] * out_scale.
constexpr int kGemmMaxGroups = 8;
struct GemmGroup {
  const __half *b_hi, *b_lo;
  int b_rows, ldb;
  int row0, M;
  float out_scale;
};
struct GroupedGemmArgs {
  const __half *a_hi, *a_lo;
  int a_rows, lda;
  int n_groups;
  GemmGroup group[kGemmMaxGroups];
  int N, K;
  float *V;  // rows indexed like A's rows (row stride ldv)
  int ldv;
  DeviceStatus *status;
};
int launch_split_gemm_grouped(const GroupedGemmArgs &g, cudaStream_t stream);
int split_gemm_smem_bytes();

}  // namespace fpp
