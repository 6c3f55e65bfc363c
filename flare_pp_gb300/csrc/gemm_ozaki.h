// FP64-accurate C = A B^T from exact fp16 digit planes on the tcgen05 tensor
// cores (gemm_ozaki.cu).  Row-major A (M x K), B (N x K), C (M x N).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstddef>

#include "common.cuh"

namespace fpp {

constexpr int kOzakiDigits = 11;    // signed digits per operand entry
constexpr int kOzakiBits = 5;       // bits per digit (|digit| <= 31)
constexpr int kOzakiChunkK = 1536;  // K columns per exact FP32 level sum

// Padded shape of one operand's digit planes: rows to a multiple of 128,
// K to a multiple of 64; plane_bytes covers all kOzakiDigits planes.
struct OzakiShape {
  int rows_pad, k_pad;
  size_t plane_bytes;
};
OzakiShape ozaki_shape(int rows, int K);

// Digit planes (kOzakiDigits x rows_pad x k_pad fp16, zero padded) and the
// power of two 2^e of each row (max |row| < 2^e) of X (rows x K, row stride
// ldx, device memory).  The entries must be finite.
int launch_ozaki_split(int rows, int K, const double *X, long long ldx, __half *planes,
                       double *p2, cudaStream_t stream);

// C (M x N, row stride ldc) = A B^T from the digit planes and powers of two
// of A (M x K) and B (N x K).  C need not be initialised.  b_lower: B is
// lower triangular (B[n][k] = 0 for k > n; an L^-1, or an R^-1 transposed),
// and the K blocks above each column tile's last row are skipped.  0 on
// success.
int launch_ozaki_gemm(int M, int N, int K, const __half *a_planes, const double *pa,
                      const __half *b_planes, const double *pb, double *C, long long ldc,
                      DeviceStatus *status, cudaStream_t stream, bool b_lower = false);

}  // namespace fpp
