// C ABI and host helper of the FP64-accurate tensor-core GEMM (gemm_ozaki.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "capi_state.h"
#include "gemm_ozaki.h"
#include "internal.h"

namespace fpp {

int ozaki_dgemm_nt(int M, int N, int K, const double *A, long long lda, const double *B,
                   long long ldb, double *C, long long ldc, OzakiWork &w, cudaStream_t st,
                   bool b_lower) {
  if (M <= 0 || N <= 0) return FPP_OK;
  if (K <= 0) return fail(FPP_ERR_INVALID, "GEMM with K <= 0");
  const OzakiShape sa = ozaki_shape(M, K), sb = ozaki_shape(N, K);
  FPP_TRY(w.a.reserve(sa.plane_bytes));
  FPP_TRY(w.b.reserve(sb.plane_bytes));
  FPP_TRY(w.pa.reserve(sizeof(double) * M));
  FPP_TRY(w.pb.reserve(sizeof(double) * N));
  if (w.status.bytes < sizeof(DeviceStatus)) {  // cleared once, then by each check
    FPP_TRY(w.status.reserve(sizeof(DeviceStatus)));
    FPP_CUDA(cudaMemsetAsync(w.status.ptr, 0, sizeof(DeviceStatus), st));
  }
  if (launch_ozaki_split(M, K, A, lda, w.a.as<__half>(), w.pa.as<double>(), st) != 0 ||
      launch_ozaki_split(N, K, B, ldb, w.b.as<__half>(), w.pb.as<double>(), st) != 0)
    return fail(FPP_ERR_CUDA, "digit-plane split launch failed");
  const int rc = launch_ozaki_gemm(M, N, K, w.a.as<__half>(), w.pa.as<double>(),
                                   w.b.as<__half>(), w.pb.as<double>(), C, ldc,
                                   w.status.as<DeviceStatus>(), st, b_lower);
  if (rc != 0) return fail(FPP_ERR_CUDA, "tensor-core FP64 GEMM launch failed (" +
                                             std::to_string(rc) + ")");
  return FPP_OK;
}

int ozaki_check_status(OzakiWork &w, cudaStream_t st) {
  if (w.status.bytes < sizeof(DeviceStatus)) return FPP_OK;  // nothing ran
  DeviceStatus h;
  FPP_CUDA(cudaMemcpyAsync(&h, w.status.ptr, sizeof(h), cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  if (h.code != 0) FPP_CUDA(cudaMemsetAsync(w.status.ptr, 0, sizeof(DeviceStatus), st));
  if (h.code != 0)
    return fail(h.code, "tensor-core FP64 GEMM: a bounded wait ran out (site " +
                            std::to_string(h.where) + ")");
  return FPP_OK;
}

}  // namespace fpp

using namespace fpp;

extern "C" int fpp_dgemm_nt(int32_t M, int32_t N, int32_t K, const double *A, int64_t lda,
                            const double *B, int64_t ldb, double *C, int64_t ldc,
                            int32_t on_device, void *stream) {
  if ((M > 0 && N > 0) && (!A || !B || !C)) return fail(FPP_ERR_INVALID, "null argument");
  if (M < 0 || N < 0 || K < 0) return fail(FPP_ERR_INVALID, "negative size");
  if (M == 0 || N == 0) return FPP_OK;
  if (K == 0) {
    if (on_device) {
      FPP_CUDA(cudaMemset2DAsync(C, sizeof(double) * ldc, 0, sizeof(double) * N, M,
                                 (cudaStream_t)stream));
    } else {
      for (int i = 0; i < M; i++) std::fill(C + (size_t)i * ldc, C + (size_t)i * ldc + N, 0.0);
    }
    return FPP_OK;
  }
  if (lda < K || ldb < K || ldc < N) return fail(FPP_ERR_INVALID, "leading dimension too small");
  cudaStream_t st = (cudaStream_t)stream;
  OzakiWork w;
  if (on_device) {
    FPP_TRY(ozaki_dgemm_nt(M, N, K, A, lda, B, ldb, C, ldc, w, st));
    return ozaki_check_status(w, st);
  }
  DevBuf dA, dB, dC;
  FPP_TRY(dA.reserve(sizeof(double) * (size_t)M * K));
  FPP_TRY(dB.reserve(sizeof(double) * (size_t)N * K));
  FPP_TRY(dC.reserve(sizeof(double) * (size_t)M * N));
  FPP_CUDA(cudaMemcpy2DAsync(dA.ptr, sizeof(double) * K, A, sizeof(double) * lda,
                             sizeof(double) * K, M, cudaMemcpyHostToDevice, st));
  FPP_CUDA(cudaMemcpy2DAsync(dB.ptr, sizeof(double) * K, B, sizeof(double) * ldb,
                             sizeof(double) * K, N, cudaMemcpyHostToDevice, st));
  FPP_TRY(ozaki_dgemm_nt(M, N, K, dA.as<double>(), K, dB.as<double>(), K, dC.as<double>(), N,
                         w, st));
  FPP_TRY(ozaki_check_status(w, st));
  FPP_CUDA(cudaMemcpy2DAsync(C, sizeof(double) * ldc, dC.ptr, sizeof(double) * N,
                             sizeof(double) * N, M, cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  return FPP_OK;
}
