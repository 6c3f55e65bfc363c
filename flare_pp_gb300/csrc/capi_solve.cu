// C ABI: SparseGP::update_matrices_QR (sparse_gp.cpp:576-610) in FP64 with
// cuSOLVER (Cholesky, Householder QR, Q^T b) and cuBLAS (triangular solves).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fpp {

// Scatter the stacked least-squares matrix in column-major order:
// A[i, j] = sqrt(noise_i) Kuf[j, i] for i < m, A[m + i, j] = L[j, i] (j >= i).
__global__ void k_stack_A(int n, int m, const double *__restrict__ Kuf,
                          const double *__restrict__ sq, const double *__restrict__ Lc,
                          double *__restrict__ A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long rows = (long long)m + n;
  if (t >= rows * n) return;
  const int j = (int)(t / rows);
  const long long i = t - (long long)j * rows;
  double v;
  if (i < m) {
    v = sq[i] * Kuf[(size_t)j * m + i];
  } else {
    const int r = (int)(i - m);
    // L is column-major lower: L[j][r] = Lc[r * n + j] for j >= r
    v = (j >= r) ? Lc[(size_t)r * n + j] : 0.0;
  }
  A[t] = v;
}

__global__ void k_scale_b(int m, int n, const double *__restrict__ y,
                          const double *__restrict__ sq, double *__restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) b[i] = sq[i] * y[i];
  else if (i < m + n) b[i] = 0.0;
}

__global__ void k_sqrt(int m, const double *__restrict__ x, double *__restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) y[i] = sqrt(x[i]);
}

__global__ void k_identity_jitter(int n, double *__restrict__ K, double jitter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) K[(size_t)i * n + i] += jitter;
}

__global__ void k_eye(int n, double *__restrict__ E) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * n) return;
  const int j = (int)(t / n), i = (int)(t - (long long)j * n);
  E[t] = (i == j) ? 1.0 : 0.0;
}

__global__ void k_transpose(int n, const double *__restrict__ X, double *__restrict__ Y) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * n) return;
  const int j = (int)(t / n), i = (int)(t - (long long)j * n);
  Y[(size_t)i * n + j] = X[t];
}

}  // namespace fpp

using namespace fpp;

#define SOLVER_OK(call, what)                                                  \
  do {                                                                         \
    cusolverStatus_t _s = (call);                                              \
    if (_s != CUSOLVER_STATUS_SUCCESS) {                                       \
      rc = fail(FPP_ERR_CUDA, std::string("cuSOLVER ") + what + " status " +   \
                                  std::to_string((int)_s));                    \
      goto done;                                                               \
    }                                                                          \
  } while (0)
#define BLAS_OK(call, what)                                                    \
  do {                                                                         \
    cublasStatus_t _s = (call);                                                \
    if (_s != CUBLAS_STATUS_SUCCESS) {                                         \
      rc = fail(FPP_ERR_CUDA, std::string("cuBLAS ") + what + " status " +     \
                                  std::to_string((int)_s));                    \
      goto done;                                                               \
    }                                                                          \
  } while (0)
#define RT_OK(call)                                                            \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) {                                                   \
      rc = cuda_fail(_e, #call);                                               \
      goto done;                                                               \
    }                                                                          \
  } while (0)

extern "C" int fpp_update_matrices_QR(int32_t n, int32_t m, const double *Kuu,
                                      const double *Kuf, const double *y,
                                      const double *noise_vector, double jitter,
                                      double *alpha, double *R_inv, double *L_inv,
                                      void *stream) {
  if (n <= 0 || m < 0) return fail(FPP_ERR_INVALID, "need n > 0 and m >= 0");
  if (!Kuu || (m > 0 && (!Kuf || !y || !noise_vector)))
    return fail(FPP_ERR_INVALID, "null argument");
  for (long long k = 0; k < (long long)m; k++)
    if (!(noise_vector[k] >= 0) || !std::isfinite(y[k]))
      return fail(FPP_ERR_NUMERIC, "noise must be >= 0 and labels finite");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = FPP_OK;
  const long long rows = (long long)m + n;
  cusolverDnHandle_t sh = nullptr;
  cublasHandle_t bh = nullptr;
  DevBuf dK, dKuf, dy, dsq, dA, db, dtau, dwork, dinfo, dE, dT;
  int lwork = 0, lw2 = 0, info = 0;
  const double one = 1.0;
  if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS)
    return fail(FPP_ERR_CUDA, "cusolverDnCreate failed");
  if (cublasCreate(&bh) != CUBLAS_STATUS_SUCCESS) {
    cusolverDnDestroy(sh);
    return fail(FPP_ERR_CUDA, "cublasCreate failed");
  }
  cusolverDnSetStream(sh, st);
  cublasSetStream(bh, st);
  if ((rc = dK.reserve(sizeof(double) * (size_t)n * n)) ||
      (rc = dKuf.reserve(sizeof(double) * std::max<size_t>(1, (size_t)n * m))) ||
      (rc = dy.reserve(sizeof(double) * std::max(1, m))) ||
      (rc = dsq.reserve(sizeof(double) * std::max(1, m))) ||
      (rc = dA.reserve(sizeof(double) * rows * n)) || (rc = db.reserve(sizeof(double) * rows)) ||
      (rc = dtau.reserve(sizeof(double) * n)) || (rc = dinfo.reserve(sizeof(int))) ||
      (rc = dE.reserve(sizeof(double) * (size_t)n * n)) ||
      (rc = dT.reserve(sizeof(double) * (size_t)n * n)))
    goto done;
  // Kuu is symmetric: row-major == column-major
  RT_OK(cudaMemcpyAsync(dK.ptr, Kuu, sizeof(double) * (size_t)n * n, cudaMemcpyHostToDevice, st));
  if (m > 0) {
    RT_OK(cudaMemcpyAsync(dKuf.ptr, Kuf, sizeof(double) * (size_t)n * m, cudaMemcpyHostToDevice, st));
    RT_OK(cudaMemcpyAsync(dy.ptr, y, sizeof(double) * m, cudaMemcpyHostToDevice, st));
    RT_OK(cudaMemcpyAsync(dsq.ptr, noise_vector, sizeof(double) * m, cudaMemcpyHostToDevice, st));
    k_sqrt<<<ceil_div(m, 256), 256, 0, st>>>(m, dsq.as<double>(), dsq.as<double>());
  }
  k_identity_jitter<<<ceil_div(n, 256), 256, 0, st>>>(n, dK.as<double>(), jitter);
  // L = chol(Kuu + jitter I), lower, column-major
  SOLVER_OK(cusolverDnDpotrf_bufferSize(sh, CUBLAS_FILL_MODE_LOWER, n, dK.as<double>(), n, &lwork),
            "potrf_bufferSize");
  SOLVER_OK(cusolverDnDgeqrf_bufferSize(sh, (int)rows, n, dA.as<double>(), (int)rows, &lw2),
            "geqrf_bufferSize");
  lwork = std::max(lwork, lw2);
  SOLVER_OK(cusolverDnDormqr_bufferSize(sh, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, (int)rows, 1, n,
                                        dA.as<double>(), (int)rows, dtau.as<double>(),
                                        db.as<double>(), (int)rows, &lw2),
            "ormqr_bufferSize");
  lwork = std::max(lwork, lw2);
  if ((rc = dwork.reserve(sizeof(double) * std::max(1, lwork)))) goto done;
  SOLVER_OK(cusolverDnDpotrf(sh, CUBLAS_FILL_MODE_LOWER, n, dK.as<double>(), n,
                             dwork.as<double>(), lwork, dinfo.as<int>()),
            "potrf");
  RT_OK(cudaMemcpyAsync(&info, dinfo.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  RT_OK(cudaStreamSynchronize(st));
  if (info != 0) {
    rc = fail(FPP_ERR_NUMERIC, "Kuu + jitter I is not positive definite");
    goto done;
  }
  // A = [sqrt(noise) Kuf^T ; L^T]
  k_stack_A<<<(unsigned)((rows * n + 255) / 256), 256, 0, st>>>(n, m, dKuf.as<double>(),
                                                               dsq.as<double>(),
                                                               dK.as<double>(), dA.as<double>());
  k_scale_b<<<(unsigned)((rows + 255) / 256), 256, 0, st>>>(m, n, dy.as<double>(),
                                                           dsq.as<double>(), db.as<double>());
  SOLVER_OK(cusolverDnDgeqrf(sh, (int)rows, n, dA.as<double>(), (int)rows, dtau.as<double>(),
                             dwork.as<double>(), lwork, dinfo.as<int>()),
            "geqrf");
  SOLVER_OK(cusolverDnDormqr(sh, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, (int)rows, 1, n,
                             dA.as<double>(), (int)rows, dtau.as<double>(), db.as<double>(),
                             (int)rows, dwork.as<double>(), lwork, dinfo.as<int>()),
            "ormqr");
  // alpha = R^-1 (Q^T b)[0:n]
  BLAS_OK(cublasDtrsv(bh, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n,
                      dA.as<double>(), (int)rows, db.as<double>(), 1),
          "trsv");
  if (alpha) {
    RT_OK(cudaMemcpyAsync(alpha, db.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  }
  if (R_inv) {
    k_eye<<<(unsigned)(((long long)n * n + 255) / 256), 256, 0, st>>>(n, dE.as<double>());
    BLAS_OK(cublasDtrsm(bh, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N,
                        CUBLAS_DIAG_NON_UNIT, n, n, &one, dA.as<double>(), (int)rows,
                        dE.as<double>(), n),
            "trsm R");
    k_transpose<<<(unsigned)(((long long)n * n + 255) / 256), 256, 0, st>>>(n, dE.as<double>(),
                                                                            dT.as<double>());
    RT_OK(cudaMemcpyAsync(R_inv, dT.ptr, sizeof(double) * (size_t)n * n,
                          cudaMemcpyDeviceToHost, st));
    RT_OK(cudaStreamSynchronize(st));
  }
  if (L_inv) {
    k_eye<<<(unsigned)(((long long)n * n + 255) / 256), 256, 0, st>>>(n, dE.as<double>());
    BLAS_OK(cublasDtrsm(bh, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                        CUBLAS_DIAG_NON_UNIT, n, n, &one, dK.as<double>(), n,
                        dE.as<double>(), n),
            "trsm L");
    k_transpose<<<(unsigned)(((long long)n * n + 255) / 256), 256, 0, st>>>(n, dE.as<double>(),
                                                                            dT.as<double>());
    RT_OK(cudaMemcpyAsync(L_inv, dT.ptr, sizeof(double) * (size_t)n * n,
                          cudaMemcpyDeviceToHost, st));
  }
  RT_OK(cudaStreamSynchronize(st));
  RT_OK(cudaGetLastError());
done:
  cudaStreamSynchronize(st);
  cublasDestroy(bh);
  cusolverDnDestroy(sh);
  return rc;
}
