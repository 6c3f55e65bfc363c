// C ABI: the log marginal likelihood of the sparse GP and its gradient in the
// hyperparameters (sigma of each NormalizedDotProduct kernel, sigma_e,
// sigma_f, sigma_s), FP64 on the GPU:
//   SparseGP::compute_likelihood_stable (sparse_gp.cpp:704-732),
//   SparseGP::compute_likelihood_gradient_stable (sparse_gp.cpp:734-862),
//   SparseGP::compute_KnK (sparse_gp.cpp:888-922).
//
// With Lambda = diag(noise_vector), r = y - Kuf^T alpha and, for kernel i
// (rows [o_i, o_i + n_i) of Kuu and Kuf; Kuu is block diagonal over the
// kernels), dKuu/dsigma_i = 2 Kuu_i / sigma_i and dKuf/dsigma_i = 2 Kuf_i /
// sigma_i on kernel i's rows and 0 elsewhere (normalized_dot_product.cpp:
// 581-615):
//   data_fit   = -1/2 y . (Lambda r)
//   complexity = 1/2 (log det Lambda - 2 sum log|L_inv_ii| + 2 sum log|R_inv_ii|)
//   d/dsigma_i = 1/2 tr(Kuu^-1 dKuu) - 1/2 tr(Pi Sigma)
//                + (dKuf^T alpha) . (Lambda r) - 1/2 alpha . (dKuu alpha),
//                Pi = dKuf Lambda Kuf^T + (its transpose) + dKuu
//   d/dsigma_x = -n_x / sigma_x + tr(KnK_x Sigma) / sigma_x^3
//                + r . (one_x r) / sigma_x^3,   KnK_x = Kuf one_x Kuf^T.
// The traces tr(KnK_x Sigma) are sums over the labels of kind x of
// k_l . (Sigma k_l) (k_l = column l of Kuf): one GEMM B = Sigma Kuf replaces
// the three n x n products of the reference, and its row blocks give the
// per-kernel traces; tr(Kuu^-1 dKuu) is formed as in the reference, by an LU
// solve of Kuu (against Kuu, then the diagonal of each kernel's block).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "capi_state.h"
#include "common.cuh"
#include "internal.h"

namespace fpp {
namespace {

#define FPP_CUBLAS_LK(call)                                                  \
  do {                                                                       \
    cublasStatus_t _s = (call);                                              \
    if (_s != CUBLAS_STATUS_SUCCESS)                                         \
      return fail(FPP_ERR_CUDA, std::string("cuBLAS: ") + #call + " status " + \
                                    std::to_string((int)_s));                \
  } while (0)
#define FPP_CUSOLVER_LK(call)                                                \
  do {                                                                       \
    cusolverStatus_t _s = (call);                                            \
    if (_s != CUSOLVER_STATUS_SUCCESS)                                       \
      return fail(FPP_ERR_CUDA, std::string("cuSOLVER: ") + #call +          \
                                    " status " + std::to_string((int)_s));   \
  } while (0)

constexpr int kLkBlocks = 256, kLkThreads = 256, kLkMaxKernels = 8;
// per-block partial sums: 0 y Lambda r, 1-3 r^2 of kind e, f, s, 4-6
// k_l . (Sigma k_l) of kind e, f, s (all rows), then per kernel i:
// 7 + 4 i: Ka_i Lambda r, 8 + 4 i .. 10 + 4 i: the traces on kernel i's rows
constexpr int kLkSums = 7 + 4 * kLkMaxKernels;

__device__ __forceinline__ double block_sum(double v, double *sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sm[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;
}

// Per-block partial sums over the labels (fixed order: the host adds the
// blocks in index order), laid out as kLkSums above.  Ka is the full
// Kuf^T alpha, Kak[i] = Kuf_i^T alpha_i (kernel i's rows); B = Sigma Kuf
// (when given).
__global__ void k_label_sums(int n, int m, int nk, const int *__restrict__ koff,
                             const double *__restrict__ y, const double *__restrict__ Ka,
                             const double *__restrict__ Kak, const int *__restrict__ kind,
                             const double *__restrict__ inv_var,
                             const double *__restrict__ Kuf, const double *__restrict__ B,
                             double *__restrict__ partial) {
  __shared__ double sm[32];
  double acc[kLkSums];
#pragma unroll
  for (int k = 0; k < kLkSums; k++) acc[k] = 0.0;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < m; l += gridDim.x * blockDim.x) {
    const int t = kind[l];
    const double nv = inv_var[t];
    const double r = y[l] - Ka[l];
    acc[0] = fma(y[l], nv * r, acc[0]);
    const double r2 = r * r;
    acc[1] += t == 0 ? r2 : 0.0;
    acc[2] += t == 1 ? r2 : 0.0;
    acc[3] += t == 2 ? r2 : 0.0;
#pragma unroll
    for (int i = 0; i < kLkMaxKernels; i++) {
      if (i >= nk) break;
      acc[7 + 4 * i] = fma(Kak[(size_t)i * m + l], nv * r, acc[7 + 4 * i]);
      if (B) {
        // column l of the row-major n x m matrices, kernel i's rows
        double q = 0.0;
        for (int row = koff[i]; row < koff[i + 1]; row++)
          q = fma(Kuf[(size_t)row * m + l], B[(size_t)row * m + l], q);
        acc[8 + 4 * i] += t == 0 ? q : 0.0;
        acc[9 + 4 * i] += t == 1 ? q : 0.0;
        acc[10 + 4 * i] += t == 2 ? q : 0.0;
        acc[4] += t == 0 ? q : 0.0;
        acc[5] += t == 1 ? q : 0.0;
        acc[6] += t == 2 ? q : 0.0;
      }
    }
  }
  for (int k = 0; k < kLkSums; k++) {
    const double s = block_sum(acc[k], sm);
    if (threadIdx.x == 0) partial[(size_t)blockIdx.x * kLkSums + k] = s;
  }
}

// sum of A .* C over the square block [o, o + len) of n x n matrices, per
// grid block: tr(A_b C_b) for a symmetric C
__global__ void k_frob(int n, int o, int len, const double *__restrict__ A,
                       const double *__restrict__ C, double *__restrict__ partial) {
  __shared__ double sm[32];
  double acc = 0.0;
  const long long nn = (long long)len * len;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nn;
       k += (long long)gridDim.x * blockDim.x) {
    const size_t idx = (size_t)(o + k / len) * n + (o + k % len);
    acc = fma(A[idx], C[idx], acc);
  }
  const double s = block_sum(acc, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// columns of Kuf not of kind t set to zero (Kuf one_t)
__global__ void k_mask_kind(int n, int m, const double *__restrict__ Kuf,
                            const int *__restrict__ kind, int t, double *__restrict__ out) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= (long long)n * m) return;
  const int l = (int)(k % m);
  out[k] = kind[l] == t ? Kuf[k] : 0.0;
}

__global__ void k_diag_sum(int n, int o, int len, const double *__restrict__ X, double *out) {
  __shared__ double sm[32];
  double acc = 0.0;
  for (int i = o + threadIdx.x; i < o + len; i += blockDim.x) acc += X[(size_t)i * n + i];
  const double s = block_sum(acc, sm);
  if (threadIdx.x == 0) out[0] = s;
}

int upload(DevBuf &b, const void *h, size_t bytes, cudaStream_t st) {
  FPP_TRY(b.reserve(std::max<size_t>(bytes, 8)));
  if (bytes) FPP_CUDA(cudaMemcpyAsync(b.ptr, h, bytes, cudaMemcpyHostToDevice, st));
  return FPP_OK;
}

}  // namespace
}  // namespace fpp

using namespace fpp;

namespace {

int likelihood_core(int32_t n, int32_t m, const double *Kuf, const double *Kuu,
                    const double *y, const int32_t *label_kind, const double *alpha,
                    const double *Sigma, const double *L_diag, const double *R_inv_diag,
                    int32_t nk, const int32_t *koff, const double *hyps,
                    int32_t want_gradient, double *out, double *KnK, cudaStream_t st) {
  if (n <= 0 || m < 0) return fail(FPP_ERR_INVALID, "bad sizes");
  if (nk < 1 || nk > kLkMaxKernels) return fail(FPP_ERR_INVALID, "1 to 8 kernels");
  if (!koff || koff[0] != 0 || koff[nk] != n)
    return fail(FPP_ERR_INVALID, "kernel row offsets must run from 0 to n");
  for (int i = 0; i < nk; i++)
    if (koff[i + 1] < koff[i]) return fail(FPP_ERR_INVALID, "kernel row offsets decrease");
  if (!Kuf && m > 0) return fail(FPP_ERR_INVALID, "null Kuf");
  if (!y && m > 0) return fail(FPP_ERR_INVALID, "null y");
  if (!label_kind && m > 0) return fail(FPP_ERR_INVALID, "null label kinds");
  if (!alpha || !L_diag || !R_inv_diag || !hyps || !out)
    return fail(FPP_ERR_INVALID, "null argument");
  if (want_gradient && (!Kuu || !Sigma)) return fail(FPP_ERR_INVALID, "null Kuu / Sigma");
  for (int k = 0; k < nk + 3; k++)
    if (!std::isfinite(hyps[k]) || hyps[k] == 0.0)
      return fail(FPP_ERR_NUMERIC, "hyperparameters must be finite and non-zero");
  long long cnt[3] = {0, 0, 0};
  for (int l = 0; l < m; l++) {
    if (label_kind[l] < 0 || label_kind[l] > 2)
      return fail(FPP_ERR_INVALID, "label kind outside 0..2");
    cnt[label_kind[l]]++;
  }
  const double noise[3] = {hyps[nk], hyps[nk + 1], hyps[nk + 2]};
  const double inv_var[3] = {1.0 / (noise[0] * noise[0]), 1.0 / (noise[1] * noise[1]),
                             1.0 / (noise[2] * noise[2])};
  cublasHandle_t h;
  if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) return fail(FPP_ERR_CUDA, "cublasCreate failed");
  struct HGuard {
    cublasHandle_t h;
    ~HGuard() { cublasDestroy(h); }
  } hg{h};
  cublasSetMathMode(h, CUBLAS_PEDANTIC_MATH);
  FPP_CUBLAS_LK(cublasSetStream(h, st));
  const double one = 1.0, zero = 0.0;
  DevBuf dKuf, dy, dkind, dalpha, dKa, dKak, dkoff, dnv, dpart, dB, dSig, dKuu, dX, dLU, dwork,
      dpiv, dinfo, dtmp, dfro;
  FPP_TRY(upload(dKuf, Kuf, sizeof(double) * (size_t)n * m, st));
  FPP_TRY(upload(dy, y, sizeof(double) * (size_t)m, st));
  FPP_TRY(upload(dkind, label_kind, sizeof(int) * (size_t)m, st));
  FPP_TRY(upload(dalpha, alpha, sizeof(double) * n, st));
  FPP_TRY(upload(dnv, inv_var, sizeof(inv_var), st));
  FPP_TRY(upload(dkoff, koff, sizeof(int32_t) * (nk + 1), st));
  FPP_TRY(dKa.reserve(sizeof(double) * std::max(m, 1)));
  FPP_TRY(dKak.reserve(sizeof(double) * (size_t)nk * std::max(m, 1)));
  // Ka = Kuf^T alpha (Kuf row-major n x m is column-major m x n), and per
  // kernel Ka_i = Kuf_i^T alpha_i from its rows
  if (m) {
    FPP_CUBLAS_LK(cublasDgemv(h, CUBLAS_OP_N, m, n, &one, dKuf.as<double>(), m,
                              dalpha.as<double>(), 1, &zero, dKa.as<double>(), 1));
    for (int i = 0; i < nk; i++) {
      const int ni = koff[i + 1] - koff[i];
      if (ni == 0) {
        FPP_CUDA(cudaMemsetAsync(dKak.as<double>() + (size_t)i * m, 0, sizeof(double) * m, st));
        continue;
      }
      FPP_CUBLAS_LK(cublasDgemv(h, CUBLAS_OP_N, m, ni, &one,
                                dKuf.as<double>() + (size_t)koff[i] * m, m,
                                dalpha.as<double>() + koff[i], 1, &zero,
                                dKak.as<double>() + (size_t)i * m, 1));
    }
  }
  const double *Bp = nullptr;
  if (want_gradient) {
    FPP_TRY(upload(dSig, Sigma, sizeof(double) * (size_t)n * n, st));
    FPP_TRY(upload(dKuu, Kuu, sizeof(double) * (size_t)n * n, st));
    if (m) {
      // B = Sigma Kuf (row-major n x m): column-major m x n = Kuf^T Sigma^T
      FPP_TRY(dB.reserve(sizeof(double) * (size_t)n * m));
      FPP_CUBLAS_LK(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, n, &one, dKuf.as<double>(), m,
                                dSig.as<double>(), n, &zero, dB.as<double>(), m));
      Bp = dB.as<double>();
    }
  }
  FPP_TRY(dpart.reserve(sizeof(double) * kLkBlocks * kLkSums));
  FPP_CUDA(cudaMemsetAsync(dpart.ptr, 0, sizeof(double) * kLkBlocks * kLkSums, st));
  if (m) {
    k_label_sums<<<kLkBlocks, kLkThreads, 0, st>>>(
        n, m, nk, dkoff.as<int>(), dy.as<double>(), dKa.as<double>(), dKak.as<double>(),
        dkind.as<int>(), dnv.as<double>(), dKuf.as<double>(), Bp, dpart.as<double>());
    FPP_CUDA(cudaGetLastError());
  }
  std::vector<double> tr_kuu_sigma(nk, 0.0), tr_kinv(nk, 0.0), a_kuu_a(nk, 0.0);
  if (want_gradient) {
    const long long nn = (long long)n * n;
    FPP_TRY(dfro.reserve(sizeof(double) * kLkBlocks * nk));
    FPP_TRY(dtmp.reserve(sizeof(double) * (n + nk)));
    cublasSetPointerMode(h, CUBLAS_POINTER_MODE_HOST);
    for (int i = 0; i < nk; i++) {
      const int o = koff[i], ni = koff[i + 1] - koff[i];
      if (ni == 0) continue;
      k_frob<<<kLkBlocks, kLkThreads, 0, st>>>(n, o, ni, dKuu.as<double>(), dSig.as<double>(),
                                               dfro.as<double>() + (size_t)i * kLkBlocks);
      FPP_CUDA(cudaGetLastError());
      // alpha_i . (Kuu_i alpha_i)
      FPP_CUBLAS_LK(cublasDgemv(h, CUBLAS_OP_N, ni, ni, &one, dKuu.as<double>() + (size_t)o * n + o,
                                n, dalpha.as<double>() + o, 1, &zero, dtmp.as<double>(), 1));
      FPP_CUBLAS_LK(cublasDdot(h, ni, dtmp.as<double>(), 1, dalpha.as<double>() + o, 1,
                               &a_kuu_a[i]));
    }
    // tr(Kuu^-1 dKuu_i): LU of Kuu solved against Kuu, then each kernel's
    // diagonal block scaled by 2 / sigma_i
    cusolverDnHandle_t sh;
    if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS)
      return fail(FPP_ERR_CUDA, "cusolverDnCreate failed");
    struct SGuard {
      cusolverDnHandle_t h;
      ~SGuard() { cusolverDnDestroy(h); }
    } sg{sh};
    FPP_CUSOLVER_LK(cusolverDnSetStream(sh, st));
    FPP_TRY(dLU.reserve(sizeof(double) * nn));
    FPP_TRY(dX.reserve(sizeof(double) * nn));
    FPP_CUDA(cudaMemcpyAsync(dLU.ptr, dKuu.ptr, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    FPP_CUDA(cudaMemcpyAsync(dX.ptr, dKuu.ptr, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    int lwork = 0;
    FPP_CUSOLVER_LK(cusolverDnDgetrf_bufferSize(sh, n, n, dLU.as<double>(), n, &lwork));
    FPP_TRY(dwork.reserve(sizeof(double) * std::max(lwork, 1)));
    FPP_TRY(dpiv.reserve(sizeof(int) * n));
    FPP_TRY(dinfo.reserve(sizeof(int) * 2));
    FPP_CUSOLVER_LK(cusolverDnDgetrf(sh, n, n, dLU.as<double>(), n, dwork.as<double>(),
                                     dpiv.as<int>(), dinfo.as<int>()));
    // Kuu is symmetric: its row-major and column-major forms agree
    FPP_CUSOLVER_LK(cusolverDnDgetrs(sh, CUBLAS_OP_N, n, n, dLU.as<double>(), n, dpiv.as<int>(),
                                     dX.as<double>(), n, dinfo.as<int>() + 1));
    for (int i = 0; i < nk; i++) {
      k_diag_sum<<<1, 256, 0, st>>>(n, koff[i], koff[i + 1] - koff[i], dX.as<double>(),
                                    dtmp.as<double>() + n + i);
      FPP_CUDA(cudaGetLastError());
    }
    int info[2] = {0, 0};
    std::vector<double> fro((size_t)kLkBlocks * nk, 0.0);
    FPP_CUDA(cudaMemcpyAsync(info, dinfo.ptr, sizeof(info), cudaMemcpyDeviceToHost, st));
    FPP_CUDA(cudaMemcpyAsync(tr_kinv.data(), dtmp.as<double>() + n, sizeof(double) * nk,
                             cudaMemcpyDeviceToHost, st));
    FPP_CUDA(cudaMemcpyAsync(fro.data(), dfro.ptr, sizeof(double) * fro.size(),
                             cudaMemcpyDeviceToHost, st));
    FPP_CUDA(cudaStreamSynchronize(st));
    if (info[0] != 0) return fail(FPP_ERR_NUMERIC, "Kuu is singular (LU)");
    for (int i = 0; i < nk; i++) {
      if (koff[i + 1] == koff[i]) {
        tr_kinv[i] = 0.0;
        continue;
      }
      for (int b = 0; b < kLkBlocks; b++) tr_kuu_sigma[i] += fro[(size_t)i * kLkBlocks + b];
    }
  }
  if (KnK && m) {
    // Kuf one_x Kuf^T for x = e, f, s (row-major n x n)
    DevBuf dM, dC;
    FPP_TRY(dM.reserve(sizeof(double) * (size_t)n * m));
    FPP_TRY(dC.reserve(sizeof(double) * (size_t)n * n));
    for (int t = 0; t < 3; t++) {
      const long long nm = (long long)n * m;
      k_mask_kind<<<(unsigned)((nm + 255) / 256), 256, 0, st>>>(n, m, dKuf.as<double>(),
                                                               dkind.as<int>(), t,
                                                               dM.as<double>());
      FPP_CUDA(cudaGetLastError());
      FPP_CUBLAS_LK(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, n, n, m, &one, dKuf.as<double>(), m,
                                dM.as<double>(), m, &zero, dC.as<double>(), n));
      FPP_CUDA(cudaMemcpyAsync(KnK + (size_t)t * n * n, dC.ptr, sizeof(double) * (size_t)n * n,
                               cudaMemcpyDeviceToHost, st));
      FPP_CUDA(cudaStreamSynchronize(st));
    }
  } else if (KnK) {
    std::fill(KnK, KnK + (size_t)3 * n * n, 0.0);
  }
  std::vector<double> part((size_t)kLkBlocks * kLkSums);
  FPP_CUDA(cudaMemcpyAsync(part.data(), dpart.ptr, sizeof(double) * part.size(),
                           cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  double S[kLkSums] = {0};
  for (int b = 0; b < kLkBlocks; b++)
    for (int k = 0; k < kLkSums; k++) S[k] += part[(size_t)b * kLkSums + k];
  const double data_fit = -0.5 * S[0];
  const double constant = -0.5 * (double)m * std::log(6.283185307179586476925);
  double noise_det = 0.0;
  if (want_gradient) {
    noise_det = -2.0 * ((double)cnt[0] * std::log(std::fabs(noise[0])) +
                        (double)cnt[1] * std::log(std::fabs(noise[1])) +
                        (double)cnt[2] * std::log(std::fabs(noise[2])));
  } else {
    for (int t = 0; t < 3; t++) noise_det += (double)cnt[t] * std::log(inv_var[t]);
  }
  double kuu_inv_det = 0.0, sigma_inv_det = 0.0;
  for (int i = 0; i < n; i++) {
    kuu_inv_det -= 2 * std::log(std::fabs(L_diag[i]));
    sigma_inv_det += 2 * std::log(std::fabs(R_inv_diag[i]));
  }
  const double complexity = 0.5 * (noise_det + kuu_inv_det + sigma_inv_det);
  out[0] = complexity + data_fit + constant;
  out[1] = data_fit;
  out[2] = complexity;
  out[3] = constant;
  if (want_gradient) {
    for (int i = 0; i < nk; i++) {
      const double g = 2.0 / hyps[i];
      double tx = 0.0;
      for (int t = 0; t < 3; t++) tx += S[8 + 4 * i + t] * inv_var[t];
      const double tr_pi_sigma = 2.0 * g * tx + g * tr_kuu_sigma[i];
      const double cg = 0.5 * g * tr_kinv[i] - 0.5 * tr_pi_sigma;
      const double dg = g * S[7 + 4 * i] - 0.5 * g * a_kuu_a[i];
      out[4 + i] = cg + dg;
    }
    for (int t = 0; t < 3; t++) {
      const double s3 = noise[t] * noise[t] * noise[t];
      out[4 + nk + t] = (-(double)cnt[t] / noise[t] + S[4 + t] / s3) + S[1 + t] / s3;
    }
  }
  return FPP_OK;
}

}  // namespace

extern "C" int fpp_likelihood_gradient_stable(
    int32_t n, int32_t m, const double *Kuf, const double *Kuu, const double *y,
    const int32_t *label_kind, const double *alpha, const double *Sigma,
    const double *L_diag, const double *R_inv_diag, const double *hyps,
    int32_t want_gradient, double *out, double *KnK, void *stream) {
  const int32_t koff[2] = {0, n};
  return likelihood_core(n, m, Kuf, Kuu, y, label_kind, alpha, Sigma, L_diag, R_inv_diag, 1,
                         koff, hyps, want_gradient, out, KnK, (cudaStream_t)stream);
}

extern "C" int fpp_likelihood_gradient_stable_kernels(
    int32_t n, int32_t m, const double *Kuf, const double *Kuu, const double *y,
    const int32_t *label_kind, const double *alpha, const double *Sigma,
    const double *L_diag, const double *R_inv_diag, int32_t n_kernels,
    const int32_t *kernel_offsets, const double *hyps, int32_t want_gradient, double *out,
    double *KnK, void *stream) {
  return likelihood_core(n, m, Kuf, Kuu, y, label_kind, alpha, Sigma, L_diag, R_inv_diag,
                         n_kernels, kernel_offsets, hyps, want_gradient, out, KnK,
                         (cudaStream_t)stream);
}
