// NormalizedDotProduct kernel form in FP64 (normalized_dot_product.cpp:115-210).
//
// Mean prediction through the adjoint (no stored derivatives):
//   z = phat D^T (cuBLAS),  E_i = sig2 sum_k a_k z^p,  C = sig2 a p z^(p-1),
//   G = C D (cuBLAS),       dE/dp_i = (G_i - (sum_k C_ik z_ik) phat_i) / |p_i|.
// Full kernel matrix (variance, training columns) through stored derivatives,
// as the reference does: fd = D dp^T (cuBLAS), then the energy, force and
// stress columns assembled per sparse environment.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernel_form.h"

namespace fpp {

#define LAUNCH_OK (cudaGetLastError() == cudaSuccess ? 0 : -1)

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double powi(double x, double p) {
  if (p == 1.0) return x;
  if (p == 2.0) return x * x;
  if (p == 0.0) return 1.0;
  return pow(x, p);
}

// One warp per operand row: E, C in place of z, zc = sum_k C z.
__global__ void k_kernel_c(int rows, int S, double *__restrict__ Z, int ldz,
                           const double *__restrict__ alpha_eff,
                           const double *__restrict__ rownorm, double sig2,
                           double power, double *__restrict__ E,
                           double *__restrict__ zc) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  const bool empty = !(rownorm[row] >= 1e-8);
  double e = 0.0, c = 0.0;
  for (int k = lane; k < S; k += 32) {
    const double z = Z[(size_t)row * ldz + k];
    const double a = alpha_eff[k];
    double ck = 0.0;
    if (!empty) {
      e += sig2 * a * powi(z, power);
      ck = sig2 * a * power * powi(z, power - 1.0);
      c += ck * z;
    }
    Z[(size_t)row * ldz + k] = ck;
  }
  e = wsum(e);
  c = wsum(c);
  if (lane == 0) {
    E[row] = e;
    zc[row] = c;
  }
}

__global__ void k_kernel_w(int rows, int nd, const double *__restrict__ G, int ldg,
                           const double *__restrict__ phat, int ldp,
                           const double *__restrict__ zc,
                           const double *__restrict__ rownorm, double *__restrict__ w,
                           int ldw) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)rows * nd) return;
  const int row = (int)(t / nd), d = (int)(t - (long long)row * nd);
  const double n = rownorm[row];
  double v = 0.0;
  if (n >= 1e-8) v = (G[(size_t)row * ldg + d] - zc[row] * phat[(size_t)row * ldp + d]) / n;
  w[(size_t)row * ldw + d] = v;
}

__global__ void k_gather_rows(int noa, const int *__restrict__ row_of_atom,
                              const double *__restrict__ v_atom,
                              double *__restrict__ v_row) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < noa) v_row[row_of_atom[i]] = v_atom[i];
}

// ---- full kernel matrix ----------------------------------------------------
// energy column: K[k, 0] += sig2 sum_i nd_ki^p   (one warp per sparse row)
__global__ void k_envs_energy(int S, int ns, const double *__restrict__ ndm, int ldn,
                              const double *__restrict__ snorm,
                              const double *__restrict__ anorm, double sig2,
                              double power, double *__restrict__ K, int ldk) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= S) return;
  double e = 0.0;
  if (snorm[k] >= 1e-8)
    for (int i = lane; i < ns; i += 32)
      if (anorm[i] >= 1e-8) e += sig2 * powi(ndm[(size_t)k * ldn + i], power);
  e = wsum(e);
  if (lane == 0) K[(size_t)k * ldk] += e;
}

// fkv[k, q*3+comp] = sig2 p nd^(p-1) (fd / |p_i| - nd sfd / |p_i|^2)
__global__ void k_envs_fkv(int S, int nq, double *__restrict__ fd, int ldf,
                           const double *__restrict__ ndm, int ldn,
                           const int *__restrict__ q_atom,
                           const double *__restrict__ sfd,
                           const double *__restrict__ snorm,
                           const double *__restrict__ anorm, double sig2,
                           double power) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)S * 3 * nq) return;
  const int k = (int)(t / (3ll * nq));
  const int r = (int)(t - (long long)k * 3 * nq);
  const int q = r / 3;
  const int i = q_atom[q];
  const double ni = anorm[i];
  double v = 0.0;
  if (snorm[k] >= 1e-8 && ni >= 1e-8) {
    const double nd = ndm[(size_t)k * ldn + i];
    const double dval = power * powi(nd, power - 1.0);
    v = sig2 * dval * (fd[(size_t)k * ldf + r] / ni - nd * sfd[r] / (ni * ni));
  }
  fd[(size_t)k * ldf + r] = v;
}

// force columns: K[k, 1+3a+c] += sum_{p in a} fkv[dmap p] - fkv[dmap rev p]
__global__ void k_envs_force(int S, int noa, const double *__restrict__ fkv, int ldf,
                             const int *__restrict__ offset,
                             const int *__restrict__ rev,
                             const int *__restrict__ dmap, double *__restrict__ K,
                             int ldk) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)S * noa) return;
  const int k = (int)(t / noa), a = (int)(t - (long long)k * noa);
  double F[3] = {0, 0, 0};
  for (int p = offset[a]; p < offset[a + 1]; p++) {
    const int q1 = dmap[p], q2 = rev[p] >= 0 ? dmap[rev[p]] : -1;
    for (int c = 0; c < 3; c++) {
      if (q1 >= 0) F[c] += fkv[(size_t)k * ldf + 3 * q1 + c];
      if (q2 >= 0) F[c] -= fkv[(size_t)k * ldf + 3 * q2 + c];
    }
  }
  for (int c = 0; c < 3; c++) K[(size_t)k * ldk + 1 + 3 * a + c] += F[c];
}

// stress columns: K[k, 1+3N+sc] -= sum_q fkv[q, c] r_q[c2] / V (one block per k)
__global__ void k_envs_stress(int S, int nq, const double *__restrict__ fkv, int ldf,
                              const int *__restrict__ q_pair,
                              const dvec4 *__restrict__ rel, double vol_inv, int noa,
                              double *__restrict__ K, int ldk) {
  const int k = blockIdx.x;
  if (k >= S) return;
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const dvec4 r = rel[q_pair[q]];
    const double rr[3] = {r.y, r.z, r.w};
    for (int c = 0; c < 3; c++) {
      const double f = fkv[(size_t)k * ldf + 3 * q + c];
      for (int c2 = 0; c2 < 3; c2++) acc[c * 3 + c2] += f * rr[c2];
    }
  }
  __shared__ double sm[9][128];
  for (int j = 0; j < 9; j++) sm[j][threadIdx.x] = acc[j];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int j = 0; j < 9; j++) sm[j][threadIdx.x] += sm[j][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int idx[6] = {0, 1, 2, 4, 5, 8};  // xx xy xz yy yz zz
    for (int j = 0; j < 6; j++)
      K[(size_t)k * ldk + 1 + 3 * noa + j] -= sm[idx[j]][0] * vol_inv;
  }
}

// envs_envs block: K[i][j] = sig2 z^p for non-empty environments
// (Z may alias K when ldz == ldk: each element is read and written by one thread)
__global__ void k_envs_block(int S1, int S2, const double *Z, int ldz,
                             const double *__restrict__ n1, const double *__restrict__ n2,
                             double sig2, double power, double *K, int ldk) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)S1 * S2) return;
  const int i = (int)(t / S2), j = (int)(t - (long long)i * S2);
  double v = 0.0;
  if (n1[i] >= 1e-8 && n2[j] >= 1e-8) v = sig2 * powi(Z[(size_t)i * ldz + j], power);
  K[(size_t)i * ldk + j] = v;
}

int launch_envs_block(int S1, int S2, const double *Z, int ldz, const double *n1,
                      const double *n2, double sig2, double power, double *K, int ldk,
                      cudaStream_t st) {
  long long n = (long long)S1 * S2;
  if (n == 0) return 0;
  k_envs_block<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(S1, S2, Z, ldz, n1, n2, sig2,
                                                           power, K, ldk);
  return LAUNCH_OK;
}

// row sums of squares: out[j] = sum_k V[j, k]^2
__global__ void k_row_sq(int rows, int cols, const double *__restrict__ V, int ldv,
                         double *__restrict__ out) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= rows) return;
  double s = 0.0;
  for (int k = lane; k < cols; k += 32) {
    const double v = V[(size_t)j * ldv + k];
    s += v * v;
  }
  s = wsum(s);
  if (lane == 0) out[j] = s;
}


int launch_kernel_c(int rows, int S, double *Z, int ldz, const double *alpha_eff,
                    const double *rownorm, double sig2, double power, double *E,
                    double *zc, cudaStream_t st) {
  if (rows == 0) return 0;
  k_kernel_c<<<ceil_div(rows, 4), 128, 0, st>>>(rows, S, Z, ldz, alpha_eff, rownorm,
                                                sig2, power, E, zc);
  return LAUNCH_OK;
}

int launch_kernel_w(int rows, int nd, const double *G, int ldg, const double *phat,
                    int ldp, const double *zc, const double *rownorm, double *w,
                    int ldw, cudaStream_t st) {
  long long n = (long long)rows * nd;
  if (n == 0) return 0;
  k_kernel_w<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rows, nd, G, ldg, phat, ldp,
                                                          zc, rownorm, w, ldw);
  return LAUNCH_OK;
}

int launch_gather_rows(int noa, const int *row_of_atom, const double *v_atom,
                       double *v_row, cudaStream_t st) {
  if (noa == 0) return 0;
  k_gather_rows<<<ceil_div(noa, 256), 256, 0, st>>>(noa, row_of_atom, v_atom, v_row);
  return LAUNCH_OK;
}

int launch_envs_energy(int S, int ns, const double *ndm, int ldn, const double *snorm,
                       const double *anorm, double sig2, double power, double *K,
                       int ldk, cudaStream_t st) {
  if (S == 0 || ns == 0) return 0;
  k_envs_energy<<<ceil_div(S, 4), 128, 0, st>>>(S, ns, ndm, ldn, snorm, anorm, sig2,
                                                power, K, ldk);
  return LAUNCH_OK;
}

int launch_envs_fkv(int S, int nq, double *fd, int ldf, const double *ndm, int ldn,
                    const int *q_atom, const double *sfd, const double *snorm,
                    const double *anorm, double sig2, double power, cudaStream_t st) {
  long long n = (long long)S * 3 * nq;
  if (n == 0) return 0;
  k_envs_fkv<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(S, nq, fd, ldf, ndm, ldn,
                                                         q_atom, sfd, snorm, anorm,
                                                         sig2, power);
  return LAUNCH_OK;
}

int launch_envs_force(int S, int noa, const double *fkv, int ldf, const int *offset,
                      const int *rev, const int *dmap, double *K, int ldk,
                      cudaStream_t st) {
  long long n = (long long)S * noa;
  if (n == 0) return 0;
  k_envs_force<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(S, noa, fkv, ldf, offset,
                                                           rev, dmap, K, ldk);
  return LAUNCH_OK;
}

int launch_envs_stress(int S, int nq, const double *fkv, int ldf, const int *q_pair,
                       const dvec4 *rel, double vol_inv, int noa, double *K, int ldk,
                       cudaStream_t st) {
  if (S == 0) return 0;
  k_envs_stress<<<S, 128, 0, st>>>(S, nq, fkv, ldf, q_pair, rel, vol_inv, noa, K, ldk);
  return LAUNCH_OK;
}

int launch_row_sq(int rows, int cols, const double *V, int ldv, double *out,
                  cudaStream_t st) {
  if (rows == 0) return 0;
  k_row_sq<<<ceil_div(rows, 4), 128, 0, st>>>(rows, cols, V, ldv, out);
  return LAUNCH_OK;
}

// 32 x 32 tiles through shared memory (the extra column avoids bank conflicts)
__global__ void k_transpose(int rows, int cols, const double *__restrict__ src, int lds,
                            double *__restrict__ dst, int ldd) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[k][threadIdx.x] = src[(size_t)r * lds + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[(size_t)c * ldd + r] = tile[threadIdx.x][k];
  }
}

int launch_transpose(int rows, int cols, const double *src, int lds, double *dst, int ldd,
                     cudaStream_t st) {
  if (rows <= 0 || cols <= 0) return 0;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose<<<grid, block, 0, st>>>(rows, cols, src, lds, dst, ldd);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

__global__ void k_pair_flags(long long n, const int *__restrict__ nbr_i,
                             const int *__restrict__ nbr_s, const dvec4 *__restrict__ rel,
                             const int *__restrict__ species, int sp, CutRow cut,
                             int *__restrict__ flags) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p > n) return;
  if (p == n) {
    flags[n] = 0;
    return;
  }
  flags[p] = (species[nbr_i[p]] == sp && rel[p].x <= cut.c[nbr_s[p]]) ? 1 : 0;
}

__global__ void k_pair_scatter(long long n, const int *__restrict__ flags,
                               const int *__restrict__ pos, const int *__restrict__ nbr_i,
                               const int *__restrict__ row_of_atom, int row0,
                               int *__restrict__ plist, int *__restrict__ qatom,
                               int *__restrict__ dmap) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (flags[p]) {
    const int q = pos[p];
    plist[q] = (int)p;
    qatom[q] = row_of_atom[nbr_i[p]] - row0;
    dmap[p] = q;
  } else {
    dmap[p] = -1;
  }
}

int launch_pair_flags(long long n_pairs, const int *nbr_i, const int *nbr_s, const dvec4 *rel,
                      const int *species, int sp, CutRow cut, int *flags, cudaStream_t st) {
  const int tb = 256;
  k_pair_flags<<<(int)((n_pairs + 1 + tb - 1) / tb), tb, 0, st>>>(n_pairs, nbr_i, nbr_s, rel,
                                                                  species, sp, cut, flags);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_pair_scatter(long long n_pairs, const int *flags, const int *pos, const int *nbr_i,
                        const int *row_of_atom, int row0, int *plist, int *qatom, int *dmap,
                        cudaStream_t st) {
  if (n_pairs <= 0) return 0;
  const int tb = 256;
  k_pair_scatter<<<(int)((n_pairs + tb - 1) / tb), tb, 0, st>>>(n_pairs, flags, pos, nbr_i,
                                                                row_of_atom, row0, plist,
                                                                qatom, dmap);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace fpp
