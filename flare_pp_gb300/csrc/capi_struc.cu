// C ABI: structure-structure kernels of the NormalizedDotProduct kernel,
// NormalizedDotProduct::struc_struc and ::self_kernel_struc
// (src/flare_pp/kernels/normalized_dot_product.cpp:212-578), in FP64.
//
// The reference accumulates, per central species and atom pair (i, j), the
// energy, force and stress blocks from the stored descriptor derivatives.
// Here that sum is one product of three matrices per species,
//
//   K += A1 . KV . A2^T,
//
// where KV ((1 + 3 P1) x (1 + 3 P2), P = descriptor pairs of the species) holds
// in its first row and column the energy/force terms (sum over the partner
// atom) and elsewhere the force/force terms kern_val(k, l) of
// normalized_dot_product.cpp:371-391 for derivative rows k of struc1 and l of
// struc2, and A ((1 + 3N + 6) x (1 + 3P)) maps derivative rows to outputs:
// +1 at the central atom's component, -1 at the neighbor's, -coord / volume
// at the stress entries (xx, xy, xz, yy, yz, zz), 1 for the energy.  The
// dense products run in cuBLAS DGEMM; KV is formed by one kernel from the
// GEMMs dot = P1 P2^T, fd1 = F1 P2^T, fd2 = F2 P1^T, ff = F1 F2^T of the
// reference.  Memory is quadratic in the pair count, as in the reference:
// these kernels serve small structures (tests, DTC variances).
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "b2_kernels.h"
#include "capi_state.h"
#include "common.cuh"
#include "internal.h"

namespace fpp {
namespace {

#define SS_CUBLAS(call)                                                      \
  do {                                                                       \
    cublasStatus_t _s = (call);                                              \
    if (_s != CUBLAS_STATUS_SUCCESS)                                         \
      return fail(FPP_ERR_CUDA, std::string("cuBLAS: ") + #call + " status " + \
                                    std::to_string((int)_s));                \
  } while (0)

int handle(cudaStream_t st, cublasHandle_t *out) {
  thread_local cublasHandle_t h = nullptr;
  if (!h) {
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) return fail(FPP_ERR_CUDA, "cublasCreate failed");
    cublasSetMathMode(h, CUBLAS_PEDANTIC_MATH);
  }
  if (cublasSetStream(h, st) != CUBLAS_STATUS_SUCCESS)
    return fail(FPP_ERR_CUDA, "cublasSetStream failed");
  *out = h;
  return FPP_OK;
}

// Row-major C (M x N) = op(A) op(B) + beta C through column-major cuBLAS.
int gemm_rm(cublasHandle_t h, bool ta, bool tb, int M, int N, int K, const double *A,
            int lda, const double *B, int ldb, double beta, double *C, int ldc) {
  if (M == 0 || N == 0) return FPP_OK;
  const double one = 1.0;
  SS_CUBLAS(cublasDgemm(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, N,
                        M, K, &one, B, ldb, A, lda, &beta, C, ldc));
  return FPP_OK;
}

__global__ void k_rows(int n_rows, int n_cols, const int *__restrict__ idx,
                       const double *__restrict__ in, double *__restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n_rows * n_cols) return;
  const int r = (int)(t / n_cols), c = (int)(t - (long long)r * n_cols);
  out[t] = in[(size_t)idx[r] * n_cols + c];
}

__global__ void k_pick(int n, const int *__restrict__ idx, const double *__restrict__ in,
                       double *__restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = in[idx[t]];
}

struct KVArgs {
  int n1, n2, r1, r2;  // atoms and derivative rows (3 per pair) of each side
  double sig2, power, empty;
  const double *dot, *a1, *a2, *fd1, *fd2, *ff, *sfd1, *sfd2;
  const int *own1, *own2;  // local atom of each derivative row
};

__device__ __forceinline__ bool kv_ok(const KVArgs &g, int i, int j) {
  return g.a1[i] >= g.empty && g.a2[j] >= g.empty;
}

// d k(i, j) / d r_l for a row l of struc2 (the energy/force factor of
// normalized_dot_product.cpp:299-306), times sigma^2 c2.
__device__ __forceinline__ double kv_ef(const KVArgs &g, int i, int j, int l) {
  const double ni = g.a1[i], nj = g.a2[j], nij = ni * nj;
  const double d = g.dot[(size_t)i * g.n2 + j];
  const double nd = d / nij;
  const double c2 = g.power * pow(nd, g.power - 1);
  const double f1 = g.fd2[(size_t)l * g.n1 + i] / nij;
  const double f2 = d * g.sfd2[l] / (ni * nj * nj * nj);
  return g.sig2 * c2 * (f1 - f2);
}

__device__ __forceinline__ double kv_fe(const KVArgs &g, int i, int j, int k) {
  const double ni = g.a1[i], nj = g.a2[j], nij = ni * nj;
  const double d = g.dot[(size_t)i * g.n2 + j];
  const double nd = d / nij;
  const double c2 = g.power * pow(nd, g.power - 1);
  const double f1 = g.fd1[(size_t)k * g.n2 + j] / nij;
  const double f2 = d * g.sfd1[k] / (nj * ni * ni * ni);
  return g.sig2 * c2 * (f1 - f2);
}

__global__ void k_kvhat(KVArgs g, double *__restrict__ KV) {
  const int cols = g.r2 + 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)(g.r1 + 1) * cols) return;
  const int row = (int)(t / cols), col = (int)(t - (long long)row * cols);
  double v = 0.0;
  if (row == 0 && col == 0) {
    for (int i = 0; i < g.n1; i++)
      for (int j = 0; j < g.n2; j++)
        if (kv_ok(g, i, j)) {
          const double nd = g.dot[(size_t)i * g.n2 + j] / (g.a1[i] * g.a2[j]);
          v += g.sig2 * pow(nd, g.power);
        }
  } else if (row == 0) {
    const int l = col - 1, j = g.own2[l];
    for (int i = 0; i < g.n1; i++)
      if (kv_ok(g, i, j)) v += kv_ef(g, i, j, l);
  } else if (col == 0) {
    const int k = row - 1, i = g.own1[k];
    for (int j = 0; j < g.n2; j++)
      if (kv_ok(g, i, j)) v += kv_fe(g, i, j, k);
  } else {
    const int k = row - 1, l = col - 1;
    const int i = g.own1[k], j = g.own2[l];
    if (kv_ok(g, i, j)) {
      const double ni = g.a1[i], nj = g.a2[j], nij = ni * nj;
      const double ni2 = ni * ni, nj2 = nj * nj;
      const double d = g.dot[(size_t)i * g.n2 + j];
      const double nd = d / nij;
      const double c1 = (g.power - 1) * g.power * pow(nd, g.power - 2);
      const double c2 = g.power * pow(nd, g.power - 1);
      const double fd1 = g.fd1[(size_t)k * g.n2 + j], fd2 = g.fd2[(size_t)l * g.n1 + i];
      const double s1 = g.sfd1[k], s2 = g.sfd2[l];
      const double v1 = fd1 / nij - nd * s1 / ni2;
      const double v2 = fd2 / nij - nd * s2 / nj2;
      const double v3 = g.ff[(size_t)k * g.r2 + l] / nij;
      const double v4 = s1 * fd2 / (ni2 * ni * nj);
      const double v5 = s2 * fd1 / (ni * nj2 * nj);
      const double v6 = s1 * s2 * nd / (ni2 * nj2);
      v = g.sig2 * (c1 * v1 * v2 + c2 * (v3 - v4 - v5 + v6));
    }
  }
  KV[t] = v;
}

// out[a] += sum_k A[a, k] T[k, a]  (diagonal of A . T), A row-major n x m,
// T row-major m x n.
__global__ void k_diag_prod(int n, int m, const double *__restrict__ A,
                            const double *__restrict__ T, double *__restrict__ out) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  double s = 0.0;
  for (int k = 0; k < m; k++) {
    const double x = A[(size_t)a * m + k];
    if (x != 0.0) s += x * T[(size_t)k * n + a];
  }
  out[a] += s;
}

// One structure's descriptors and stored derivatives, grouped by central
// species (b2.cpp:76-179 / b3.cpp:29-132 semantics).
struct Side {
  int noa = 0, n_out = 0;
  double volume = 0;
  std::vector<std::vector<int>> atoms;    // per species, atom indices
  std::vector<std::vector<int>> pairs;    // per species, descriptor-pair indices
  std::vector<int> pair_atom, pair_nbr;   // per descriptor pair
  std::vector<double> pair_xyz;           // per descriptor pair, 3 coordinates
  DevBuf dp, fdots;                       // (3 npl) x nd, 3 npl
  const double *p = nullptr, *norms = nullptr;
};

int build_side(fpp_b2 *b2, fpp_structure *s, cudaStream_t st, Side &D) {
  StructureState &S = s->st;
  const B2Args &a = b2->args;
  const int ns = a.n_species, nd = a.n_d;
  for (int i = 0; i < S.noa; i++)
    if (S.species_host[i] >= ns)
      return fail(FPP_ERR_INVALID, "structure species exceeds the descriptor's n_species");
  FPP_TRY(upload_pair_tab(b2->pair_tab, b2->pair_tab_host, st));
  FPP_TRY(forward64(s, a, b2->pair_tab.as<int>(), true, st));
  D.noa = S.noa;
  D.n_out = 1 + 3 * S.noa + 6;
  D.volume = S.ci.volume;
  D.p = S.p64.as<double>();
  D.norms = S.norm64.as<double>();
  std::vector<int> off(S.noa + 1, 0), nbr_i(S.n_pairs), nbr_j(S.n_pairs), nbr_s(S.n_pairs);
  std::vector<dvec4> rel(S.n_pairs);
  FPP_CUDA(cudaStreamSynchronize(st));
  if (S.noa)
    FPP_CUDA(cudaMemcpy(off.data(), S.nbr_offset.ptr, sizeof(int) * (S.noa + 1),
                        cudaMemcpyDeviceToHost));
  if (S.n_pairs) {
    FPP_CUDA(cudaMemcpy(nbr_i.data(), S.nbr_i.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(nbr_j.data(), S.nbr_j.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(nbr_s.data(), S.nbr_s.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(rel.data(), S.nbr_rel.ptr, sizeof(dvec4) * S.n_pairs, cudaMemcpyDeviceToHost));
  }
  D.atoms.assign(ns, {});
  D.pairs.assign(ns, {});
  std::vector<int> plist;
  for (int i = 0; i < S.noa; i++) {
    const int si = S.species_host[i];
    D.atoms[si].push_back(i);
    for (int p = off[i]; p < off[i + 1]; p++)
      if (rel[p].x <= a.cutoffs[si * ns + nbr_s[p]]) {
        D.pairs[si].push_back((int)plist.size());
        D.pair_atom.push_back(i);
        D.pair_nbr.push_back(nbr_j[p]);
        D.pair_xyz.push_back(rel[p].y);
        D.pair_xyz.push_back(rel[p].z);
        D.pair_xyz.push_back(rel[p].w);
        plist.push_back(p);
      }
  }
  const int npl = (int)plist.size();
  FPP_TRY(D.dp.reserve(sizeof(double) * 3 * (size_t)std::max(npl, 1) * nd));
  FPP_TRY(D.fdots.reserve(sizeof(double) * 3 * (size_t)std::max(npl, 1)));
  if (npl) {
    DevBuf d_plist;
    FPP_TRY(d_plist.reserve(sizeof(int) * npl));
    FPP_CUDA(cudaMemcpy(d_plist.ptr, plist.data(), sizeof(int) * npl, cudaMemcpyHostToDevice));
    B2Args aa = a;
    aa.noa = S.noa;
    if (launch_b2_dp(aa, npl, d_plist.as<int>(), S.nbr_i.as<int>(), S.nbr_s.as<int>(),
                     S.nbr_rel.as<dvec4>(), S.species.as<int>(), b2->pair_tab.as<int>(),
                     S.c64.as<double>(), S.p64.as<double>(), D.dp.as<double>(), nd,
                     D.fdots.as<double>(), st) != 0)
      return fail(FPP_ERR_CUDA, "stored-derivative kernel launch failed");
    FPP_CUDA(cudaStreamSynchronize(st));
  }
  return FPP_OK;
}

// Output map A (n_out x (1 + 3 P)) of one side's species block, row-major.
std::vector<double> output_map(const Side &D, int sp) {
  const std::vector<int> &pl = D.pairs[sp];
  const int cols = 1 + 3 * (int)pl.size();
  std::vector<double> A((size_t)D.n_out * cols, 0.0);
  A[0] = 1.0;
  const double vi = 1.0 / D.volume;
  const int sidx[3] = {0, 3, 5};
  for (size_t k = 0; k < pl.size(); k++) {
    const int q = pl[k];
    const int c = D.pair_atom[q], nb = D.pair_nbr[q];
    for (int m = 0; m < 3; m++) {
      const int col = 1 + 3 * (int)k + m;
      A[(size_t)(1 + 3 * c + m) * cols + col] += 1.0;
      A[(size_t)(1 + 3 * nb + m) * cols + col] -= 1.0;
      for (int p = m; p < 3; p++)
        A[(size_t)(1 + 3 * D.noa + sidx[m] + (p - m)) * cols + col] -=
            D.pair_xyz[3 * q + p] * vi;
    }
  }
  return A;
}

struct Block {
  DevBuf P, a, F, sfd, own;
  int n = 0, r = 0;
};

int gather_block(const Side &D, int sp, int nd, cudaStream_t st, Block &B) {
  const std::vector<int> &at = D.atoms[sp], &pl = D.pairs[sp];
  B.n = (int)at.size();
  B.r = 3 * (int)pl.size();
  std::vector<int> rows(B.r), own(B.r), local(D.noa, -1);
  for (int k = 0; k < B.n; k++) local[at[k]] = k;
  for (size_t k = 0; k < pl.size(); k++)
    for (int m = 0; m < 3; m++) {
      rows[3 * k + m] = 3 * pl[k] + m;
      own[3 * k + m] = local[D.pair_atom[pl[k]]];
    }
  DevBuf d_at, d_rows;
  FPP_TRY(B.P.reserve(sizeof(double) * std::max<size_t>(1, (size_t)B.n * nd)));
  FPP_TRY(B.a.reserve(sizeof(double) * std::max(1, B.n)));
  FPP_TRY(B.F.reserve(sizeof(double) * std::max<size_t>(1, (size_t)B.r * nd)));
  FPP_TRY(B.sfd.reserve(sizeof(double) * std::max(1, B.r)));
  FPP_TRY(B.own.reserve(sizeof(int) * std::max(1, B.r)));
  FPP_TRY(d_at.reserve(sizeof(int) * std::max(1, B.n)));
  FPP_TRY(d_rows.reserve(sizeof(int) * std::max(1, B.r)));
  if (B.n) FPP_CUDA(cudaMemcpy(d_at.ptr, at.data(), sizeof(int) * B.n, cudaMemcpyHostToDevice));
  if (B.r) {
    FPP_CUDA(cudaMemcpy(d_rows.ptr, rows.data(), sizeof(int) * B.r, cudaMemcpyHostToDevice));
    FPP_CUDA(cudaMemcpy(B.own.ptr, own.data(), sizeof(int) * B.r, cudaMemcpyHostToDevice));
  }
  if (B.n) {
    const long long t = (long long)B.n * nd;
    k_rows<<<(unsigned)((t + 255) / 256), 256, 0, st>>>(B.n, nd, d_at.as<int>(), D.p,
                                                         B.P.as<double>());
    k_pick<<<ceil_div(B.n, 256), 256, 0, st>>>(B.n, d_at.as<int>(), D.norms, B.a.as<double>());
  }
  if (B.r) {
    const long long t = (long long)B.r * nd;
    k_rows<<<(unsigned)((t + 255) / 256), 256, 0, st>>>(B.r, nd, d_rows.as<int>(),
                                                         D.dp.as<double>(), B.F.as<double>());
    k_pick<<<ceil_div(B.r, 256), 256, 0, st>>>(B.r, d_rows.as<int>(), D.fdots.as<double>(),
                                               B.sfd.as<double>());
  }
  FPP_CUDA(cudaGetLastError());
  FPP_CUDA(cudaStreamSynchronize(st));  // index buffers are freed on return
  return FPP_OK;
}

// K (n1o x n2o, row-major, device) = sum over species of A1 KV A2^T; with
// diag != nullptr only the diagonal of the (square) result is accumulated.
int struc_kernel(fpp_b2 *b2, double sigma, double power, fpp_structure *s1,
                 fpp_structure *s2, cudaStream_t st, DevBuf &K, DevBuf *diag) {
  const int nd = b2->args.n_d, ns = b2->args.n_species;
  Side D1, D2;
  FPP_TRY(build_side(b2, s1, st, D1));
  const bool same = (s1 == s2);
  if (!same) FPP_TRY(build_side(b2, s2, st, D2));
  const Side &E2 = same ? D1 : D2;
  const int n1o = D1.n_out, n2o = E2.n_out;
  cublasHandle_t h;
  FPP_TRY(handle(st, &h));
  if (diag) {
    FPP_TRY(diag->reserve(sizeof(double) * n1o));
    FPP_CUDA(cudaMemsetAsync(diag->ptr, 0, sizeof(double) * n1o, st));
  } else {
    FPP_TRY(K.reserve(sizeof(double) * (size_t)n1o * n2o));
    FPP_CUDA(cudaMemsetAsync(K.ptr, 0, sizeof(double) * (size_t)n1o * n2o, st));
  }
  const double sig2 = sigma * sigma;
  for (int sp = 0; sp < ns; sp++) {
    Block B1, B2s;
    FPP_TRY(gather_block(D1, sp, nd, st, B1));
    FPP_TRY(gather_block(E2, sp, nd, st, B2s));
    if (B1.n == 0 || B2s.n == 0) continue;
    const int n1 = B1.n, n2 = B2s.n, r1 = B1.r, r2 = B2s.r;
    DevBuf dot, fd1, fd2, ff, KV, A1, A2, T;
    FPP_TRY(dot.reserve(sizeof(double) * (size_t)n1 * n2));
    FPP_TRY(fd1.reserve(sizeof(double) * std::max<size_t>(1, (size_t)r1 * n2)));
    FPP_TRY(fd2.reserve(sizeof(double) * std::max<size_t>(1, (size_t)r2 * n1)));
    FPP_TRY(ff.reserve(sizeof(double) * std::max<size_t>(1, (size_t)r1 * r2)));
    FPP_TRY(gemm_rm(h, false, true, n1, n2, nd, B1.P.as<double>(), nd, B2s.P.as<double>(), nd,
                    0.0, dot.as<double>(), n2));
    FPP_TRY(gemm_rm(h, false, true, r1, n2, nd, B1.F.as<double>(), nd, B2s.P.as<double>(), nd,
                    0.0, fd1.as<double>(), n2));
    FPP_TRY(gemm_rm(h, false, true, r2, n1, nd, B2s.F.as<double>(), nd, B1.P.as<double>(), nd,
                    0.0, fd2.as<double>(), n1));
    FPP_TRY(gemm_rm(h, false, true, r1, r2, nd, B1.F.as<double>(), nd, B2s.F.as<double>(), nd,
                    0.0, ff.as<double>(), r2));
    // the reference throws for power < 2 when a normalized dot product of two
    // non-empty environments is 0 (normalized_dot_product.cpp:283-288)
    if (power < 2) {
      std::vector<double> hd((size_t)n1 * n2), ha(n1), hb(n2);
      FPP_CUDA(cudaStreamSynchronize(st));
      FPP_CUDA(cudaMemcpy(hd.data(), dot.ptr, sizeof(double) * hd.size(), cudaMemcpyDeviceToHost));
      FPP_CUDA(cudaMemcpy(ha.data(), B1.a.ptr, sizeof(double) * n1, cudaMemcpyDeviceToHost));
      FPP_CUDA(cudaMemcpy(hb.data(), B2s.a.ptr, sizeof(double) * n2, cudaMemcpyDeviceToHost));
      for (int i = 0; i < n1; i++)
        for (int j = 0; j < n2; j++)
          if (ha[i] >= 1e-8 && hb[j] >= 1e-8 &&
              std::fabs(hd[(size_t)i * n2 + j] / (ha[i] * hb[j])) < 1e-8)
            return fail(FPP_ERR_NUMERIC,
                        "Dot product of descriptors is 0, and the negative power "
                        "function in force-force kernel diverges.");
    }
    FPP_TRY(KV.reserve(sizeof(double) * (size_t)(r1 + 1) * (r2 + 1)));
    KVArgs g;
    g.n1 = n1;
    g.n2 = n2;
    g.r1 = r1;
    g.r2 = r2;
    g.sig2 = sig2;
    g.power = power;
    g.empty = 1e-8;
    g.dot = dot.as<double>();
    g.a1 = B1.a.as<double>();
    g.a2 = B2s.a.as<double>();
    g.fd1 = fd1.as<double>();
    g.fd2 = fd2.as<double>();
    g.ff = ff.as<double>();
    g.sfd1 = B1.sfd.as<double>();
    g.sfd2 = B2s.sfd.as<double>();
    g.own1 = B1.own.as<int>();
    g.own2 = B2s.own.as<int>();
    const long long nkv = (long long)(r1 + 1) * (r2 + 1);
    k_kvhat<<<(unsigned)((nkv + 255) / 256), 256, 0, st>>>(g, KV.as<double>());
    FPP_CUDA(cudaGetLastError());
    const std::vector<double> hA1 = output_map(D1, sp), hA2 = output_map(E2, sp);
    FPP_TRY(A1.reserve(sizeof(double) * hA1.size()));
    FPP_TRY(A2.reserve(sizeof(double) * hA2.size()));
    FPP_CUDA(cudaMemcpyAsync(A1.ptr, hA1.data(), sizeof(double) * hA1.size(),
                             cudaMemcpyHostToDevice, st));
    FPP_CUDA(cudaMemcpyAsync(A2.ptr, hA2.data(), sizeof(double) * hA2.size(),
                             cudaMemcpyHostToDevice, st));
    // T = KV . A2^T  ((1 + r1) x n2o), then K += A1 . T
    FPP_TRY(T.reserve(sizeof(double) * (size_t)(r1 + 1) * n2o));
    FPP_TRY(gemm_rm(h, false, true, r1 + 1, n2o, r2 + 1, KV.as<double>(), r2 + 1,
                    A2.as<double>(), r2 + 1, 0.0, T.as<double>(), n2o));
    if (diag) {
      k_diag_prod<<<ceil_div(n1o, 128), 128, 0, st>>>(n1o, r1 + 1, A1.as<double>(),
                                                      T.as<double>(), diag->as<double>());
      FPP_CUDA(cudaGetLastError());
    } else {
      FPP_TRY(gemm_rm(h, false, false, n1o, n2o, r1 + 1, A1.as<double>(), r1 + 1,
                      T.as<double>(), n2o, 1.0, K.as<double>(), n2o));
    }
    FPP_CUDA(cudaStreamSynchronize(st));  // block buffers are freed on return
  }
  return FPP_OK;
}

int check_args(const fpp_b2 *b2, double sigma, double power) {
  if (!b2) return fail(FPP_ERR_INVALID, "null descriptor");
  if (!std::isfinite(sigma) || !std::isfinite(power))
    return fail(FPP_ERR_INVALID, "sigma and power must be finite");
  if (power < 1.0) return fail(FPP_ERR_UNSUPPORTED, "power < 1");
  return FPP_OK;
}

}  // namespace
}  // namespace fpp

using namespace fpp;

extern "C" int fpp_struc_struc(const fpp_b2 *b2, double sigma, double power,
                               fpp_structure *s1, fpp_structure *s2, double *kernel_mat,
                               void *stream) {
  FPP_TRY(check_args(b2, sigma, power));
  if (!s1 || !s2 || !kernel_mat) return fail(FPP_ERR_INVALID, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf K;
  FPP_TRY(struc_kernel(const_cast<fpp_b2 *>(b2), sigma, power, s1, s2, st, K, nullptr));
  FPP_CUDA(cudaStreamSynchronize(st));
  const size_t n = (size_t)(1 + 3 * s1->st.noa + 6) * (1 + 3 * s2->st.noa + 6);
  FPP_CUDA(cudaMemcpy(kernel_mat, K.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return FPP_OK;
}

extern "C" int fpp_self_kernel_struc(const fpp_b2 *b2, double sigma, double power,
                                     fpp_structure *s, double *kernel_vec, void *stream) {
  FPP_TRY(check_args(b2, sigma, power));
  if (!s || !kernel_vec) return fail(FPP_ERR_INVALID, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf K, d;
  FPP_TRY(struc_kernel(const_cast<fpp_b2 *>(b2), sigma, power, s, s, st, K, &d));
  FPP_CUDA(cudaStreamSynchronize(st));
  FPP_CUDA(cudaMemcpy(kernel_vec, d.ptr, sizeof(double) * (1 + 3 * s->st.noa + 6),
                      cudaMemcpyDeviceToHost));
  return FPP_OK;
}
