// C ABI: the per-atom uncertainty of the LAMMPS compute flare/std/atom
// (lammps_plugins/compute_flare_std_atom.cpp:98-207) on LAMMPS-shaped arrays,
// and the coefficients it reads.
//
// Per listed atom i of species s with B2 vector p, |p|^2 >= 1e-8:
//   L_inv form (:185-202):  k_j = (dhat_j . phat)^power over the sparse set of
//       s (zero for the other species), var = 1 - sigma^2 |L_inv k|^2;
//   variance-map form (:178-183):  var = p^T M_s p / |p|^2 / sigma^2, the
//       power-2 energy form of compute_energy_and_u with M_s in place of beta;
//   std_i = sqrt(var), or -sqrt(-var) when var < 0.  Atoms with |p|^2 < 1e-8,
//   and every entry not in ilist, are 0.
// The variance map is NormalizedDotProduct::compute_varmap_coefficients
// (normalized_dot_product.cpp:761-850), power 1 only:
//   M_s = sigma^2 I [first sparse environment of s non-empty]
//         - sigma^4 Dhat_s^T (Kuu^-1)_ss Dhat_s,   Kuu^-1 = L_inv^T L_inv.
// Everything is FP64: var is the difference of two terms near 1 for an
// environment the sparse set covers, so the rounding of a lower precision
// would dominate the small variances this compute exists to report.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "b2_kernels.h"
#include "capi_state.h"
#include "common.cuh"
#include "internal.h"
#include "kernel_form.h"

namespace fpp {
namespace {

#define FPP_CUBLAS_STD(call)                                                 \
  do {                                                                       \
    cublasStatus_t _s = (call);                                              \
    if (_s != CUBLAS_STATUS_SUCCESS)                                         \
      return fail(FPP_ERR_CUDA, std::string("cuBLAS: ") + #call + " status " + \
                                    std::to_string((int)_s));                \
  } while (0)

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp per listed atom: var from the map form (phat . y, y = M phat) or
// from the L_inv form (q = |L_inv k|^2), then the signed square root.
__global__ void k_std_finish(int inum, const int *__restrict__ row_of_atom,
                             const double *__restrict__ norm, const double *__restrict__ phat,
                             const double *__restrict__ Y, int ldp, int nd,
                             const double *__restrict__ q, double sig2, int use_map,
                             double *__restrict__ std_out) {
  const int ii = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (ii >= inum) return;
  const int row = row_of_atom[ii];
  const double n = norm[ii];
  double var;
  if (use_map) {
    double acc = 0.0;
    for (int k = lane; k < nd; k += 32)
      acc = fma(phat[(size_t)row * ldp + k], Y[(size_t)row * ldp + k], acc);
    var = warp_sum(acc) / sig2;
  } else {
    var = 1.0 - sig2 * q[row];
  }
  if (lane == 0) {
    double v = 0.0;
    if (n * n >= 1e-8) v = var >= 0.0 ? sqrt(var) : -sqrt(-var);
    std_out[ii] = v;
  }
}

__global__ void k_add_diag(int n, double *__restrict__ M, double v) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) M[(size_t)k * n + k] += v;
}

}  // namespace
}  // namespace fpp

using namespace fpp;

extern "C" {

int fpp_model_set_L_inv(fpp_model *m, int32_t n, const double *L_inv) {
  if (!m || (n > 0 && !L_inv)) return fail(FPP_ERR_INVALID, "null argument");
  if (n != m->n_sparse_total)
    return fail(FPP_ERR_INVALID, "L_inv size does not match the sparse set");
  FPP_TRY(m->L_inv.reserve(sizeof(double) * std::max(1, n) * std::max(1, n)));
  if (n)
    FPP_CUDA(cudaMemcpy(m->L_inv.ptr, L_inv, sizeof(double) * (size_t)n * n,
                        cudaMemcpyHostToDevice));
  m->has_L_inv = true;
  // Kuu of one NormalizedDotProduct kernel is zero between species, so its
  // Cholesky factor and that factor's inverse are block diagonal; the
  // uncertainty products then run species block by species block
  bool blocks = true;
  for (int a = 0; a < m->n_species && blocks; a++) {
    const auto &sa = m->sp[a];
    for (int i = sa.sparse_offset; i < sa.sparse_offset + sa.n_sparse && blocks; i++)
      for (int j = 0; j < n; j++)
        if ((j < sa.sparse_offset || j >= sa.sparse_offset + sa.n_sparse) &&
            L_inv[(size_t)i * n + j] != 0.0) {
          blocks = false;
          break;
        }
  }
  m->L_inv_species_blocks = blocks;
  bool lower = true;
  for (int i = 0; i < n && lower; i++)
    for (int j = i + 1; j < n; j++)
      if (L_inv[(size_t)i * n + j] != 0.0) {
        lower = false;
        break;
      }
  m->L_inv_lower = lower;
  return FPP_OK;
}

int fpp_model_set_varmap(fpp_model *m, const double *varmap) {
  if (!m || !varmap) return fail(FPP_ERR_INVALID, "null argument");
  const size_t sz = (size_t)m->n_species * m->n_d * m->n_d;
  FPP_TRY(m->varmap.reserve(sizeof(double) * std::max<size_t>(sz, 1)));
  if (sz) FPP_CUDA(cudaMemcpy(m->varmap.ptr, varmap, sizeof(double) * sz, cudaMemcpyHostToDevice));
  m->has_varmap = true;
  return FPP_OK;
}

int fpp_model_compute_varmap(fpp_model *m, double *varmap, void *stream) {
  if (!m) return fail(FPP_ERR_INVALID, "null model");
  if (m->power != 1.0)
    return fail(FPP_ERR_UNSUPPORTED,
                "Mapping coefficients of the normalized dot product kernel are "
                "implemented for power 1 only.");
  if (!m->has_L_inv) return fail(FPP_ERR_INVALID, "L_inv not set (fpp_model_set_L_inv)");
  cudaStream_t st = (cudaStream_t)stream;
  const int nd = m->n_d, n = m->n_sparse_total;
  const size_t per = (size_t)nd * nd;
  FPP_TRY(m->varmap.reserve(sizeof(double) * std::max<size_t>(per * m->n_species, 1)));
  FPP_CUDA(cudaMemsetAsync(m->varmap.ptr, 0, sizeof(double) * per * m->n_species, st));
  cublasHandle_t h;
  FPP_TRY(get_cublas(m, st, &h));
  const double one = 1.0, zero = 0.0;
  const double sig2 = m->sigma * m->sigma, msig4 = -sig2 * sig2;
  DevBuf Kinv, T;
  for (int s = 0; s < m->n_species; s++) {
    const int S = m->sp[s].n_sparse, off = m->sp[s].sparse_offset;
    if (S == 0) continue;
    double *M = m->varmap.as<double>() + per * s;
    FPP_TRY(Kinv.reserve(sizeof(double) * (size_t)S * S));
    FPP_TRY(T.reserve(sizeof(double) * (size_t)S * nd));
    // (Kuu^-1)_ss = L_inv[:, blk]^T L_inv[:, blk]; rows above the block are
    // zero in the lower triangle
    const double *Lb = m->L_inv.as<double>() + off + (size_t)off * n;
    FPP_CUBLAS_STD(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, S, S, n - off, &one, Lb, n, Lb,
                               n, &zero, Kinv.as<double>(), S));
    // T = (Kuu^-1)_ss Dhat_s; the rows of empty environments are zero in
    // Dhat_s, which drops them from both sums as the reference's skips do
    FPP_CUBLAS_STD(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, nd, S, S, &one,
                               m->sp[s].d_dhat.as<double>(), nd, Kinv.as<double>(), S, &zero,
                               T.as<double>(), nd));
    // M = -sigma^4 Dhat_s^T T
    FPP_CUBLAS_STD(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, nd, nd, S, &msig4, T.as<double>(),
                               nd, m->sp[s].d_dhat.as<double>(), nd, &zero, M, nd));
    // the self-kernel term, added while visiting the pair (0, 0)
    if (m->sp[s].norms[0] >= 1e-8) {
      k_add_diag<<<(nd + 127) / 128, 128, 0, st>>>(nd, M, sig2);
      FPP_CUDA(cudaGetLastError());
    }
    FPP_CUDA(cudaStreamSynchronize(st));  // Kinv / T are reused by the next species
  }
  FPP_CUDA(cudaStreamSynchronize(st));
  m->has_varmap = true;
  if (varmap && per * m->n_species)
    FPP_CUDA(cudaMemcpy(varmap, m->varmap.ptr, sizeof(double) * per * m->n_species,
                        cudaMemcpyDeviceToHost));
  return FPP_OK;
}

int fpp_std_atom_compute(fpp_model *m, int32_t nlocal, int32_t nall, const double *x,
                         const int32_t *type, int32_t inum, const int32_t *ilist,
                         const int32_t *numneigh, const int32_t *neighbors,
                         int32_t use_map, double *stds, void *stream) {
  if (!m) return fail(FPP_ERR_INVALID, "null model");
  if (m->args.kind != kB2)
    return fail(FPP_ERR_UNSUPPORTED, "flare/std/atom evaluates B2 models only");
  if (nall > 0 && !stds) return fail(FPP_ERR_INVALID, "null output");
  if (use_map && !m->has_varmap)
    return fail(FPP_ERR_INVALID, "variance map not set (fpp_model_set_varmap)");
  if (!use_map && !m->has_L_inv)
    return fail(FPP_ERR_INVALID, "L_inv not set (fpp_model_set_L_inv)");
  cudaStream_t st = (cudaStream_t)stream;
  FPP_TRY(lammps_load(m, nlocal, nall, x, type, inum, ilist, numneigh, neighbors, st));
  for (int k = 0; k < nall; k++) stds[k] = 0.0;
  if (inum == 0) return FPP_OK;
  fpp_structure *s = &m->lammps->s;
  StructureState &S = s->st;
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  B2Args a = m->args;
  a.noa = inum;
  a.strict = 1;  // the pair style's filter rsq < rc^2 (single_bond_multiple_cutoffs)
  FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), false, st));
  const int nd = m->n_d, ldp = round_up(nd, 64), n = m->n_sparse_total;
  const double sig2 = m->sigma * m->sigma;
  cublasHandle_t h;
  FPP_TRY(get_cublas(m, st, &h));
  const double one = 1.0, zero = 0.0;
  const double *phat = S.phat64.as<double>();
  DevBuf q, rown, K, V, out;
  FPP_TRY(out.reserve(sizeof(double) * inum));
  if (use_map) {
    // y = M_s phat for the rows of species s (into V64, sized by forward64)
    for (int sp = 0; sp < m->n_species; sp++) {
      if (s->n_rows[sp] == 0) continue;
      FPP_CUBLAS_STD(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, nd, s->n_rows[sp], nd, &one,
                                 m->varmap.as<double>() + (size_t)sp * nd * nd, nd,
                                 phat + (size_t)s->row_off[sp] * ldp, ldp, &zero,
                                 S.V64.as<double>() + (size_t)s->row_off[sp] * ldp, ldp));
    }
  } else {
    const int R = s->total_rows;
    FPP_TRY(q.reserve(sizeof(double) * std::max(1, R)));
    FPP_TRY(rown.reserve(sizeof(double) * std::max(1, R)));
    FPP_CUDA(cudaMemsetAsync(q.ptr, 0, sizeof(double) * std::max(1, R), st));
    FPP_CUDA(cudaMemsetAsync(rown.ptr, 0, sizeof(double) * std::max(1, R), st));
    if (launch_gather_rows(inum, s->row_of_atom.as<int>(), S.norm64.as<double>(),
                           rown.as<double>(), st) != 0)
      return fail(FPP_ERR_CUDA, "gather launch failed");
    // atoms in chunks: K (rows x S_s) and V (rows x n) stay near 256 MB each
    const int chunk = std::max(128, (int)std::min<long long>(1 << 25, (1ll << 25) / std::max(1, n)));
    for (int sp = 0; sp < m->n_species; sp++) {
      const int Ss = m->sp[sp].n_sparse, off = m->sp[sp].sparse_offset, nsa = s->n_rows[sp];
      if (Ss == 0 || nsa == 0) continue;
      const int nv = n - off;  // rows of L_inv[:, blk] that can be non-zero
      for (int r0 = 0; r0 < nsa; r0 += chunk) {
        const int rc = std::min(chunk, nsa - r0);
        const int row0 = s->row_off[sp] + r0;
        FPP_TRY(K.reserve(sizeof(double) * (size_t)rc * Ss));
        FPP_TRY(V.reserve(sizeof(double) * (size_t)rc * nv));
        // z = phat . dhat_j, then k = z^power (sigma^2 = 1: the compute's
        // kernel vector carries no signal variance)
        FPP_CUBLAS_STD(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, Ss, rc, nd, &one,
                                   m->sp[sp].d_dhat.as<double>(), nd,
                                   phat + (size_t)row0 * ldp, ldp, &zero, K.as<double>(), Ss));
        if (launch_envs_block(rc, Ss, K.as<double>(), Ss, rown.as<double>() + row0,
                              m->sp[sp].d_norms.as<double>(), 1.0, m->power, K.as<double>(),
                              Ss, st) != 0)
          return fail(FPP_ERR_CUDA, "kernel-vector launch failed");
        // v = L_inv[:, blk] k for rows off..n-1 of L_inv
        FPP_CUBLAS_STD(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, nv, rc, Ss, &one,
                                   m->L_inv.as<double>() + off + (size_t)off * n, n,
                                   K.as<double>(), Ss, &zero, V.as<double>(), nv));
        if (launch_row_sq(rc, nv, V.as<double>(), nv, q.as<double>() + row0, st) != 0)
          return fail(FPP_ERR_CUDA, "row-norm launch failed");
        FPP_CUDA(cudaStreamSynchronize(st));  // K / V are reused by the next chunk
      }
    }
  }
  k_std_finish<<<(inum + 3) / 4, 128, 0, st>>>(inum, s->row_of_atom.as<int>(),
                                               S.norm64.as<double>(), phat,
                                               S.V64.as<double>(), ldp, nd, q.as<double>(),
                                               sig2, use_map ? 1 : 0, out.as<double>());
  FPP_CUDA(cudaGetLastError());
  std::vector<double> hs(inum);
  FPP_CUDA(cudaStreamSynchronize(st));
  FPP_TRY(check_status(S, st, "flare/std/atom"));
  FPP_CUDA(cudaMemcpy(hs.data(), out.ptr, sizeof(double) * inum, cudaMemcpyDeviceToHost));
  for (int ii = 0; ii < inum; ii++) stds[ilist[ii]] = hs[ii];
  return FPP_OK;
}

}  // extern "C"
