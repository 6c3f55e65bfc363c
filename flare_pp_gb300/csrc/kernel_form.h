// Launch interface of the FP64 kernel-form helpers.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace fpp {
int launch_kernel_c(int rows, int S, double *Z, int ldz, const double *alpha_eff,
                    const double *rownorm, double sig2, double power, double *E,
                    double *zc, cudaStream_t st);
int launch_kernel_w(int rows, int nd, const double *G, int ldg, const double *phat,
                    int ldp, const double *zc, const double *rownorm, double *w,
                    int ldw, cudaStream_t st);
int launch_gather_rows(int noa, const int *row_of_atom, const double *v_atom,
                       double *v_row, cudaStream_t st);
int launch_envs_energy(int S, int ns, const double *ndm, int ldn, const double *snorm,
                       const double *anorm, double sig2, double power, double *K,
                       int ldk, cudaStream_t st);
int launch_envs_fkv(int S, int nq, double *fd, int ldf, const double *ndm, int ldn,
                    const int *q_atom, const double *sfd, const double *snorm,
                    const double *anorm, double sig2, double power, cudaStream_t st);
int launch_envs_force(int S, int noa, const double *fkv, int ldf, const int *offset,
                      const int *rev, const int *dmap, double *K, int ldk,
                      cudaStream_t st);
int launch_envs_stress(int S, int nq, const double *fkv, int ldf, const int *q_pair,
                       const dvec4 *rel, double vol_inv, int noa, double *K, int ldk,
                       cudaStream_t st);
int launch_envs_block(int S1, int S2, const double *Z, int ldz, const double *n1,
                      const double *n2, double sig2, double power, double *K, int ldk,
                      cudaStream_t st);
int launch_row_sq(int rows, int cols, const double *V, int ldv, double *out,
                  cudaStream_t st);
// The descriptor pairs of one species: flags[p] = 1 when pair p's central
// atom has species sp and r <= cut[neighbor species] (b2.cpp:277), flags[n]
// = 0; then, from the exclusive scan pos of flags, plist[pos[p]] = p,
// qatom[pos[p]] = the central atom's row within its species block, dmap[p]
// = pos[p] or -1.
constexpr int kSelMaxSpecies = 8;
struct CutRow {
  double c[kSelMaxSpecies];
};
int launch_pair_flags(long long n_pairs, const int *nbr_i, const int *nbr_s, const dvec4 *rel,
                      const int *species, int sp, CutRow cut, int *flags, cudaStream_t st);
int launch_pair_scatter(long long n_pairs, const int *flags, const int *pos, const int *nbr_i,
                        const int *row_of_atom, int row0, int *plist, int *qatom, int *dmap,
                        cudaStream_t st);
// dst[c][r] = src[r][c] for r < rows, c < cols (row-major, leading dims)
int launch_transpose(int rows, int cols, const double *src, int lds, double *dst, int ldd,
                     cudaStream_t st);
}  // namespace fpp
