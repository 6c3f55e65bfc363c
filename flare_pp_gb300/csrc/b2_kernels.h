// Launch interface of the B2 forward / adjoint kernels.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "geom.cuh"

#include <cstddef>

namespace fpp {

constexpr int kMaxSpecies = 8;

enum DescKind { kB2 = 0, kB3 = 1 };

// Shape of a B2 or B3 descriptor (kind); for B3, n_d = n_tri * n_ls and the
// pair table passed to the kernels lists the radial triples instead of pairs.
struct B2Args {
  int noa;
  int kind;          // DescKind
  int n_ls, n_tri;   // B3: triangles (l1, l2, l3) and radial triples
  int n_species, N, lmax, H, n_d;
  int cutoff_kind;  // CutoffKind
  int window;       // neighbors staged per pass in the forward kernel
  int strict;       // pair filter rsq < rc^2 (pair style) instead of r <= rc (B2)
  double r1;
  double cutoffs[kMaxSpecies * kMaxSpecies];
  // FP32 copies for the FP32 kernels, and bounds such that a pair whose
  // FP32 distance is below cut_lo is surely inside the FP64 cutoff and one
  // above cut_hi surely outside (only pairs between are decided in FP64)
  float r1f;
  float cutoffs32[kMaxSpecies * kMaxSpecies];
  float cut_lo[kMaxSpecies * kMaxSpecies], cut_hi[kMaxSpecies * kMaxSpecies];
  // 1 / (rc - r1) per species pair as an FP32 hi/lo split (the Chebyshev
  // argument without a per-pair division or a rounded reciprocal)
  float cinv_hi[kMaxSpecies * kMaxSpecies], cinv_lo[kMaxSpecies * kMaxSpecies];
  size_t smem_per_warp;      // filled by the launcher
  size_t smem_per_warp_adj;  // filled by the launcher
};

// Row of u = dE/dc per atom, laid out like the single bond c:
// [species][n][lm].
inline __host__ __device__ int u_row_stride(const B2Args &a) {
  return a.n_species * a.N * a.H;
}

enum WMode { kWFromV2 = 0, kWFromV1 = 1, kWGiven = 2 };

struct AdjArgs {
  int mode;              // WMode
  int strict;            // pair filter rsq < rc^2 (pair style) instead of r <= rc
  double empty_thresh;   // on |p|^2 for the mapped forms
  float empty_thresh_f;  // the same for the FP32 kernels
  // mapped power 2: V = beta phat rows (one of V32 / V64), phat operands
  const float *V32;
  const double *V64;
  int ldv;
  const double *phat64;
  const __half *phat_hi, *phat_lo;  // mixed: centred operand delta = phat - pbar
  int ldp;
  const float *pbar;                // [n_species][n_d] centre of the mixed operand
  const float *gvec;                // [n_species][n_d] beta pbar
  double c0[kMaxSpecies];           // pbar^T beta pbar
  float c0_hi[kMaxSpecies], c0_lo[kMaxSpecies];  // the same as float-float
  // mapped power 1: beta vector per species [n_species][n_d]
  const double *beta1;
  // given dE/dp and energies per operand row (row stride ldp)
  const double *w_given;
  const double *e_given;
  DeviceStatus *status;  // staged adjoint: where a wait that ran out is recorded
};

struct Neigh {
  const int *offset;
  const dvec4 *rel;     // FP64 pairs (valid unless geom.wp is set)
  const float4 *rel32;
  const int *nbr_s;
  const int *rev;
  const NbGeom *geom;   // exact distances on demand (nullptr: rel is the FP64 table)
};

int upload_harmonic_tables(cudaStream_t stream);
void fill_fp32_cutoffs(B2Args &a);  // from r1 and cutoffs
int upload_descriptor_tables(cudaStream_t stream);  // B3 coupling tables
int b3_n_ls_host(int lmax);
size_t forward_smem_per_warp(const B2Args &a, size_t elem);
size_t adjoint_smem_per_warp(const B2Args &a, size_t elem);

template <typename T>
int launch_b2_forward(B2Args a, const Neigh &nb, const int *species,
                      const int *row_of_atom, const int *pair_tab, T *c_out,
                      T *p_out, double *norm_out, double *phat64, __half *phat_hi,
                      __half *phat_lo, int ldp, const float *pbar, cudaStream_t stream);

template <typename T>
int launch_b2_adjoint(B2Args a, const AdjArgs &g, const Neigh &nb,
                      const int *species, const int *row_of_atom,
                      const int *pair_tab, const T *c_in, const double *norm_in,
                      double *atom_e, T *pair_f, double *forces, double *atom_vir,
                      double *reduce_out, bool gather, T *u_buf, long long n_pairs,
                      const int *nbr_i, cudaStream_t stream);

// Kuf by the adjoint route (FP64): one persistent launch over work items
// (structure, atom) of a batch of training structures.
struct KufStruc {
  const double *c64;        // noa x sb single-bond coefficients, atom order
  const double *phat64;     // normalised B2 rows (species-sorted), stride ldp
  const double *norm64;     // noa
  const int *row_of_atom, *species, *offset, *nbr_j, *nbr_s;
  const dvec4 *rel;         // (r, x, y, z) of r_ij = x_j - x_i
  const int *force_col;     // noa: column of the atom's x force label, -1 none
  long long col_e, col_s;   // energy and first stress column, -1 none
  double vol_inv;
};
struct KufSpecies {
  const double *dhat;       // n_sparse x n_d normalised sparse descriptors
  const double *norms;      // n_sparse
  int n_sparse, row0;       // rows of this species in Kuf
};
struct KufArgs {
  B2Args a;
  const KufStruc *strucs;
  const int2 *items;        // (structure, atom)
  int n_items;
  KufSpecies sp[kMaxSpecies];
  const int *pair_tab;
  double sig2, power;
  int ldp;
  double *kuf;              // n_sparse_total x n_labels, row-major (added to)
  long long n_labels;
};
// ks sparse environments per pass and threads per block (the tile shape);
// shared-memory bytes the shape needs (0 if it does not fit).
size_t kuf_adjoint_smem(const B2Args &a, int ks, int threads);
int launch_kuf_adjoint(const KufArgs &k, int ks, int threads, int n_items, int item0,
                       cudaStream_t stream);

int launch_b2_dp(const B2Args &a, int npl, const int *plist, const int *nbr_i,
                 const int *nbr_s, const dvec4 *rel, const int *species,
                 const int *pair_tab, const double *c_in, const double *p_in,
                 double *dp, int ldd, double *force_dots, cudaStream_t stream);

}  // namespace fpp
