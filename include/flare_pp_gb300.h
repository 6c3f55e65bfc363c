/*
 * flare_pp_gb300 -- C ABI of the GB300 (sm_103a) implementation of the
 * flare++ prediction path: periodic neighbor lists, the B2 descriptor, the
 * NormalizedDotProduct kernel against a sparse set, SparseGP mean / SOR
 * variance prediction, and the mapped-beta pair style.
 *
 * Conventions
 *  - Every entry point returns an int status: FPP_OK (0) or a negative
 *    FPP_ERR_* code; fpp_last_error() gives the message for the calling
 *    thread.
 *  - Matrices are row-major.  A cell is 3x3 with the lattice vectors as rows
 *    (the reference's Structure::cell).  Positions are noa x 3.
 *  - Pointers documented as "host" are read or written synchronously; the
 *    ones documented as "device" must be device memory and are used in
 *    stream order on `stream` (a cudaStream_t passed as void*, NULL for the
 *    legacy default stream).
 *  - The library allocates and owns the device memory behind each handle.
 *  - No entry point is safe to call concurrently on the same handle.
 *
 * Each declaration names the reference interface it replaces
 * (mir-group/flare_pp, paths relative to the project root).
 */
#ifndef FLARE_PP_GB300_H
#define FLARE_PP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FPP_VERSION 1

enum fpp_status {
  FPP_OK = 0,
  FPP_ERR_INVALID = -1,     /* bad argument: size, pointer, enum value */
  FPP_ERR_CUDA = -2,        /* a CUDA runtime or library call failed */
  FPP_ERR_OOM = -3,         /* a device allocation failed */
  FPP_ERR_TIMEOUT = -4,     /* a device-side wait ran out of its spin budget */
  FPP_ERR_UNSUPPORTED = -5, /* valid input this library does not implement */
  FPP_ERR_CAPACITY = -6,    /* input beyond a documented maximum */
  FPP_ERR_NUMERIC = -7      /* non-finite input, or a zero dot product with
                               power < 2 in the force-force kernel */
};

enum fpp_precision {
  FPP_PREC_FP64 = 0,  /* FP64 descriptors, FP64 contractions (cuBLAS DGEMM) */
  FPP_PREC_MIXED = 1  /* FP32 descriptors with compensated sums, tcgen05
                         contraction on split-fp16 operands, FP32 accumulate */
};

/* Message of the last failing call on this thread ("" if none). */
const char *fpp_last_error(void);
/* FPP_VERSION of the loaded library. */
int fpp_version(void);

/* ------------------------------------------------------------------------
 * Structure: periodic cell + neighbor list built on the GPU.
 * Replaces Structure::Structure(cell, species, positions, cutoff, ...)
 * (src/flare_pp/structure.h:92-97) with compute_neighbors
 * (src/flare_pp/structure.cpp:52-118), wrap_positions (:120-133) and
 * get_single_sweep_cutoff (:135-165).  Neighbor counts, order (j ascending,
 * then image shifts s1, s2, s3 ascending) and FP64 distances are identical
 * to the reference algorithm.
 * ---------------------------------------------------------------------- */
typedef struct fpp_structure fpp_structure;

/* cell: host 9 doubles; species: host noa ints in [0, n_species);
 * positions: host noa*3 doubles.  Builds the neighbor list (dist < cutoff,
 * dist != 0).  noa may be 0. */
int fpp_structure_create(const double *cell, const int32_t *species,
                         const double *positions, int32_t noa, double cutoff,
                         void *stream, fpp_structure **out);
/* New positions for the same cell, species and cutoff; rebuilds the
 * neighbor list.  positions_on_device != 0 means `positions` is a device
 * pointer (noa*3 doubles). */
int fpp_structure_set_positions(fpp_structure *s, const double *positions,
                                int positions_on_device, void *stream);
/* Neighbor reuse within a skin, as a molecular-dynamics engine keeps its
 * lists (the reference's pair style receives such lists from LAMMPS: neighbor
 * skin with neigh_modify check yes): the list is built at cutoff + skin, and
 * fpp_structure_set_positions then refreshes only the pair vectors while no
 * atom has moved more than skin / 2 since the last build (it rebuilds
 * otherwise).  Descriptors filter pairs by their own cutoffs, so predictions
 * equal those of a list at the cutoff up to FP64 rounding of the refreshed
 * vectors; the neighbor attributes then include the pairs in the skin, and the
 * wrapped positions are not re-wrapped between builds.  skin = 0 (the
 * default) restores the reference's semantics.  Rebuilds the list now.  No
 * counterpart in the reference's Structure. */
int fpp_structure_set_skin(fpp_structure *s, double skin, void *stream);
/* Neighbor builds and reuses since creation, and the list's cutoff (cutoff +
 * skin); each pointer may be NULL. */
int fpp_structure_neighbor_stats(const fpp_structure *s, int64_t *builds, int64_t *reuses,
                                 double *list_cutoff);
int fpp_structure_destroy(fpp_structure *s);
/* noa, total neighbors, sweep, volume. */
int fpp_structure_info(const fpp_structure *s, int32_t *noa,
                       int64_t *n_neighbors, int32_t *sweep, double *volume);
/* Host copies of the reference's neighbor attributes (structure.h:12-49);
 * any pointer may be NULL.  relative_positions is n_neighbors x 4
 * (r, x, y, z); wrapped_positions is noa x 3. */
int fpp_structure_get_neighbors(const fpp_structure *s, int32_t *neighbor_count,
                                int32_t *cumulative_neighbor_count,
                                int32_t *structure_indices,
                                int32_t *neighbor_species,
                                double *relative_positions,
                                double *wrapped_positions);

/* Stage timing (instrumentation; no counterpart in the reference).  With
 * profiling on, each prediction on this structure records CUDA events on its
 * stream around four stages; fpp_structure_stage_times returns the last
 * call's GPU milliseconds for: neighbor list, descriptor forward pass,
 * contraction (the GEMMs), adjoint (forces, virial, reductions). */
int fpp_structure_set_profiling(fpp_structure *s, int on);
int fpp_structure_stage_times(fpp_structure *s, double *ms4);

/* ------------------------------------------------------------------------
 * B2 descriptor settings.  Replaces B2::B2(radial_basis, cutoff_function,
 * radial_hyps, cutoff_hyps, descriptor_settings[, cutoffs])
 * (src/flare_pp/descriptors/b2.h:34-46, b2.cpp:13-50).
 * Supported: radial_basis "chebyshev"; cutoff_function "quadratic" or
 * "cosine".  descriptor_settings = {n_species, N, lmax}, lmax <= 8,
 * n_species * N <= 64.  cutoffs is n_species x n_species (NULL: every entry
 * radial_hyps[1]).
 * ---------------------------------------------------------------------- */
typedef struct fpp_b2 fpp_b2;

int fpp_b2_create(const char *radial_basis, const char *cutoff_function,
                  const double *radial_hyps, int32_t n_radial_hyps,
                  const double *cutoff_hyps, int32_t n_cutoff_hyps,
                  const int32_t *descriptor_settings, const double *cutoffs,
                  fpp_b2 **out);
/* B3 descriptor settings.  Replaces B3::B3(radial_basis, cutoff_function,
 * radial_hyps, cutoff_hyps, descriptor_settings)
 * (src/flare_pp/descriptors/b3.h:29-33, b3.cpp:12-27).  The handle is an
 * fpp_b2 of kind B3: every fpp_b2_* call and fpp_model_create accept it, and
 * compute the bispectrum of b3.cpp:134-240 in its place (one cutoff,
 * radial_hyps[1], for every species pair; lmax <= 4).
 * n_d = C(n_rad + 2, 3) * n_ls, n_ls = 1, 5, 15, 34, 65 for lmax = 0..4.
 * The coefficients are the reference's (descriptors/wigner3j.cpp), including
 * the entries its lmax = 4 table holds as 0. */
int fpp_b3_create(const char *radial_basis, const char *cutoff_function,
                  const double *radial_hyps, int32_t n_radial_hyps,
                  const double *cutoff_hyps, int32_t n_cutoff_hyps,
                  const int32_t *descriptor_settings, fpp_b2 **out);
int fpp_b2_destroy(fpp_b2 *b2);
/* n_d = n_rad (n_rad + 1) / 2 * (lmax + 1), n_rad = n_species * N (B2). */
int fpp_b2_n_descriptors(const fpp_b2 *b2, int32_t *n_descriptors);

/* B2::compute_struc (b2.cpp:76-179) on the GPU, in FP64.  Host outputs in
 * atom order (the caller regroups them by species): descriptors noa x n_d,
 * norms noa.  With with_derivatives != 0 it also returns the descriptor
 * neighbor list (pairs with r <= cutoffs[s_i][s_j], b2.cpp:277) and the
 * stored derivatives of b2.cpp:181-242:
 *   desc_neighbor_count        noa
 *   desc_neighbor_indices      n_desc_pairs        (structure index of j)
 *   desc_neighbor_coordinates  n_desc_pairs x 3
 *   force_dervs                3 n_desc_pairs x n_d (row 3*pair + comp)
 *   force_dots                 3 n_desc_pairs
 * n_desc_pairs is returned first through fpp_b2_pair_count.  Any output
 * pointer may be NULL. */
int fpp_b2_pair_count(const fpp_b2 *b2, fpp_structure *s, int64_t *n_desc_pairs,
                      void *stream);
int fpp_b2_compute(const fpp_b2 *b2, fpp_structure *s, double *descriptors,
                   double *norms, int32_t *desc_neighbor_count,
                   int32_t *desc_neighbor_indices,
                   double *desc_neighbor_coordinates, double *force_dervs,
                   double *force_dots, void *stream);

/* B2 descriptors with no device allocation (no counterpart in the reference).
 * For callers that may not allocate device memory when they need descriptors:
 * an MD engine whose memory pool owns the GPU (nothing may be cudaMalloc'd
 * behind its back), or a loop with a fixed memory budget decided up front.
 * All pointers are device memory supplied by the caller:
 *   species      n_atoms, in [0, n_species)
 *   offsets      n_atoms + 1 CSR offsets into the pair arrays
 *   rel          n_pairs x 4 doubles (r, x, y, z of r_ij = x_j - x_i), 32-byte
 *                aligned (the layout of fpp_structure_get_neighbors)
 *   nbr_species  n_pairs
 *   descriptors  n_atoms x n_d (output, FP64), norms n_atoms (output)
 * Pairs enter when r <= cutoffs[s_i][s_j], as in B2::compute_struc.  The
 * kernel's scratch lives in fixed device arrays of this library (8 MiB, held
 * by every GPU that loads it until the process exits), which limits a call to
 * n_atoms * n_species * N * (lmax+1)^2 <= 2^20 (and n_atoms <= 65536);
 * larger calls return FPP_ERR_CAPACITY.  The first call on a device does a
 * one-time set-up (it resolves the arrays' addresses, uploads constant tables
 * and synchronizes the stream): make it before any stream capture.  Calls
 * share the scratch, which keeps the last call's contents: two calls that
 * overlap on the GPU (different streams, or different threads) race. */
int fpp_b2_descriptors_noalloc(const fpp_b2 *b2, int32_t n_atoms,
                               const int32_t *species, const int32_t *offsets,
                               const double *rel, const int32_t *nbr_species,
                               double *descriptors, double *norms, void *stream);

/* ------------------------------------------------------------------------
 * Model: one NormalizedDotProduct kernel (sigma, power) over B2, with its
 * sparse set and weights.  Replaces the prediction state of
 * SparseGP(std::vector<Kernel*>, sigma_e, sigma_f, sigma_s)
 * (src/flare_pp/bffs/sparse_gp.h:48-49) over NormalizedDotProduct(sigma,
 * power) (src/flare_pp/kernels/normalized_dot_product.h:11-73).
 * ---------------------------------------------------------------------- */
typedef struct fpp_model fpp_model;

int fpp_model_create(const fpp_b2 *b2, double sigma, double power,
                     fpp_model **out);
int fpp_model_destroy(fpp_model *m);
/* Sparse environments of one species, as the rows of
 * ClusterDescriptor::descriptors[s] (descriptor.h:61-90), their norms and
 * the matching slice of SparseGP::alpha.  Host arrays. */
int fpp_model_set_sparse(fpp_model *m, int32_t species, int32_t n_sparse,
                         const double *descriptors, const double *norms,
                         const double *alpha);
/* R_inv of SparseGP::update_matrices_QR (sparse_gp.cpp:604-606), n x n with
 * n the total sparse count in species order; enables SOR variance. */
int fpp_model_set_R_inv(fpp_model *m, int32_t n, const double *R_inv);
/* Mapped coefficients of compute_map_coeff_pow2 / _pow1
 * (normalized_dot_product.cpp:645-759), computed on the GPU in FP64 from the
 * sparse set and alpha.  Needed by fpp_predict_mapped / fpp_pair_compute.
 * beta_packed (host, optional): n_species x n_d (n_d+1)/2 for power 2,
 * n_species x n_d for power 1, in the reference's packed layout. */
int fpp_model_compute_beta(fpp_model *m, double *beta_packed, void *stream);
/* Load mapped coefficients directly, in the potential file's packed layout
 * (pair_flare.cpp:363-395: off-diagonals stored doubled). */
int fpp_model_set_beta(fpp_model *m, int32_t power, const double *beta_packed);

/* ------------------------------------------------------------------------
 * Prediction.
 * ---------------------------------------------------------------------- */
/* NormalizedDotProduct::envs_struc (normalized_dot_product.cpp:115-210) for
 * the model's sparse set against the structure, FP64: kernel_mat is host,
 * n_sparse_total x (1 + 3 noa + 6), row-major. */
int fpp_envs_struc(fpp_model *m, fpp_structure *s, double *kernel_mat,
                   void *stream);

/* NormalizedDotProduct::envs_envs (normalized_dot_product.cpp:27-87): the
 * kernel between the sparse sets of two models over the same descriptor
 * (m1's sigma and power), FP64; kernel_mat is host, n1 x n2 row-major. */
int fpp_envs_envs(fpp_model *m1, fpp_model *m2, double *kernel_mat, void *stream);

/* SparseGP::predict_mean (sparse_gp.cpp:612-628) and, with variance_efs !=
 * NULL, predict_SOR (:630-649), in the kernel form, FP64.  mean_efs and
 * variance_efs are host arrays of 1 + 3 noa + 6: energy, forces, stress
 * (xx, xy, xz, yy, yz, zz). */
int fpp_predict(fpp_model *m, fpp_structure *s, double *mean_efs,
                double *variance_efs, void *stream);

/* SparseGP::compute_cluster_uncertainties (sparse_gp.cpp:93-133) for the
 * model's single kernel: per cluster (atom environment) the energy variance
 * k(c, c) - |L_inv k(sparse, c)|^2, FP64 on the GPU.  L_inv is the host
 * n x n (row-major) inverse Cholesky factor of Kuu + jitter I (the L_inv of
 * fpp_update_matrices_QR), n = the model's sparse-set size.  variances (host,
 * noa) are in cluster order: species by species, atoms in structure order.
 * This is SparseGP::predict_local_uncertainties' uncertainty
 * (sparse_gp.cpp:682-702). */
int fpp_local_uncertainties(fpp_model *m, fpp_structure *s, const double *L_inv,
                            int32_t n, double *variances, void *stream);

/* The energy of SparseGP::predict_SOR (sparse_gp.cpp:630-649) at MD sizes:
 * energy = k_E . alpha and energy_variance = |R_inv^T k_E|^2, the first
 * entries of mean_efs and variance_efs, with k_E[k] = sum over atoms i of
 * k(sparse k, atom i); and, with local_variances != NULL, the per-atom
 * variances of SparseGP::compute_cluster_uncertainties (sparse_gp.cpp:
 * 93-133), k(i, i) - |L_inv k(sparse, i)|^2, in structure atom order.  Only
 * the energy column of the kernel matrix is formed (no force or stress
 * columns), FP64 on the GPU; when L_inv is zero across species blocks (one
 * NormalizedDotProduct kernel) the L_inv products run block by block.
 * Requires fpp_model_set_R_inv for energy_variance and fpp_model_set_L_inv
 * for local_variances.  Outputs are host pointers; NULL skips one. */
int fpp_predict_energy_uncertainty(fpp_model *m, fpp_structure *s, double *energy,
                                   double *energy_variance, double *local_variances,
                                   void *stream);

/* SparseGP::update_Kuf / stack_Kuf for a batch of training structures
 * (sparse_gp.cpp:392-462, 464-552, 565-574): the sparse-environment columns
 * of each structure's labels, [E] [F of the listed atoms] [S], stacked in
 * structure order into kuf (host, n_sparse_total x n_labels, row-major),
 * FP64 on the GPU.  The columns are the envs_struc values of
 * normalized_dot_product.cpp:115-210, formed by the adjoint route (no
 * stored descriptor derivatives): one persistent launch over the (structure,
 * atom) work list of the whole batch, no synchronization per structure; the
 * kernel's tile shape (sparse environments per pass, threads per block) is
 * autotuned once per device and descriptor shape and cached in the file
 * $FPP_TUNE_CACHE (else $HOME/.cache/flare_pp_gb300/tiles.txt).  Additions
 * into other atoms' columns are FP64 atomics, so results vary between runs
 * at the level of FP64 rounding.  B2 models only.
 * label_mask[k]: bit 0 energy, bit 1 forces, bit 2 stress of structure k;
 * atom_offsets (n_structures + 1) and atoms list the force atoms of each
 * structure (the reference's atom_indices; NULL: every atom).  n_labels must
 * equal the total label count (FPP_ERR_INVALID otherwise). */
int fpp_kuf_batched(fpp_model *m, fpp_structure *const *structures,
                    int32_t n_structures, const int32_t *label_mask,
                    const int32_t *atom_offsets, const int32_t *atoms,
                    double *kuf, int64_t n_labels, void *stream);
/* The tile shape the last fpp_kuf_batched call on m used (sparse
 * environments per pass, threads per block), and (each may be NULL) the
 * CUDA-event time of its Kuf kernel in ms and its (structure, atom) work
 * items.  No counterpart in the reference (an instrumentation call). */
int fpp_model_kuf_tiles(const fpp_model *m, int32_t *ks, int32_t *threads,
                        float *kernel_ms, int64_t *n_items);

/* NormalizedDotProduct::struc_struc (normalized_dot_product.cpp:212-444):
 * the full energy/force/stress covariance of two structures, FP64, from the
 * descriptor's stored derivatives.  kernel_mat is a host array
 * (1 + 3 noa1 + 6) x (1 + 3 noa2 + 6), row-major.  FPP_ERR_NUMERIC where the
 * reference throws (power < 2 and a zero normalized dot product).  Memory
 * grows with the product of the two structures' pair counts, as in the
 * reference: meant for small structures. */
int fpp_struc_struc(const fpp_b2 *descriptor, double sigma, double power,
                    fpp_structure *s1, fpp_structure *s2, double *kernel_mat,
                    void *stream);

/* NormalizedDotProduct::self_kernel_struc (:446-578): the diagonal of
 * struc_struc(s, s), a host array of 1 + 3 noa + 6. */
int fpp_self_kernel_struc(const fpp_b2 *descriptor, double sigma, double power,
                          fpp_structure *s, double *kernel_vec, void *stream);

/* Energy, forces and stress of the same model through its mapped
 * coefficients (the pair style's evaluation, pair_flare.cpp:95-180, on the
 * periodic structure), in `precision`.  Outputs are host arrays unless
 * outputs_on_device != 0: energy (1), forces (noa x 3), stress (6, flare
 * order), atom_energies (noa, optional).  Requires fpp_model_compute_beta
 * or fpp_model_set_beta.  With device outputs the call returns without
 * synchronizing the stream (outputs are written in stream order); a
 * device-side error of such a call is reported by the next call that
 * synchronizes on the structure (fpp_structure_set_positions included).
 *
 * FPP_PREC_MIXED evaluates E_i = c0 + 2 g.delta + delta.(beta delta) on the
 * offset delta = phat - pbar from a per-species centre pbar (g = beta pbar,
 * c0 = pbar.g in FP64).  The tensor cores accumulate beta delta in FP32 with
 * truncation, so the energy error grows with |delta| |beta delta|: it is
 * smallest when pbar is the mean environment of the structures predicted.
 * So each species is centred on the first structure the mixed form evaluates
 * that contains it (the normalised mean of that structure's unit descriptors,
 * from an FP64 forward pass; a one-time cost that synchronizes the stream);
 * later structures reuse that centre.  fpp_model_compute_beta /
 * fpp_model_set_beta reset it; fpp_model_center_on sets it explicitly.
 * The centre is a numerical device: results equal the FP64 form's to within
 * the mixed form's error whatever it is. */
int fpp_predict_mapped(fpp_model *m, fpp_structure *s, int precision,
                       double *energy, double *forces, double *stress,
                       double *atom_energies, int outputs_on_device,
                       void *stream);
/* The mapped form of fpp_predict_mapped for a batch of structures of any
 * sizes in one pass (the batched prediction that pair_flare / SparseGP
 * callers otherwise loop over): the structures' atoms and neighbor lists are
 * packed into one structure, so the forward pass, the contraction and the
 * adjoint each run as one launch over all atoms; each structure's energy and
 * virial are then summed over its own atoms and pairs.  energies: n_structures
 * doubles; forces: 3 x (total atoms), the structures' atoms in order;
 * stresses: 6 x n_structures (xx xy xz yy yz zz); host memory, each may be
 * NULL.  Same precisions and results as fpp_predict_mapped per structure (up
 * to the order of the sums).  Synchronizes the stream. */
int fpp_predict_mapped_batched(fpp_model *m, fpp_structure *const *structures,
                               int32_t n_structures, int precision, double *energies,
                               double *forces, double *stresses, void *stream);

/* Recentre the mixed form on a structure: pbar of every species with atoms in
 * s becomes the normalised mean of their unit descriptors (FP64 forward pass,
 * synchronizes the stream).  Deterministic: later predictions depend only on
 * the model and the structures it was centred on.  No reference counterpart
 * (pair_flare.cpp evaluates in FP64 throughout). */
int fpp_model_center_on(fpp_model *m, fpp_structure *s, void *stream);

/* ------------------------------------------------------------------------
 * SparseGP::update_matrices_QR (src/flare_pp/bffs/sparse_gp.cpp:576-610) in
 * FP64 on the GPU (cuSOLVER):
 *   L = chol(Kuu + jitter I),  A = [diag(sqrt(noise)) Kuf^T ; L^T],  A = Q R,
 *   alpha = R^-1 Q^T [sqrt(noise) y ; 0],  R_inv = R^-1,  L_inv = L^-1.
 * Host arrays: Kuu n x n, Kuf n x m (row-major), y and noise_vector m (the
 * reference's 1/sigma^2 per label).  Outputs (host, each optional): alpha n,
 * R_inv n x n, L_inv n x n (row-major).  FPP_ERR_NUMERIC if Kuu + jitter I
 * is not positive definite.
 * ---------------------------------------------------------------------- */
int fpp_update_matrices_QR(int32_t n, int32_t m, const double *Kuu,
                           const double *Kuf, const double *y,
                           const double *noise_vector, double jitter,
                           double *alpha, double *R_inv, double *L_inv,
                           void *stream);

/* ------------------------------------------------------------------------
 * PairFLARE::compute(eflag, vflag) (lammps_plugins/pair_flare.cpp:68-184)
 * with LAMMPS-shaped host arrays: x is nall x 3 (owned then ghost atoms),
 * type is 1-based (nall), the full neighbor list is given as numneigh[inum]
 * and the concatenated neighbor indices (local or ghost, into x) in ilist
 * order.  Forces are ADDED into f (nall x 3); eng_vdwl receives the summed
 * energy, virial[6] the LAMMPS virial (xx, yy, zz, xy, xz, yz) from
 * ev_tally_xyz, eatom (optional, nall) the per-atom energies.  Requires
 * mapped coefficients on the model.
 * ---------------------------------------------------------------------- */
int fpp_pair_compute(fpp_model *m, int32_t nlocal, int32_t nall,
                     const double *x, const int32_t *type, int32_t inum,
                     const int32_t *ilist, const int32_t *numneigh,
                     const int32_t *neighbors, int precision, double *f,
                     double *eng_vdwl, double *virial, double *eatom,
                     void *stream);
/* Device-memory cap of the pair style (the MAXMEM of the Kokkos pair style,
 * pair_flare_kokkos.cpp:145-177 and :741): fpp_pair_compute then evaluates
 * the listed atoms in batches sized so that the mapped coefficients and the
 * per-atom buffers fit in `bytes` (the batches' sizes differ by at most one
 * atom, the first ones the larger); FPP_ERR_CAPACITY ("Not enough memory for
 * even a single atom!") if one atom does not fit.  0 (the default): one
 * batch.  fpp_model_pair_batches reports the batch count of the last call. */
int fpp_model_set_max_memory(fpp_model *m, double bytes);
int fpp_model_pair_batches(const fpp_model *m, int32_t *n_batches);

/* ------------------------------------------------------------------------
 * Training side: the log marginal likelihood and its hyperparameter gradient
 * for one NormalizedDotProduct kernel (and, below, for several), FP64 on the
 * GPU.
 * SparseGP::compute_likelihood_stable (sparse_gp.cpp:704-732) and, with
 * want_gradient, compute_likelihood_gradient_stable (sparse_gp.cpp:734-862).
 * Host inputs: Kuf n x m (row-major), Kuu n x n (the kernel matrix without
 * jitter), y m, label_kind m (0 energy, 1 force, 2 stress), alpha n,
 * Sigma n x n (= R_inv R_inv^T), L_diag n and R_inv_diag n (diagonals of
 * L_inv and R_inv from fpp_update_matrices_QR), hyps[4] = sigma, sigma_e,
 * sigma_f, sigma_s.  out[4] = log marginal likelihood, data fit, complexity
 * penalty, constant term; with want_gradient also out[4..7] = d/d hyps
 * (Kuu and Sigma are then required).  KnK (host, optional): 3 x n x n,
 * Kuf one_x Kuf^T for x = energy, force, stress (SparseGP::compute_KnK,
 * sparse_gp.cpp:888-922).  FPP_ERR_NUMERIC for a zero or non-finite
 * hyperparameter or a singular Kuu.
 * ---------------------------------------------------------------------- */
int fpp_likelihood_gradient_stable(int32_t n, int32_t m, const double *Kuf,
                                   const double *Kuu, const double *y,
                                   const int32_t *label_kind, const double *alpha,
                                   const double *Sigma, const double *L_diag,
                                   const double *R_inv_diag, const double *hyps,
                                   int32_t want_gradient, double *out, double *KnK,
                                   void *stream);
/* The same for a SparseGP with several NormalizedDotProduct kernels
 * (sparse_gp.h:48-49): kernel i owns rows [kernel_offsets[i],
 * kernel_offsets[i+1]) of Kuu (block diagonal) and Kuf, n_kernels <= 8;
 * hyps = sigma_0 .. sigma_{n_kernels-1}, sigma_e, sigma_f, sigma_s (the
 * order of SparseGP::set_hyperparameters, sparse_gp.cpp:1105-1140); out has
 * 4 + n_kernels + 3 entries: the four likelihood terms, then d/d hyps in
 * the same order. */
int fpp_likelihood_gradient_stable_kernels(
    int32_t n, int32_t m, const double *Kuf, const double *Kuu, const double *y,
    const int32_t *label_kind, const double *alpha, const double *Sigma,
    const double *L_diag, const double *R_inv_diag, int32_t n_kernels,
    const int32_t *kernel_offsets, const double *hyps, int32_t want_gradient, double *out,
    double *KnK, void *stream);

/* ------------------------------------------------------------------------
 * ComputeFlareStdAtom (lammps_plugins/compute_flare_std_atom.cpp): the
 * per-atom uncertainty of the LAMMPS compute flare/std/atom.
 * ---------------------------------------------------------------------- */
/* L_inv of the sparse set (the L_inverse file's block, read by
 * ComputeFlareStdAtom::read_L_inverse, compute_flare_std_atom.cpp:456-568):
 * host n x n row-major lower triangle, n = the model's sparse-set size. */
int fpp_model_set_L_inv(fpp_model *m, int32_t n, const double *L_inv);
/* NormalizedDotProduct::compute_varmap_coefficients
 * (normalized_dot_product.cpp:761-850) on the GPU in FP64 from the sparse
 * set, sigma and L_inv (Kuu^-1 = L_inv^T L_inv); power-1 models only
 * (FPP_ERR_UNSUPPORTED otherwise, with the reference's message).  varmap
 * (host, optional): n_species x n_d^2, row-major, the layout
 * SparseGP::write_varmap_coefficients writes (sparse_gp.cpp:1208-1281).
 * The map is kept on the model for fpp_std_atom_compute. */
int fpp_model_compute_varmap(fpp_model *m, double *varmap, void *stream);
/* Load a variance map (ComputeFlareStdAtom::read_file,
 * compute_flare_std_atom.cpp:345-454): n_species x n_d^2, row-major. */
int fpp_model_set_varmap(fpp_model *m, const double *varmap);
/* ComputeFlareStdAtom::compute_peratom (compute_flare_std_atom.cpp:98-207)
 * with the LAMMPS-shaped arrays of fpp_pair_compute.  use_map = 1: the
 * variance-map form, var = p.(M p) / |p|^2 / sigma^2; use_map = 0: the
 * L_inv form, var = 1 - sigma^2 |L_inv k|^2 with k_j = (dhat_j . phat)^power
 * over the sparse set of the atom's species.  stds (host, nall) receives
 * sqrt(var) (-sqrt(-var) when var < 0) at the listed atoms and 0 elsewhere
 * and for empty environments (|p|^2 < 1e-8).  FP64 on the GPU. */
int fpp_std_atom_compute(fpp_model *m, int32_t nlocal, int32_t nall,
                         const double *x, const int32_t *type, int32_t inum,
                         const int32_t *ilist, const int32_t *numneigh,
                         const int32_t *neighbors, int32_t use_map,
                         double *stds, void *stream);

/* FP64-accurate C = A B^T on the fp16 tensor cores: row-major A (M x K, row
 * stride lda), B (N x K, ldb), C (M x N, ldc).  Each row of A and of B is cut
 * into 11 exact 5-bit digit planes relative to its largest entry; the level
 * sums of the digit products are exact in the FP32 accumulators and are added
 * in FP64, so every product keeps ~55 bits of each operand relative to its
 * row's largest entry (the error bound of an FP64 GEMM, with |a_ik| |b_jk|
 * replaced by max_k |a_ik| max_k |b_jk|).  The kernel-form GEMMs of
 * envs_struc / predict_SOR (normalized_dot_product.cpp:140-143,
 * sparse_gp.cpp:630-649) run on it.  Entries must be finite.  on_device: A,
 * B, C are device pointers (queued on stream, then synchronized), else host
 * arrays. */
int fpp_dgemm_nt(int32_t M, int32_t N, int32_t K, const double *A, int64_t lda,
                 const double *B, int64_t ldb, double *C, int64_t ldc, int32_t on_device,
                 void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FLARE_PP_GB300_H */
