// Definitions of the opaque C ABI handles.
#pragma once
#include <cublas_v2.h>
#include <cuda_fp16.h>

#include <vector>

#include "b2_kernels.h"
#include "internal.h"

struct fpp_structure {
  fpp::StructureState st;
  int version = 0;
  // species-sorted row layout used by the contraction operands
  int layout_species = -1;
  std::vector<int> row_off;     // per species, first row (multiple of 128)
  std::vector<int> n_rows;      // per species, atom count
  int total_rows = 0;
  fpp::DevBuf row_of_atom;      // int32[noa]
};

// Device copies of LAMMPS-shaped arrays and the structure-shaped workspace
// the pair style and the uncertainty compute run on (owned by a model).
struct fpp_lammps_ws {
  fpp_structure s;
  fpp::DevBuf d_x, d_type, d_ilist, d_nbrs, d_f, d_vir, d_e;
};

struct fpp_b2 {
  fpp::B2Args args{};
  double rcut = 0;
  double max_cutoff = 0;
  std::vector<int> pair_tab_host;
  fpp::DevBuf pair_tab;  // uploaded lazily
};

struct fpp_model {
  fpp::B2Args args{};
  std::vector<int> pair_tab_host;
  fpp::DevBuf pair_tab;
  double sigma = 1, power = 2;
  int n_species = 1, n_d = 0;
  int ldb = 0;                          // padded row length of beta operands
  struct Species {
    int n_sparse = 0;
    int sparse_offset = 0;              // into the stacked alpha / R_inv
    std::vector<double> desc;           // unnormalised rows (host copy)
    std::vector<double> norms, alpha;
    fpp::DevBuf d_desc;                 // double[n_sparse * n_d] unnormalised
    fpp::DevBuf d_dhat;                 // double[n_sparse * n_d] normalised (0 if empty)
    fpp::DevBuf d_norms, d_alpha;       // double[n_sparse]
    fpp::DevBuf beta64;                 // double[n_d * ldb] dense symmetric
    fpp::DevBuf beta_hi, beta_lo;       // half[n_d_pad * ldb] split operands
    double beta_scale = 1;              // beta ~ (hi + lo/2048) / beta_scale
    std::vector<double> B_host;         // dense beta (n_d x n_d), power 2
  };
  std::vector<Species> sp;
  int beta_power = 0;                   // 0: no mapped coefficients yet
  // centre of the mixed-precision operand (per species): pbar, beta pbar,
  // pbar^T beta pbar; per species, whether pbar is already the mean of a
  // structure's environments (the mixed form centres each species on the
  // first structure it evaluates that contains the species)
  fpp::DevBuf pbar32, g32;
  std::vector<double> c0;
  std::vector<char> centred;
  fpp::DevBuf beta1;                    // double[n_species * n_d] (power 1)
  int n_sparse_total = 0;
  fpp::DevBuf R_inv;                    // double[n * n]
  bool has_R_inv = false;
  bool R_inv_upper = false;             // R_inv is upper triangular (as from the QR)
  // ComputeFlareStdAtom coefficients: L_inv (n x n, row-major lower
  // triangle) and the variance map (per species n_d x n_d, row-major)
  fpp::DevBuf L_inv;
  bool has_L_inv = false;
  bool L_inv_species_blocks = false;    // L_inv is zero across species blocks
  bool L_inv_lower = false;             // L_inv is lower triangular
  fpp::DevBuf varmap;
  bool has_varmap = false;
  fpp_lammps_ws *lammps = nullptr;      // LAMMPS-array workspace
  double max_memory = 0;                // pair style's device-memory cap (0: none)
  int kuf_ks = 0, kuf_threads = 0;      // tile shape of the last batched Kuf
  float kuf_ms = 0.f;                   // its Kuf kernel's CUDA-event time
  long long kuf_items = 0;              // (structure, atom) work items of it
  int last_pair_batches = 0;            // atom batches of the last pair compute
  fpp::OzakiWork oz;                    // kernel-form GEMM workspace
  fpp_structure *batch = nullptr;       // packed structure of a batched prediction
  fpp::DevBuf batch_aoff, batch_poff, batch_sums, batch_src;
  // envs_struc workspace (grown on demand, kept between calls)
  fpp::DevBuf es_rown, es_ndm, es_flags, es_pos, es_scan, es_plist, es_qatom, es_dmap,
      es_dp, es_sfd, es_fd;
  void *cublas = nullptr;               // cublasHandle_t
};

namespace fpp {
// constant-memory tables of the descriptor kernels (harmonic normalisations,
// B3 couplings), uploaded once per device before the first kernel that reads
// them
int ensure_tables(cudaStream_t stream);
int prepare_structure(fpp_structure *s, cudaStream_t stream);
int ensure_layout(fpp_structure *s, int n_species, cudaStream_t stream);
int mapped_core(fpp_model *m, fpp_structure *s, int precision, cudaStream_t st,
                int strict);
// Validates LAMMPS-shaped arrays (pair_flare.cpp:68-100: x, 1-based type,
// full neighbor list in ilist order) and loads them into m->lammps: pair
// list with the FP64 pair geometry, species per listed atom.
int lammps_load(fpp_model *m, int32_t nlocal, int32_t nall, const double *x,
                const int32_t *type, int32_t inum, const int32_t *ilist,
                const int32_t *numneigh, const int32_t *neighbors, cudaStream_t st);
int get_cublas(fpp_model *m, cudaStream_t st, cublasHandle_t *out);
int upload_pair_tab(DevBuf &buf, const std::vector<int> &tab, cudaStream_t st);
// FP64 forward pass: c64, norm64 (atom order), phat64 rows, p64 (atom order)
// when want_p.
int forward64(fpp_structure *s, const B2Args &a0, const int *pair_tab, bool want_p,
              cudaStream_t st);
// tile shape of the batched Kuf kernel (autotuned, cached per device and
// descriptor shape)
int kuf_tiles(fpp_model *m, const KufArgs &ka, int n_items, cudaStream_t st, int *ks,
              int *threads);
// FP64-accurate C = A B^T (row-major, device memory) on the tensor cores by
// exact fp16 digit planes (gemm_ozaki.cu); w holds the planes between calls.
// Queued on st; ozaki_check_status synchronizes st and reports a bounded
// wait that ran out.
// b_lower: B is lower triangular (the zero blocks are skipped).
int ozaki_dgemm_nt(int M, int N, int K, const double *A, long long lda, const double *B,
                   long long ldb, double *C, long long ldc, OzakiWork &w, cudaStream_t st,
                   bool b_lower = false);
int ozaki_check_status(OzakiWork &w, cudaStream_t st);
}  // namespace fpp
