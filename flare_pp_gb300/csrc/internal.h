// Internal host-side state behind the C ABI handles.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/flare_pp_gb300.h"
#include "geom.cuh"

namespace fpp {

// Thread-local error reporting for the C ABI.
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
#define FPP_CUDA(call)                                    \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return ::fpp::cuda_fail(_e, #call); \
  } while (0)
#define FPP_TRY(call)                 \
  do {                                \
    int _rc = (call);                 \
    if (_rc != FPP_OK) return _rc;    \
  } while (0)

// Grow-only device buffer.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : ptr(o.ptr), bytes(o.bytes) {
    o.ptr = nullptr;
    o.bytes = 0;
  }
  ~DevBuf();
  int reserve(size_t n);  // at least n bytes; contents not preserved
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

// Workspace of the FP64-accurate tensor-core GEMM (digit planes and row
// powers of two of both operands, status word), kept between calls.
struct OzakiWork {
  DevBuf a, b, pa, pb, status;
};

// Cell quantities of Structure (structure.cpp:15-35), computed on the host
// with the oracle's operation order and no contraction.
struct CellInfo {
  double cell[9];
  double ct[9], ct_inv[9], cdot[9], cdot_inv[9];
  double volume;
  double height[3];  // distance between opposite faces
  double single_sweep_cutoff;
  double cutoff;
  int sweep;
  int nb[3];         // neighbor-search bins per lattice direction
};

int make_cell_info(const double *cell, double cutoff, CellInfo *ci);

// Small host-visible block (pinned, mapped) that kernels and copies fill
// with the values the host must read after a step: one synchronization
// instead of one per value.
struct HostReadback {
  int total_pairs;
  int overflow;
  int pad[2];
  int status[4];   // DeviceStatus
  double red[16];  // reduction outputs (energy, virial sums)
  // exact-distance geometry of the current neighbor list, read by the FP32
  // kernels (through the mapped pointer) only for pairs next to a cutoff;
  // written by the host after the neighbor build's synchronization
  NbGeom geom;
};

struct StructureState {
  int noa = 0;
  HostReadback *rb = nullptr;      // host pointer (nullptr until first use)
  HostReadback *rb_dev = nullptr;  // the same block as a device pointer
  int n_species_max = 0;
  CellInfo ci{};
  std::vector<int32_t> species_host;
  // atoms
  DevBuf positions;      // double[noa*3]
  DevBuf species;        // int32[noa]
  DevBuf wrapped;        // dvec4[noa] (x, y, z, unused)
  DevBuf wrapped32;      // float4[noa] (leading float of each coordinate)
  DevBuf wrapped_lo;     // float4[noa] (wrapped - wrapped32, the float-float tail)
  DevBuf frac;           // dvec4[noa] wrapped fractional coordinates
  DevBuf atom_bin;       // int32[noa]
  DevBuf bin_count;      // int32[n_bins]
  DevBuf bin_start;      // int32[n_bins + 1]
  DevBuf bin_cursor;     // int32[n_bins]
  DevBuf bin_atoms;      // int32[noa]
  DevBuf binned;         // float4[noa] positions in bin order, atom index in .w
  DevBuf slab;           // int64[noa * 256] per-atom sorted neighbor keys
  DevBuf flags;          // int32[4] device flags (slab overflow)
  // neighbors (CSR over atoms, reference order)
  int64_t n_pairs = 0;
  DevBuf nbr_count;      // int32[noa]
  DevBuf nbr_offset;     // int32[noa + 1]  (int64 when n_pairs >= 2^31 is rejected)
  DevBuf nbr_key_tmp;    // int64[n_pairs]
  DevBuf nbr_key;        // int64[n_pairs]  j * n_shift + shift index
  DevBuf nbr_i;          // int32[n_pairs]  central atom
  DevBuf nbr_j;          // int32[n_pairs]  neighbor atom (structure index)
  DevBuf nbr_s;          // int32[n_pairs]  neighbor species
  DevBuf nbr_rel;        // dvec4[n_pairs] (r, x, y, z); valid when rel64_valid
  bool rel64_valid = false;  // filled on demand by ensure_rel64
  DevBuf nbr_rel32;      // float4[n_pairs]  (x, y, z, r)
  DevBuf nbr_rev;        // int32[n_pairs]  index of the reverse pair
  DevBuf scan_tmp;       // CUB scratch
  DevBuf status;         // DeviceStatus
  // neighbor reuse within a skin (fpp_structure_set_skin): the list is built
  // at base_cutoff + skin; while no atom has moved more than skin / 2 since
  // that build, new positions only refresh the pair geometry
  double base_cutoff = 0, skin = 0;
  bool have_build = false;
  DevBuf pos_build, wrapped_build;       // positions and wrapped positions at the build
  DevBuf disp_max;                       // uint64: bits of max |x - x_build|^2
  long long n_builds = 0, n_reuses = 0;
  // descriptor / prediction workspace (sized by the callers)
  DevBuf c64, p64, norm64;            // FP64 single-bond, B2, norms
  DevBuf phat64;                      // FP64 normalised B2 rows (species-sorted)
  DevBuf c32, p32, pn64;              // FP32 single-bond, B2, FP64 norms
  DevBuf phat_hi, phat_lo;            // split fp16 operands (species-sorted)
  DevBuf order, order_inv;            // species-sorted atom order
  DevBuf V, V64;                      // beta p products
  DevBuf w64;                         // dE/dp (FP64 path)
  DevBuf u;                           // dE/dc per atom (adjoint)
  DevBuf pair_f;                      // double3/float per pair force
  DevBuf atom_e;                      // per-atom energies (double)
  DevBuf atom_vir;                    // per-atom virial partials (double[6])
  DevBuf forces;                      // double[noa*3]
  DevBuf reduce_out;                  // double[16]
  std::vector<int> species_count;     // per species atom count
  // stage timing (fpp_structure_set_profiling)
  bool profile = false;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  bool ev_nb = false, ev_pred = false;  // which stages were recorded last
  void mark(int k, cudaStream_t s) {
    if (profile && ev[k]) cudaEventRecord(ev[k], s);
  }
  // recorded after the neighbor readback: the host waits on it, not on the
  // work queued behind it
  cudaEvent_t nb_ready = nullptr;
  ~StructureState() {
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    if (nb_ready) cudaEventDestroy(nb_ready);
    if (rb) cudaFreeHost(rb);
  }
};

int build_neighbors(StructureState &st, cudaStream_t stream);
// build_neighbors, or (skin > 0, no atom moved more than skin / 2 since the
// last build) a refresh of the pair geometry of the existing list
int update_neighbors(StructureState &st, cudaStream_t stream, bool *reused);
// the FP64 pair table for the callers that return or consume FP64 geometry
int ensure_rel64(StructureState &st, cudaStream_t stream);
// exact-distance geometry of the structure's neighbor list (geom.cuh)
NbGeom nb_geom(const StructureState &st);
int check_status(StructureState &st, cudaStream_t stream, const char *what);
// allocate the readback block on first use
int ensure_readback(StructureState &st);
// report (and clear) a device status already copied into st.rb->status
int status_from_readback(StructureState &st, cudaStream_t stream, const char *what);

}  // namespace fpp
