// C ABI: error reporting, device buffers, Structure and B2 handles.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "b2_kernels.h"
#include "capi_state.h"
#include "common.cuh"
#include "internal.h"

namespace fpp {

static thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? FPP_ERR_OOM : FPP_ERR_CUDA;
}

DevBuf::~DevBuf() {
  if (ptr) cudaFree(ptr);
}

int DevBuf::reserve(size_t n) {
  if (n <= bytes && ptr) return FPP_OK;
  if (ptr) {
    cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  size_t want = n < 256 ? 256 : n;
  cudaError_t e = cudaMalloc(&ptr, want);
  if (e != cudaSuccess) {
    ptr = nullptr;
    cudaGetLastError();
    return fail(FPP_ERR_OOM, "device allocation of " + std::to_string(want) +
                                 " bytes failed");
  }
  bytes = want;
  return FPP_OK;
}

int ensure_tables(cudaStream_t stream) {
  // the harmonic normalisation and B3 coupling tables live in constant memory
  // of this module; upload them once per device (under a lock: host threads
  // may make their first call on a device at the same time)
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static bool uploaded[kMaxDev] = {false};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(FPP_ERR_CUDA, "no CUDA device");
  if (dev < 0 || dev >= kMaxDev) return fail(FPP_ERR_UNSUPPORTED, "device index beyond 63");
  std::lock_guard<std::mutex> lock(mu);
  if (uploaded[dev]) return FPP_OK;
  if (upload_harmonic_tables(stream) != 0)
    return fail(FPP_ERR_CUDA, "upload of harmonic tables failed");
  if (upload_descriptor_tables(stream) != 0)
    return fail(FPP_ERR_CUDA, "upload of B3 coupling tables failed");
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "upload of harmonic tables");
  uploaded[dev] = true;
  return FPP_OK;
}

int prepare_structure(fpp_structure *s, cudaStream_t stream) {
  FPP_TRY(ensure_tables(stream));
  s->st.mark(0, stream);
  bool reused = false;
  int rc = update_neighbors(s->st, stream, &reused);
  s->st.mark(1, stream);
  s->st.ev_nb = s->st.profile;
  return rc;
}

}  // namespace fpp

using namespace fpp;

extern "C" {

const char *fpp_last_error(void) { return g_last_error.c_str(); }

int fpp_version(void) { return FPP_VERSION; }

int fpp_structure_create(const double *cell, const int32_t *species,
                         const double *positions, int32_t noa, double cutoff,
                         void *stream, fpp_structure **out) {
  if (!out || !cell) return fail(FPP_ERR_INVALID, "null argument");
  *out = nullptr;
  if (noa < 0) return fail(FPP_ERR_INVALID, "noa < 0");
  if (noa > 0 && (!species || !positions)) return fail(FPP_ERR_INVALID, "null argument");
  for (int i = 0; i < noa; i++)
    if (species[i] < 0 || species[i] >= 1 << 16)
      return fail(FPP_ERR_INVALID, "species out of range");
  for (long long k = 0; k < 3ll * noa; k++)
    if (!std::isfinite(positions[k])) return fail(FPP_ERR_NUMERIC, "positions are not finite");
  auto *s = new fpp_structure();
  StructureState &st = s->st;
  st.noa = noa;
  st.base_cutoff = cutoff;
  int rc = make_cell_info(cell, cutoff, &st.ci);
  if (rc != FPP_OK) {
    delete s;
    return rc;
  }
  st.species_host.assign(species, species + noa);
  int smax = 0;
  for (int i = 0; i < noa; i++) smax = std::max(smax, species[i] + 1);
  st.n_species_max = smax;
  cudaStream_t cs = (cudaStream_t)stream;
  if ((rc = st.positions.reserve(sizeof(double) * 3 * std::max(noa, 1))) != FPP_OK ||
      (rc = st.species.reserve(sizeof(int) * std::max(noa, 1))) != FPP_OK) {
    delete s;
    return rc;
  }
  cudaError_t e = cudaSuccess;
  if (noa > 0) {
    e = cudaMemcpyAsync(st.positions.ptr, positions, sizeof(double) * 3 * noa,
                        cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(st.species.ptr, species, sizeof(int) * noa,
                          cudaMemcpyHostToDevice, cs);
  }
  if (e != cudaSuccess) {
    delete s;
    return cuda_fail(e, "structure upload");
  }
  rc = prepare_structure(s, cs);
  if (rc == FPP_OK) rc = check_status(st, cs, "neighbor list");
  if (rc != FPP_OK) {
    delete s;
    return rc;
  }
  *out = s;
  return FPP_OK;
}

int fpp_structure_set_positions(fpp_structure *s, const double *positions,
                                int positions_on_device, void *stream) {
  if (!s || (!positions && s->st.noa > 0)) return fail(FPP_ERR_INVALID, "null argument");
  cudaStream_t cs = (cudaStream_t)stream;
  if (s->st.noa > 0)
    FPP_CUDA(cudaMemcpyAsync(s->st.positions.ptr, positions,
                             sizeof(double) * 3 * s->st.noa,
                             positions_on_device ? cudaMemcpyDeviceToDevice
                                                 : cudaMemcpyHostToDevice,
                             cs));
  s->version++;
  FPP_TRY(prepare_structure(s, cs));
  return FPP_OK;
}

int fpp_structure_set_skin(fpp_structure *s, double skin, void *stream) {
  if (!s) return fail(FPP_ERR_INVALID, "null structure");
  if (!(skin >= 0) || !std::isfinite(skin)) return fail(FPP_ERR_INVALID, "skin must be >= 0");
  StructureState &st = s->st;
  CellInfo ci;
  FPP_TRY(make_cell_info(st.ci.cell, st.base_cutoff + skin, &ci));
  st.ci = ci;
  st.skin = skin;
  st.have_build = false;
  s->version++;
  return prepare_structure(s, (cudaStream_t)stream);
}

int fpp_structure_neighbor_stats(const fpp_structure *s, int64_t *builds, int64_t *reuses,
                                 double *list_cutoff) {
  if (!s) return fail(FPP_ERR_INVALID, "null structure");
  if (builds) *builds = s->st.n_builds;
  if (reuses) *reuses = s->st.n_reuses;
  if (list_cutoff) *list_cutoff = s->st.ci.cutoff;
  return FPP_OK;
}

int fpp_structure_set_profiling(fpp_structure *s, int on) {
  if (!s) return fail(FPP_ERR_INVALID, "null structure");
  StructureState &S = s->st;
  if (on && !S.ev[0])
    for (auto &e : S.ev) FPP_CUDA(cudaEventCreate(&e));
  S.profile = on != 0;
  S.ev_nb = S.ev_pred = false;
  return FPP_OK;
}

int fpp_structure_stage_times(fpp_structure *s, double *ms4) {
  if (!s || !ms4) return fail(FPP_ERR_INVALID, "null argument");
  StructureState &S = s->st;
  for (int k = 0; k < 4; k++) ms4[k] = 0.0;
  if (!S.ev[0]) return FPP_OK;
  float t;
  if (S.ev_nb) {
    FPP_CUDA(cudaEventSynchronize(S.ev[1]));
    FPP_CUDA(cudaEventElapsedTime(&t, S.ev[0], S.ev[1]));
    ms4[0] = t;
  }
  if (S.ev_pred) {
    FPP_CUDA(cudaEventSynchronize(S.ev[5]));
    FPP_CUDA(cudaEventElapsedTime(&t, S.ev[2], S.ev[3]));
    ms4[1] = t;
    FPP_CUDA(cudaEventElapsedTime(&t, S.ev[3], S.ev[4]));
    ms4[2] = t;
    FPP_CUDA(cudaEventElapsedTime(&t, S.ev[4], S.ev[5]));
    ms4[3] = t;
  }
  return FPP_OK;
}

int fpp_structure_destroy(fpp_structure *s) {
  delete s;
  return FPP_OK;
}

int fpp_structure_info(const fpp_structure *s, int32_t *noa, int64_t *n_neighbors,
                       int32_t *sweep, double *volume) {
  if (!s) return fail(FPP_ERR_INVALID, "null structure");
  if (noa) *noa = s->st.noa;
  if (n_neighbors) *n_neighbors = s->st.n_pairs;
  if (sweep) *sweep = s->st.ci.sweep;
  if (volume) *volume = s->st.ci.volume;
  return FPP_OK;
}

int fpp_structure_get_neighbors(const fpp_structure *s, int32_t *neighbor_count,
                                int32_t *cumulative_neighbor_count,
                                int32_t *structure_indices, int32_t *neighbor_species,
                                double *relative_positions, double *wrapped_positions) {
  if (!s) return fail(FPP_ERR_INVALID, "null structure");
  const StructureState &st = s->st;
  const int noa = st.noa;
  const int64_t np = st.n_pairs;
  FPP_TRY(ensure_rel64(const_cast<StructureState &>(st), nullptr));
  FPP_CUDA(cudaDeviceSynchronize());
  std::vector<int> off(noa + 1, 0);
  if (noa > 0)
    FPP_CUDA(cudaMemcpy(off.data(), st.nbr_offset.ptr, sizeof(int) * (noa + 1),
                        cudaMemcpyDeviceToHost));
  if (neighbor_count)
    for (int i = 0; i < noa; i++) neighbor_count[i] = off[i + 1] - off[i];
  if (cumulative_neighbor_count)
    for (int i = 0; i <= noa; i++) cumulative_neighbor_count[i] = off[i];
  if (np > 0) {
    if (structure_indices)
      FPP_CUDA(cudaMemcpy(structure_indices, st.nbr_j.ptr, sizeof(int) * np,
                          cudaMemcpyDeviceToHost));
    if (neighbor_species)
      FPP_CUDA(cudaMemcpy(neighbor_species, st.nbr_s.ptr, sizeof(int) * np,
                          cudaMemcpyDeviceToHost));
    if (relative_positions) {
      static_assert(sizeof(dvec4) == 4 * sizeof(double), "dvec4 layout");
      FPP_CUDA(cudaMemcpy(relative_positions, st.nbr_rel.ptr, sizeof(dvec4) * np,
                          cudaMemcpyDeviceToHost));
    }
  }
  if (wrapped_positions && noa > 0) {
    std::vector<dvec4> w(noa);
    FPP_CUDA(cudaMemcpy(w.data(), st.wrapped.ptr, sizeof(dvec4) * noa,
                        cudaMemcpyDeviceToHost));
    for (int i = 0; i < noa; i++) {
      wrapped_positions[3 * i] = w[i].x;
      wrapped_positions[3 * i + 1] = w[i].y;
      wrapped_positions[3 * i + 2] = w[i].z;
    }
  }
  return FPP_OK;
}

int fpp_b2_create(const char *radial_basis, const char *cutoff_function,
                  const double *radial_hyps, int32_t n_radial_hyps,
                  const double *cutoff_hyps, int32_t n_cutoff_hyps,
                  const int32_t *descriptor_settings, const double *cutoffs,
                  fpp_b2 **out) {
  (void)cutoff_hyps;
  (void)n_cutoff_hyps;
  if (!out || !radial_basis || !cutoff_function || !radial_hyps || !descriptor_settings)
    return fail(FPP_ERR_INVALID, "null argument");
  *out = nullptr;
  if (std::string(radial_basis) != "chebyshev")
    return fail(FPP_ERR_UNSUPPORTED, "radial basis '" + std::string(radial_basis) +
                                         "' is not implemented (chebyshev only)");
  int kind;
  if (std::string(cutoff_function) == "quadratic")
    kind = kQuadratic;
  else if (std::string(cutoff_function) == "cosine")
    kind = kCosine;
  else
    return fail(FPP_ERR_UNSUPPORTED, "cutoff function '" + std::string(cutoff_function) +
                                         "' is not implemented (quadratic, cosine)");
  if (n_radial_hyps < 2) return fail(FPP_ERR_INVALID, "radial_hyps needs {r1, rcut}");
  const int ns = descriptor_settings[0], N = descriptor_settings[1],
            lmax = descriptor_settings[2];
  if (ns < 1 || ns > kMaxSpecies) return fail(FPP_ERR_CAPACITY, "n_species must be 1..8");
  if (N < 1 || N > kMaxN) return fail(FPP_ERR_CAPACITY, "N must be 1..16");
  if (lmax < 0 || lmax > kMaxL) return fail(FPP_ERR_CAPACITY, "lmax must be 0..8");
  auto *b = new fpp_b2();
  B2Args &a = b->args;
  std::memset(&a, 0, sizeof(a));
  a.n_species = ns;
  a.N = N;
  a.lmax = lmax;
  a.H = (lmax + 1) * (lmax + 1);
  const int nr = ns * N;
  a.n_d = nr * (nr + 1) / 2 * (lmax + 1);
  a.cutoff_kind = kind;
  a.window = 64;
  a.r1 = radial_hyps[0];
  b->rcut = radial_hyps[1];
  for (int i = 0; i < ns * ns; i++) {
    double v = cutoffs ? cutoffs[i] : radial_hyps[1];
    if (!(v > 0) || !std::isfinite(v)) {
      delete b;
      return fail(FPP_ERR_INVALID, "cutoffs must be positive");
    }
    a.cutoffs[(i / ns) * ns + (i % ns)] = v;
    b->max_cutoff = std::max(b->max_cutoff, v);
  }
  fill_fp32_cutoffs(a);
  // (n1, n2 >= n1) table in the reference's counter order (b2.cpp:209-231)
  std::vector<int> tab;
  for (int n1 = 0; n1 < nr; n1++)
    for (int n2 = n1; n2 < nr; n2++) tab.push_back(n1 | (n2 << 16));
  b->pair_tab_host = tab;
  *out = b;
  return FPP_OK;
}

int fpp_b3_create(const char *radial_basis, const char *cutoff_function,
                  const double *radial_hyps, int32_t n_radial_hyps,
                  const double *cutoff_hyps, int32_t n_cutoff_hyps,
                  const int32_t *descriptor_settings, fpp_b2 **out) {
  if (!out || !descriptor_settings) return fail(FPP_ERR_INVALID, "null argument");
  *out = nullptr;
  if (descriptor_settings[2] < 0 || descriptor_settings[2] > 4)
    return fail(FPP_ERR_CAPACITY, "B3 lmax must be 0..4 (b3.cpp:150-160)");
  // one cutoff, radial_hyps[1], for every species pair (b3.cpp:258)
  fpp_b2 *b = nullptr;
  FPP_TRY(fpp_b2_create(radial_basis, cutoff_function, radial_hyps, n_radial_hyps,
                        cutoff_hyps, n_cutoff_hyps, descriptor_settings, nullptr, &b));
  B2Args &a = b->args;
  const int nr = a.n_species * a.N;
  a.kind = kB3;
  a.n_ls = b3_n_ls_host(a.lmax);
  a.n_tri = nr * (nr + 1) * (nr + 2) / 6;
  a.n_d = a.n_tri * a.n_ls;
  // radial triples n1 <= n2 <= n3 in the reference's counter order (b3.cpp:176-178)
  std::vector<int> tab;
  for (int n1 = 0; n1 < nr; n1++)
    for (int n2 = n1; n2 < nr; n2++)
      for (int n3 = n2; n3 < nr; n3++) tab.push_back(n1 | (n2 << 8) | (n3 << 16));
  b->pair_tab_host = tab;
  *out = b;
  return FPP_OK;
}

int fpp_b2_destroy(fpp_b2 *b2) {
  delete b2;
  return FPP_OK;
}

int fpp_b2_n_descriptors(const fpp_b2 *b2, int32_t *n) {
  if (!b2 || !n) return fail(FPP_ERR_INVALID, "null argument");
  *n = b2->args.n_d;
  return FPP_OK;
}

}  // extern "C"
