// C ABI: descriptors, model, predictions.
#include <cub/cub.cuh>
#include <cublas_v2.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "b2_kernels.h"
#include "capi_state.h"
#include "common.cuh"
#include "gemm_tc.h"
#include "internal.h"
#include "kernel_form.h"

namespace fpp {

static inline int round_up(int v, int m) { return (v + m - 1) / m * m; }
static int center_from_sparse(fpp_model *m);

#define FPP_CUBLAS(call)                                                     \
  do {                                                                       \
    cublasStatus_t _s = (call);                                              \
    if (_s != CUBLAS_STATUS_SUCCESS)                                         \
      return fail(FPP_ERR_CUDA, std::string("cuBLAS: ") + #call + " status " + \
                                    std::to_string((int)_s));                \
  } while (0)

int get_cublas(fpp_model *m, cudaStream_t st, cublasHandle_t *out) {
  if (!m->cublas) {
    cublasHandle_t h;
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS)
      return fail(FPP_ERR_CUDA, "cublasCreate failed");
    cublasSetMathMode(h, CUBLAS_PEDANTIC_MATH);
    m->cublas = h;
  }
  cublasHandle_t h = (cublasHandle_t)m->cublas;
  if (cublasSetStream(h, st) != CUBLAS_STATUS_SUCCESS)
    return fail(FPP_ERR_CUDA, "cublasSetStream failed");
  *out = h;
  return FPP_OK;
}

int upload_pair_tab(DevBuf &buf, const std::vector<int> &tab, cudaStream_t st) {
  if (buf.ptr) return FPP_OK;
  FPP_TRY(buf.reserve(sizeof(int) * tab.size()));
  FPP_CUDA(cudaMemcpyAsync(buf.ptr, tab.data(), sizeof(int) * tab.size(),
                           cudaMemcpyHostToDevice, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  return FPP_OK;
}

int ensure_layout(fpp_structure *s, int ns, cudaStream_t st) {
  StructureState &S = s->st;
  // species are fixed once the structure exists (the pair path resets
  // layout_species when it replaces them), so the check below runs once
  if (s->layout_species == ns && s->row_of_atom.ptr) return FPP_OK;
  for (int i = 0; i < S.noa; i++)
    if (S.species_host[i] >= ns)
      return fail(FPP_ERR_INVALID, "structure species exceeds the descriptor's n_species");
  s->n_rows.assign(ns, 0);
  s->row_off.assign(ns, 0);
  for (int i = 0; i < S.noa; i++) s->n_rows[S.species_host[i]]++;
  int r = 0;
  for (int k = 0; k < ns; k++) {
    s->row_off[k] = r;
    r += round_up(std::max(s->n_rows[k], 1), 128);
  }
  s->total_rows = r;
  std::vector<int> roa(std::max(S.noa, 1), 0), cnt(ns, 0);
  for (int i = 0; i < S.noa; i++) {
    int sp = S.species_host[i];
    roa[i] = s->row_off[sp] + cnt[sp]++;
  }
  FPP_TRY(s->row_of_atom.reserve(sizeof(int) * roa.size()));
  FPP_CUDA(cudaMemcpyAsync(s->row_of_atom.ptr, roa.data(), sizeof(int) * roa.size(),
                           cudaMemcpyHostToDevice, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  s->layout_species = ns;
  return FPP_OK;
}

// Reserve a buffer and zero it when it had to grow.
static int reserve_zero(DevBuf &b, size_t bytes, cudaStream_t st) {
  bool grow = bytes > b.bytes || !b.ptr;
  FPP_TRY(b.reserve(bytes));
  if (grow) FPP_CUDA(cudaMemsetAsync(b.ptr, 0, b.bytes, st));
  return FPP_OK;
}

static Neigh neigh_of(StructureState &S) {
  Neigh nb;
  nb.offset = S.nbr_offset.as<int>();
  nb.rel = S.nbr_rel.as<dvec4>();
  nb.rel32 = S.nbr_rel32.as<float4>();
  nb.nbr_s = S.nbr_s.as<int>();
  nb.rev = S.nbr_rev.as<int>();
  // without the FP64 table, exact distances near a cutoff are recomputed
  // from the positions (the FP32 kernels need them for a few pairs only)
  nb.geom = (S.rel64_valid || !S.rb_dev) ? nullptr : &S.rb_dev->geom;
  return nb;
}

// FP64 forward: c64, norm64 (atom order), phat64 rows, optional p64 atom order.
int forward64(fpp_structure *s, const B2Args &a0, const int *pair_tab, bool want_p,
              cudaStream_t st) {
  StructureState &S = s->st;
  B2Args a = a0;
  a.noa = S.noa;
  const int ldp = round_up(a.n_d, 64);
  const int sb = a.n_species * a.N * a.H;
  FPP_TRY(ensure_layout(s, a.n_species, st));
  FPP_TRY(ensure_rel64(S, st));
  FPP_TRY(S.c64.reserve(sizeof(double) * std::max(1, S.noa) * sb));
  FPP_TRY(S.norm64.reserve(sizeof(double) * std::max(1, S.noa)));
  FPP_TRY(reserve_zero(S.p64, want_p ? sizeof(double) * std::max(1, S.noa) * a.n_d : 8, st));
  FPP_TRY(reserve_zero(S.V64, sizeof(double) * (size_t)s->total_rows * ldp, st));
  FPP_TRY(reserve_zero(S.w64, sizeof(double) * (size_t)s->total_rows * ldp, st));
  FPP_TRY(reserve_zero(S.phat64, sizeof(double) * (size_t)s->total_rows * ldp, st));
  if (launch_b2_forward<double>(a, neigh_of(S), S.species.as<int>(),
                                s->row_of_atom.as<int>(), pair_tab, S.c64.as<double>(),
                                want_p ? S.p64.as<double>() : nullptr,
                                S.norm64.as<double>(), S.phat64.as<double>(),
                                nullptr, nullptr, ldp, nullptr, st) != 0)
    return fail(FPP_ERR_CUDA, "B2 forward (FP64) launch failed");
  return FPP_OK;
}

// Tile shape of the adjoint Kuf kernel (sparse environments per pass,
// threads per block), chosen by timing the candidates that fit in shared
// memory on a prefix of the work list (CUDA events on the stream) and cached
// per device and descriptor shape: in this process, and in a text file
// ($FPP_TUNE_CACHE, else $HOME/.cache/flare_pp_gb300/tiles.txt; one line
// "key ks threads" per shape) so that later processes skip the timing.
static std::string kuf_tune_path() {
  if (const char *p = std::getenv("FPP_TUNE_CACHE")) return p;
  if (const char *h = std::getenv("HOME")) return std::string(h) + "/.cache/flare_pp_gb300/tiles.txt";
  return std::string();
}

static std::string kuf_tune_key(const B2Args &a) {
  int dev = 0;
  cudaDeviceProp prop;
  std::string name = "gpu";
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess)
    name = prop.name;
  for (char &ch : name)
    if (ch == ' ') ch = '_';
  return "kuf_adjoint:" + name + ":ns" + std::to_string(a.n_species) + ":N" +
         std::to_string(a.N) + ":l" + std::to_string(a.lmax);
}

int kuf_tiles(fpp_model *m, const KufArgs &ka, int n_items, cudaStream_t st, int *ks,
              int *threads) {
  (void)m;
  static std::mutex mu;
  static std::map<std::string, std::pair<int, int>> memo;
  const std::string key = kuf_tune_key(ka.a);
  std::lock_guard<std::mutex> lock(mu);
  auto hit = memo.find(key);
  if (hit == memo.end()) {
    const std::string path = kuf_tune_path();
    if (!path.empty()) {
      std::ifstream in(path);
      std::string k2;
      int a2, b2;
      while (in >> k2 >> a2 >> b2)
        if (k2 == key && kuf_adjoint_smem(ka.a, a2, b2) > 0) memo[key] = {a2, b2};
    }
    hit = memo.find(key);
  }
  if (hit != memo.end()) {
    *ks = hit->second.first;
    *threads = hit->second.second;
    return FPP_OK;
  }
  const int sample = std::min(n_items, 2048);
  cudaEvent_t e0, e1;
  FPP_CUDA(cudaEventCreate(&e0));
  FPP_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bks = 0, bth = 0;
  for (int t : {128, 256})
    for (int c : {2, 4, 8, 16}) {
      if (kuf_adjoint_smem(ka.a, c, t) == 0) continue;
      // once to warm, once timed
      if (launch_kuf_adjoint(ka, c, t, sample, 0, st) != 0) continue;
      FPP_CUDA(cudaEventRecord(e0, st));
      if (launch_kuf_adjoint(ka, c, t, sample, 0, st) != 0) continue;
      FPP_CUDA(cudaEventRecord(e1, st));
      FPP_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      FPP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        bks = c;
        bth = t;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (bks == 0) return fail(FPP_ERR_UNSUPPORTED, "no Kuf tile shape fits in shared memory");
  memo[key] = {bks, bth};
  const std::string path = kuf_tune_path();
  if (!path.empty()) {
    const size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) {
      // best effort: create the directory chain
      std::string dir = path.substr(0, slash), cur;
      size_t pos = 0;
      while ((pos = dir.find('/', pos + 1)) != std::string::npos) {
        cur = dir.substr(0, pos);
        mkdir(cur.c_str(), 0755);
      }
      mkdir(dir.c_str(), 0755);
    }
    std::ofstream out(path, std::ios::app);
    if (out) out << key << " " << bks << " " << bth << "\n";
  }
  *ks = bks;
  *threads = bth;
  return FPP_OK;
}

// Mixed forward: c32, norms (atom order; FP32 hi/lo pairs in pn64's 8-byte
// slots), split fp16 phat rows.
static int forward32(fpp_structure *s, const B2Args &a0, const int *pair_tab,
                     const float *pbar, cudaStream_t st) {
  StructureState &S = s->st;
  B2Args a = a0;
  a.noa = S.noa;
  const int ldp = round_up(a.n_d, 64);
  const int sb = a.n_species * a.N * a.H;
  FPP_TRY(ensure_layout(s, a.n_species, st));
  FPP_TRY(S.c32.reserve(sizeof(float) * std::max(1, S.noa) * sb));
  FPP_TRY(S.pn64.reserve(sizeof(double) * std::max(1, S.noa)));
  FPP_TRY(reserve_zero(S.phat_hi, sizeof(__half) * (size_t)s->total_rows * ldp, st));
  FPP_TRY(reserve_zero(S.phat_lo, sizeof(__half) * (size_t)s->total_rows * ldp, st));
  if (launch_b2_forward<float>(a, neigh_of(S), S.species.as<int>(),
                               s->row_of_atom.as<int>(), pair_tab, S.c32.as<float>(),
                               nullptr, S.pn64.as<double>(), nullptr,
                               S.phat_hi.as<__half>(), S.phat_lo.as<__half>(), ldp,
                               pbar, st) != 0)
    return fail(FPP_ERR_CUDA, "B2 forward (FP32) launch failed");
  return FPP_OK;
}

// energy and the flare-order stress -(1/V) sum f_a r_b from the reduced row
__global__ void k_finish(const double *__restrict__ red, double vi, double *energy,
                         double *stress) {
  if (threadIdx.x != 0) return;
  if (energy) energy[0] = red[0];
  if (stress) {
    stress[0] = -red[1] * vi;
    stress[1] = -red[2] * vi;
    stress[2] = -red[3] * vi;
    stress[3] = -red[5] * vi;
    stress[4] = -red[6] * vi;
    stress[5] = -red[9] * vi;
  }
}

static int finish_outputs(fpp_structure *s, cudaStream_t st, double *energy,
                          double *forces, double *stress, double *atom_energies,
                          int on_device) {
  StructureState &S = s->st;
  if (on_device) {
    // stays asynchronous: the outputs are written in stream order, and a
    // device-side error of this call is reported by the next synchronizing
    // call on the structure (the status word is only cleared once read)
    if (energy || stress) {
      k_finish<<<1, 32, 0, st>>>(S.reduce_out.as<double>(), 1.0 / S.ci.volume, energy, stress);
      FPP_CUDA(cudaGetLastError());
    }
    if (forces && S.noa)
      FPP_CUDA(cudaMemcpyAsync(forces, S.forces.ptr, sizeof(double) * 3 * S.noa,
                               cudaMemcpyDeviceToDevice, st));
    if (atom_energies && S.noa)
      FPP_CUDA(cudaMemcpyAsync(atom_energies, S.atom_e.ptr, sizeof(double) * S.noa,
                               cudaMemcpyDeviceToDevice, st));
    return FPP_OK;
  }
  // every device-to-host copy of the call, then one synchronization
  FPP_TRY(ensure_readback(S));
  FPP_CUDA(cudaMemcpyAsync(S.rb->red, S.reduce_out.ptr, sizeof(double) * 10,
                           cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaMemcpyAsync(S.rb->status, S.status.ptr, sizeof(DeviceStatus),
                           cudaMemcpyDeviceToHost, st));
  if (forces && S.noa)
    FPP_CUDA(cudaMemcpyAsync(forces, S.forces.ptr, sizeof(double) * 3 * S.noa,
                             cudaMemcpyDeviceToHost, st));
  if (atom_energies && S.noa)
    FPP_CUDA(cudaMemcpyAsync(atom_energies, S.atom_e.ptr, sizeof(double) * S.noa,
                             cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  FPP_TRY(status_from_readback(S, st, "prediction"));
  const double *red = S.rb->red;
  const double vi = 1.0 / S.ci.volume;
  // -(1/V) sum f_a r_b, order xx xy xz yy yz zz
  double sv[6] = {-red[1] * vi, -red[2] * vi, -red[3] * vi,
                  -red[5] * vi, -red[6] * vi, -red[9] * vi};
  if (energy) energy[0] = red[0];
  if (stress)
    for (int k = 0; k < 6; k++) stress[k] = sv[k];
  return FPP_OK;
}

static int adjoint_buffers(StructureState &S, size_t elem, int sb) {
  const size_t np = std::max<int64_t>(S.n_pairs, 1);
  FPP_TRY(S.u.reserve(elem * (size_t)std::max(1, S.noa) * sb));
  FPP_TRY(S.atom_e.reserve(sizeof(double) * std::max(1, S.noa)));
  FPP_TRY(S.pair_f.reserve(elem * 4 * np));
  FPP_TRY(S.forces.reserve(sizeof(double) * 3 * std::max(1, S.noa)));
  FPP_TRY(S.atom_vir.reserve(sizeof(double) * 9 * std::max(1, S.noa)));
  FPP_TRY(S.reduce_out.reserve(sizeof(double) * 16));
  return FPP_OK;
}

static int model_check(fpp_model *m, fpp_structure *s) {
  if (!m || !s) return fail(FPP_ERR_INVALID, "null handle");
  for (int k = 0; k < m->n_species; k++)
    if (m->sp[k].n_sparse < 0) return fail(FPP_ERR_INVALID, "sparse set missing");
  return FPP_OK;
}

}  // namespace fpp

using namespace fpp;

extern "C" {

int fpp_b2_pair_count(const fpp_b2 *b2, fpp_structure *s, int64_t *n_desc_pairs,
                      void *stream) {
  if (!b2 || !s || !n_desc_pairs) return fail(FPP_ERR_INVALID, "null argument");
  StructureState &S = s->st;
  const int ns = b2->args.n_species;
  FPP_TRY(ensure_rel64(S, (cudaStream_t)stream));
  for (int i = 0; i < S.noa; i++)
    if (S.species_host[i] >= ns)
      return fail(FPP_ERR_INVALID, "structure species exceeds the descriptor's n_species");
  std::vector<int> nbr_i(S.n_pairs), nbr_s(S.n_pairs);
  std::vector<dvec4> rel(S.n_pairs);
  FPP_CUDA(cudaDeviceSynchronize());
  if (S.n_pairs) {
    FPP_CUDA(cudaMemcpy(nbr_i.data(), S.nbr_i.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(nbr_s.data(), S.nbr_s.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(rel.data(), S.nbr_rel.ptr, sizeof(dvec4) * S.n_pairs, cudaMemcpyDeviceToHost));
  }
  int64_t c = 0;
  for (int64_t p = 0; p < S.n_pairs; p++)
    if (rel[p].x <= b2->args.cutoffs[S.species_host[nbr_i[p]] * ns + nbr_s[p]]) c++;
  *n_desc_pairs = c;
  return FPP_OK;
}

int fpp_b2_compute(const fpp_b2 *b2c, fpp_structure *s, double *descriptors, double *norms,
                   int32_t *desc_neighbor_count, int32_t *desc_neighbor_indices,
                   double *desc_neighbor_coordinates, double *force_dervs,
                   double *force_dots, void *stream) {
  if (!b2c || !s) return fail(FPP_ERR_INVALID, "null argument");
  fpp_b2 *b2 = const_cast<fpp_b2 *>(b2c);
  cudaStream_t st = (cudaStream_t)stream;
  StructureState &S = s->st;
  const B2Args &a = b2->args;
  FPP_TRY(upload_pair_tab(b2->pair_tab, b2->pair_tab_host, st));
  FPP_TRY(forward64(s, a, b2->pair_tab.as<int>(), true, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  if (descriptors && S.noa)
    FPP_CUDA(cudaMemcpy(descriptors, S.p64.ptr, sizeof(double) * S.noa * a.n_d,
                        cudaMemcpyDeviceToHost));
  if (norms && S.noa)
    FPP_CUDA(cudaMemcpy(norms, S.norm64.ptr, sizeof(double) * S.noa, cudaMemcpyDeviceToHost));
  const bool want_pairs = desc_neighbor_count || desc_neighbor_indices ||
                          desc_neighbor_coordinates || force_dervs || force_dots;
  if (!want_pairs) return FPP_OK;
  const int ns = a.n_species;
  std::vector<int> off(S.noa + 1, 0), nbr_i(S.n_pairs), nbr_j(S.n_pairs), nbr_s(S.n_pairs);
  std::vector<dvec4> rel(S.n_pairs);
  if (S.noa)
    FPP_CUDA(cudaMemcpy(off.data(), S.nbr_offset.ptr, sizeof(int) * (S.noa + 1),
                        cudaMemcpyDeviceToHost));
  if (S.n_pairs) {
    FPP_CUDA(cudaMemcpy(nbr_i.data(), S.nbr_i.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(nbr_j.data(), S.nbr_j.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(nbr_s.data(), S.nbr_s.ptr, sizeof(int) * S.n_pairs, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(rel.data(), S.nbr_rel.ptr, sizeof(dvec4) * S.n_pairs, cudaMemcpyDeviceToHost));
  }
  std::vector<int> plist;
  for (int i = 0; i < S.noa; i++) {
    int c = 0;
    for (int p = off[i]; p < off[i + 1]; p++) {
      if (rel[p].x <= a.cutoffs[S.species_host[i] * ns + nbr_s[p]]) {
        if (desc_neighbor_indices) desc_neighbor_indices[plist.size()] = nbr_j[p];
        if (desc_neighbor_coordinates) {
          desc_neighbor_coordinates[3 * plist.size() + 0] = rel[p].y;
          desc_neighbor_coordinates[3 * plist.size() + 1] = rel[p].z;
          desc_neighbor_coordinates[3 * plist.size() + 2] = rel[p].w;
        }
        plist.push_back(p);
        c++;
      }
    }
    if (desc_neighbor_count) desc_neighbor_count[i] = c;
  }
  if ((force_dervs || force_dots) && !plist.empty()) {
    const int npl = (int)plist.size();
    DevBuf d_plist, d_dp, d_fd;
    FPP_TRY(d_plist.reserve(sizeof(int) * npl));
    FPP_TRY(d_dp.reserve(sizeof(double) * 3 * (size_t)npl * a.n_d));
    FPP_TRY(d_fd.reserve(sizeof(double) * 3 * npl));
    FPP_CUDA(cudaMemcpy(d_plist.ptr, plist.data(), sizeof(int) * npl, cudaMemcpyHostToDevice));
    B2Args aa = a;
    aa.noa = S.noa;
    if (launch_b2_dp(aa, npl, d_plist.as<int>(), S.nbr_i.as<int>(), S.nbr_s.as<int>(),
                     S.nbr_rel.as<dvec4>(), S.species.as<int>(), b2->pair_tab.as<int>(),
                     S.c64.as<double>(), S.p64.as<double>(), d_dp.as<double>(), a.n_d,
                     d_fd.as<double>(), st) != 0)
      return fail(FPP_ERR_CUDA, "stored-derivative kernel launch failed");
    FPP_CUDA(cudaStreamSynchronize(st));
    if (force_dervs)
      FPP_CUDA(cudaMemcpy(force_dervs, d_dp.ptr, sizeof(double) * 3 * (size_t)npl * a.n_d,
                          cudaMemcpyDeviceToHost));
    if (force_dots)
      FPP_CUDA(cudaMemcpy(force_dots, d_fd.ptr, sizeof(double) * 3 * npl,
                          cudaMemcpyDeviceToHost));
  }
  return FPP_OK;
}

int fpp_model_create(const fpp_b2 *b2, double sigma, double power, fpp_model **out) {
  if (!b2 || !out) return fail(FPP_ERR_INVALID, "null argument");
  *out = nullptr;
  if (!std::isfinite(sigma) || !std::isfinite(power))
    return fail(FPP_ERR_NUMERIC, "sigma and power must be finite");
  auto *m = new fpp_model();
  m->args = b2->args;
  m->pair_tab_host = b2->pair_tab_host;
  m->sigma = sigma;
  m->power = power;
  m->n_species = b2->args.n_species;
  m->n_d = b2->args.n_d;
  m->ldb = round_up(m->n_d, 64);
  m->sp.resize(m->n_species);
  *out = m;
  return FPP_OK;
}

int fpp_model_destroy(fpp_model *m) {
  if (m && m->cublas) cublasDestroy((cublasHandle_t)m->cublas);
  if (m) {
    delete m->lammps;
    delete m->batch;
  }
  delete m;
  return FPP_OK;
}

int fpp_model_set_sparse(fpp_model *m, int32_t species, int32_t n_sparse,
                         const double *descriptors, const double *norms,
                         const double *alpha) {
  if (!m) return fail(FPP_ERR_INVALID, "null model");
  if (species < 0 || species >= m->n_species) return fail(FPP_ERR_INVALID, "bad species");
  if (n_sparse < 0 || (n_sparse > 0 && (!descriptors || !norms || !alpha)))
    return fail(FPP_ERR_INVALID, "bad sparse arrays");
  auto &sp = m->sp[species];
  const int nd = m->n_d;
  sp.n_sparse = n_sparse;
  sp.desc.assign(descriptors, descriptors + (size_t)n_sparse * nd);
  sp.norms.assign(norms, norms + n_sparse);
  sp.alpha.assign(alpha, alpha + n_sparse);
  std::vector<double> dhat((size_t)std::max(n_sparse, 1) * nd, 0.0);
  for (int k = 0; k < n_sparse; k++)
    if (norms[k] >= 1e-8)
      for (int d = 0; d < nd; d++) dhat[(size_t)k * nd + d] = descriptors[(size_t)k * nd + d] / norms[k];
  const size_t n1 = std::max(n_sparse, 1);
  FPP_TRY(sp.d_desc.reserve(sizeof(double) * n1 * nd));
  FPP_TRY(sp.d_dhat.reserve(sizeof(double) * n1 * nd));
  FPP_TRY(sp.d_norms.reserve(sizeof(double) * n1));
  FPP_TRY(sp.d_alpha.reserve(sizeof(double) * n1));
  if (n_sparse) {
    FPP_CUDA(cudaMemcpy(sp.d_desc.ptr, descriptors, sizeof(double) * n_sparse * nd, cudaMemcpyHostToDevice));
    FPP_CUDA(cudaMemcpy(sp.d_dhat.ptr, dhat.data(), sizeof(double) * n_sparse * nd, cudaMemcpyHostToDevice));
    FPP_CUDA(cudaMemcpy(sp.d_norms.ptr, norms, sizeof(double) * n_sparse, cudaMemcpyHostToDevice));
    // empty sparse environments carry no weight (normalized_dot_product.cpp:157)
    std::vector<double> aeff(n_sparse);
    for (int k = 0; k < n_sparse; k++) aeff[k] = norms[k] >= 1e-8 ? alpha[k] : 0.0;
    FPP_CUDA(cudaMemcpy(sp.d_alpha.ptr, aeff.data(), sizeof(double) * n_sparse, cudaMemcpyHostToDevice));
  }
  int off = 0;
  for (auto &x : m->sp) {
    x.sparse_offset = off;
    off += x.n_sparse;
  }
  m->n_sparse_total = off;
  m->beta_power = 0;
  return FPP_OK;
}

int fpp_model_set_R_inv(fpp_model *m, int32_t n, const double *R_inv) {
  if (!m || !R_inv) return fail(FPP_ERR_INVALID, "null argument");
  if (n != m->n_sparse_total)
    return fail(FPP_ERR_INVALID, "R_inv size does not match the sparse set");
  FPP_TRY(m->R_inv.reserve(sizeof(double) * std::max(1, n) * std::max(1, n)));
  if (n) FPP_CUDA(cudaMemcpy(m->R_inv.ptr, R_inv, sizeof(double) * n * n, cudaMemcpyHostToDevice));
  m->has_R_inv = true;
  // upper triangular (the QR solve's): the variance products skip its zeros
  bool upper = true;
  for (int i = 1; i < n && upper; i++)
    for (int j = 0; j < i; j++)
      if (R_inv[(size_t)i * n + j] != 0.0) {
        upper = false;
        break;
      }
  m->R_inv_upper = upper;
  return FPP_OK;
}

// dense symmetric beta (host, n_d x n_d) -> device FP64 and split fp16 operands
static int upload_beta(fpp_model *m, int s, const std::vector<double> &B) {
  const int nd = m->n_d, ldb = m->ldb;
  auto &sp = m->sp[s];
  std::vector<double> pad((size_t)nd * ldb, 0.0);
  double amax = 0;
  for (int i = 0; i < nd; i++)
    for (int j = 0; j < nd; j++) {
      pad[(size_t)i * ldb + j] = B[(size_t)i * nd + j];
      amax = std::max(amax, std::fabs(B[(size_t)i * nd + j]));
    }
  double scale = 1.0;
  if (amax > 0) scale = std::ldexp(1.0, (int)std::floor(std::log2(16384.0 / amax)));
  std::vector<__half> hi(pad.size()), lo(pad.size());
  for (size_t k = 0; k < pad.size(); k++) {
    const float x = (float)(pad[k] * scale);
    const __half h = __float2half_rn(x);
    const float rem = (float)((pad[k] * scale - (double)__half2float(h)) * 2048.0);
    hi[k] = h;
    lo[k] = __float2half_rn(rem);
  }
  sp.beta_scale = scale;
  sp.B_host = B;
  FPP_TRY(sp.beta64.reserve(sizeof(double) * pad.size()));
  FPP_TRY(sp.beta_hi.reserve(sizeof(__half) * pad.size()));
  FPP_TRY(sp.beta_lo.reserve(sizeof(__half) * pad.size()));
  FPP_CUDA(cudaMemcpy(sp.beta64.ptr, pad.data(), sizeof(double) * pad.size(), cudaMemcpyHostToDevice));
  FPP_CUDA(cudaMemcpy(sp.beta_hi.ptr, hi.data(), sizeof(__half) * hi.size(), cudaMemcpyHostToDevice));
  FPP_CUDA(cudaMemcpy(sp.beta_lo.ptr, lo.data(), sizeof(__half) * lo.size(), cudaMemcpyHostToDevice));
  return FPP_OK;
}

int fpp_model_compute_beta(fpp_model *m, double *beta_packed, void *stream) {
  if (!m) return fail(FPP_ERR_INVALID, "null model");
  cudaStream_t st = (cudaStream_t)stream;
  const int nd = m->n_d, ns = m->n_species;
  const double sig2 = m->sigma * m->sigma;
  if (m->power == 1.0) {
    std::vector<double> b1((size_t)ns * nd, 0.0);
    for (int s = 0; s < ns; s++) {
      auto &sp = m->sp[s];
      for (int k = 0; k < sp.n_sparse; k++) {
        if (sp.norms[k] < 1e-8) continue;
        for (int d = 0; d < nd; d++)
          b1[(size_t)s * nd + d] += sig2 * sp.desc[(size_t)k * nd + d] / sp.norms[k] * sp.alpha[k];
      }
    }
    FPP_TRY(m->beta1.reserve(sizeof(double) * b1.size()));
    FPP_CUDA(cudaMemcpy(m->beta1.ptr, b1.data(), sizeof(double) * b1.size(), cudaMemcpyHostToDevice));
    if (beta_packed) std::memcpy(beta_packed, b1.data(), sizeof(double) * b1.size());
    m->beta_power = 1;
    return center_from_sparse(m);
  }
  if (m->power != 2.0)
    return fail(FPP_ERR_UNSUPPORTED, "mapped coefficients exist for power 1 and 2 only");
  cublasHandle_t h;
  FPP_TRY(get_cublas(m, st, &h));
  const size_t np = (size_t)nd * (nd + 1) / 2;
  for (int s = 0; s < ns; s++) {
    auto &sp = m->sp[s];
    std::vector<double> B((size_t)nd * nd, 0.0);
    if (sp.n_sparse > 0) {
      // B = sig2 * Dhat^T diag(alpha) Dhat  (cuBLAS, FP64)
      DevBuf da, dB;
      FPP_TRY(da.reserve(sizeof(double) * (size_t)sp.n_sparse * nd));
      FPP_TRY(dB.reserve(sizeof(double) * (size_t)nd * nd));
      std::vector<double> dh((size_t)sp.n_sparse * nd, 0.0), ds((size_t)sp.n_sparse * nd, 0.0);
      for (int k = 0; k < sp.n_sparse; k++) {
        if (sp.norms[k] < 1e-8) continue;
        for (int d = 0; d < nd; d++) {
          const double v = sp.desc[(size_t)k * nd + d] / sp.norms[k];
          ds[(size_t)k * nd + d] = v * sp.alpha[k] * sig2;
        }
      }
      FPP_CUDA(cudaMemcpy(da.ptr, ds.data(), sizeof(double) * ds.size(), cudaMemcpyHostToDevice));
      const double one = 1.0, zero = 0.0;
      FPP_CUBLAS(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, nd, nd, sp.n_sparse, &one,
                             da.as<double>(), nd, sp.d_dhat.as<double>(), nd, &zero,
                             dB.as<double>(), nd));
      FPP_CUDA(cudaStreamSynchronize(st));
      FPP_CUDA(cudaMemcpy(B.data(), dB.ptr, sizeof(double) * B.size(), cudaMemcpyDeviceToHost));
      // symmetrise the rounding of the two triangles
      for (int i = 0; i < nd; i++)
        for (int j = i + 1; j < nd; j++) {
          const double v = 0.5 * (B[(size_t)i * nd + j] + B[(size_t)j * nd + i]);
          B[(size_t)i * nd + j] = B[(size_t)j * nd + i] = v;
        }
    }
    FPP_TRY(upload_beta(m, s, B));
    if (beta_packed) {
      size_t c = 0;
      for (int i = 0; i < nd; i++)
        for (int j = i; j < nd; j++, c++)
          beta_packed[(size_t)s * np + c] = (i == j ? 1.0 : 2.0) * B[(size_t)i * nd + j];
    }
  }
  m->beta_power = 2;
  return center_from_sparse(m);
}

int fpp_model_set_beta(fpp_model *m, int32_t power, const double *beta_packed) {
  if (!m || !beta_packed) return fail(FPP_ERR_INVALID, "null argument");
  const int nd = m->n_d, ns = m->n_species;
  if (power == 1) {
    FPP_TRY(m->beta1.reserve(sizeof(double) * (size_t)ns * nd));
    FPP_CUDA(cudaMemcpy(m->beta1.ptr, beta_packed, sizeof(double) * (size_t)ns * nd,
                        cudaMemcpyHostToDevice));
    m->beta_power = 1;
    return center_from_sparse(m);
  }
  if (power != 2) return fail(FPP_ERR_INVALID, "power must be 1 or 2");
  const size_t np = (size_t)nd * (nd + 1) / 2;
  for (int s = 0; s < ns; s++) {
    std::vector<double> B((size_t)nd * nd, 0.0);
    size_t c = 0;
    for (int i = 0; i < nd; i++)
      for (int j = i; j < nd; j++, c++) {
        const double v = beta_packed[(size_t)s * np + c];
        if (i == j)
          B[(size_t)i * nd + j] = v;
        else
          B[(size_t)i * nd + j] = B[(size_t)j * nd + i] = v / 2;
      }
    FPP_TRY(upload_beta(m, s, B));
  }
  m->beta_power = 2;
  return center_from_sparse(m);
}

}  // extern "C"

namespace fpp {

// Centre of the mixed operand for every species: pbar (rounded to FP32, the
// values the kernels use), g = beta pbar and c0 = pbar^T beta pbar in FP64.
static int set_center(fpp_model *m, const std::vector<std::vector<double>> &pbar) {
  const int nd = m->n_d, ns = m->n_species;
  std::vector<float> pb((size_t)ns * nd, 0.f), gv((size_t)ns * nd, 0.f);
  m->c0.assign(ns, 0.0);
  for (int s = 0; s < ns; s++) {
    std::vector<double> p(nd, 0.0);
    for (int d = 0; d < nd; d++) {
      pb[(size_t)s * nd + d] = (float)pbar[s][d];
      p[d] = (double)pb[(size_t)s * nd + d];
    }
    if (m->beta_power == 2 && !m->sp[s].B_host.empty()) {
      const double *B = m->sp[s].B_host.data();
      double c0 = 0;
      for (int a = 0; a < nd; a++) {
        double acc = 0;
        for (int b = 0; b < nd; b++) acc += B[(size_t)a * nd + b] * p[b];
        gv[(size_t)s * nd + a] = (float)acc;
        c0 += p[a] * acc;
      }
      m->c0[s] = c0;
    }
  }
  // g is used in FP32; c0 must then be consistent with the same pbar: the
  // energy splits as c0 + 2 g.delta + delta.V exactly for any pbar, and the
  // FP32 rounding of g only enters through delta (small).
  FPP_TRY(m->pbar32.reserve(sizeof(float) * pb.size()));
  FPP_TRY(m->g32.reserve(sizeof(float) * gv.size()));
  FPP_CUDA(cudaMemcpy(m->pbar32.ptr, pb.data(), sizeof(float) * pb.size(), cudaMemcpyHostToDevice));
  FPP_CUDA(cudaMemcpy(m->g32.ptr, gv.data(), sizeof(float) * gv.size(), cudaMemcpyHostToDevice));
  return FPP_OK;
}

// pbar from the sparse set: the normalised mean of its unit descriptors (a
// species without sparse environments keeps a zero centre).  The mixed form
// replaces it, species by species, with the mean of the first structure it
// evaluates that contains the species.
static int center_from_sparse(fpp_model *m) {
  const int nd = m->n_d;
  std::vector<std::vector<double>> pbar(m->n_species, std::vector<double>(nd, 0.0));
  for (int s = 0; s < m->n_species; s++) {
    auto &sp = m->sp[s];
    for (int k = 0; k < sp.n_sparse; k++) {
      if (sp.norms[k] < 1e-8) continue;
      for (int d = 0; d < nd; d++) pbar[s][d] += sp.desc[(size_t)k * nd + d] / sp.norms[k];
    }
    double n = 0;
    for (double v : pbar[s]) n += v * v;
    n = std::sqrt(n);
    if (n > 0)
      for (double &v : pbar[s]) v /= n;
  }
  FPP_TRY(set_center(m, pbar));
  m->centred.assign(m->n_species, 0);
  return FPP_OK;
}

// Column sums of the FP64 normalised descriptor rows of one species block:
// thread per column, rows split over blockIdx.y, fixed-order partial sums
// per (column, row chunk) combined on the host in chunk order.
__global__ void k_column_sums(const double *__restrict__ rows, int n_rows, int ldp, int nd,
                              int chunk, double *__restrict__ partial) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nd) return;
  const int r0 = blockIdx.y * chunk;
  const int r1 = min(n_rows, r0 + chunk);
  double acc = 0;
  for (int r = r0; r < r1; r++) acc += rows[(size_t)r * ldp + d];
  partial[(size_t)blockIdx.y * nd + d] = acc;
}

// pbar from a structure: the normalised mean of its atoms' unit descriptors
// (FP64 forward pass, column sums on the device), for the species with atoms
// in s that are not yet centred on a structure, or (with every_species) for
// every species with atoms in s.
static int center_from_structure(fpp_model *m, fpp_structure *s, cudaStream_t st,
                                 bool every_species = false) {
  StructureState &S = s->st;
  const int nd = m->n_d, ldp = round_up(nd, 64);
  B2Args a = m->args;
  a.noa = S.noa;
  a.strict = 0;
  FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), false, st));
  if ((int)m->centred.size() != m->n_species) m->centred.assign(m->n_species, 0);
  std::vector<std::vector<double>> pbar(m->n_species, std::vector<double>(nd, 0.0));
  std::vector<float> old((size_t)m->n_species * nd, 0.f);
  if (m->pbar32.ptr)
    FPP_CUDA(cudaMemcpy(old.data(), m->pbar32.ptr, sizeof(float) * old.size(),
                        cudaMemcpyDeviceToHost));
  constexpr int kChunks = 64;
  DevBuf partial;
  FPP_TRY(partial.reserve(sizeof(double) * (size_t)kChunks * nd));
  std::vector<double> host((size_t)kChunks * nd);
  for (int sp = 0; sp < m->n_species; sp++) {
    for (int d = 0; d < nd; d++) pbar[sp][d] = old[(size_t)sp * nd + d];
    if (s->n_rows[sp] == 0 || (m->centred[sp] && !every_species)) continue;
    const int chunk = ceil_div(s->n_rows[sp], kChunks);
    const int nchunks = ceil_div(s->n_rows[sp], chunk);
    k_column_sums<<<dim3(ceil_div(nd, 128), nchunks), 128, 0, st>>>(
        S.phat64.as<double>() + (size_t)s->row_off[sp] * ldp, s->n_rows[sp], ldp, nd, chunk,
        partial.as<double>());
    FPP_CUDA(cudaGetLastError());
    FPP_CUDA(cudaMemcpyAsync(host.data(), partial.ptr, sizeof(double) * (size_t)nchunks * nd,
                             cudaMemcpyDeviceToHost, st));
    FPP_CUDA(cudaStreamSynchronize(st));
    for (int d = 0; d < nd; d++) {
      double v = 0;
      for (int c = 0; c < nchunks; c++) v += host[(size_t)c * nd + d];
      pbar[sp][d] = v;
    }
    double n = 0;
    for (double v : pbar[sp]) n += v * v;
    n = std::sqrt(n);
    if (n > 0)
      for (double &v : pbar[sp]) v /= n;
    m->centred[sp] = 1;
  }
  return set_center(m, pbar);
}

// Forward, contraction and adjoint of the mapped form; leaves atom_e, pair_f
// and (with gather) forces / reduce_out in the structure workspace.
int mapped_core(fpp_model *m, fpp_structure *s, int precision, cudaStream_t st,
                int strict) {
  FPP_TRY(model_check(m, s));
  if (m->beta_power == 0)
    return fail(FPP_ERR_INVALID, "mapped coefficients not set (fpp_model_compute_beta)");
  if (precision != FPP_PREC_FP64 && precision != FPP_PREC_MIXED)
    return fail(FPP_ERR_INVALID, "bad precision");
  StructureState &S = s->st;
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  const int nd = m->n_d, ldp = round_up(nd, 64);
  B2Args a = m->args;
  a.noa = S.noa;
  a.strict = strict;
  const bool gather = !strict;
  AdjArgs g;
  std::memset(&g, 0, sizeof(g));
  g.mode = m->beta_power == 2 ? kWFromV2 : kWFromV1;
  g.strict = strict;
  g.empty_thresh = 1e-8;
  g.empty_thresh_f = 1e-8f;
  g.ldp = ldp;
  g.ldv = ldp;
  g.beta1 = m->beta1.as<double>();
  g.status = S.status.as<DeviceStatus>();
  S.mark(2, st);
  if (precision == FPP_PREC_FP64) {
    FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), false, st));
    S.mark(3, st);
    double *phat = S.phat64.as<double>();
    if (m->beta_power == 2) {
      cublasHandle_t h;
      FPP_TRY(get_cublas(m, st, &h));
      const double one = 1.0, zero = 0.0;
      for (int sp = 0; sp < m->n_species; sp++) {
        if (s->n_rows[sp] == 0) continue;
        FPP_CUBLAS(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, nd, s->n_rows[sp], nd, &one,
                               m->sp[sp].beta64.as<double>(), m->ldb,
                               phat + (size_t)s->row_off[sp] * ldp, ldp, &zero,
                               S.V64.as<double>() + (size_t)s->row_off[sp] * ldp, ldp));
      }
      g.V64 = S.V64.as<double>();
    }
    S.mark(4, st);
    g.phat64 = phat;
    FPP_TRY(adjoint_buffers(S, sizeof(double), u_row_stride(a)));
    if (launch_b2_adjoint<double>(a, g, neigh_of(S), S.species.as<int>(),
                                  s->row_of_atom.as<int>(), m->pair_tab.as<int>(),
                                  S.c64.as<double>(), S.norm64.as<double>(),
                                  S.atom_e.as<double>(), S.pair_f.as<double>(),
                                  S.forces.as<double>(), S.atom_vir.as<double>(),
                                  S.reduce_out.as<double>(), gather,
                                  S.u.as<double>(), S.n_pairs, S.nbr_i.as<int>(), st) != 0)
      return fail(FPP_ERR_CUDA, "adjoint (FP64) launch failed");
  } else {
    // centre every species of s that is not yet centred on a structure
    FPP_TRY(ensure_layout(s, a.n_species, st));
    if ((int)m->centred.size() != m->n_species) m->centred.assign(m->n_species, 0);
    bool recentre = false;
    for (int sp = 0; sp < m->n_species; sp++)
      if (s->n_rows[sp] > 0 && !m->centred[sp]) recentre = true;
    if (recentre) FPP_TRY(center_from_structure(m, s, st));
    FPP_TRY(forward32(s, a, m->pair_tab.as<int>(), m->pbar32.as<float>(), st));
    S.mark(3, st);
    if (m->beta_power == 2) {
      FPP_TRY(reserve_zero(S.V, sizeof(float) * (size_t)s->total_rows * ldp, st));
      GroupedGemmArgs ga;
      std::memset(&ga, 0, sizeof(ga));
      ga.a_hi = S.phat_hi.as<__half>();
      ga.a_lo = S.phat_lo.as<__half>();
      ga.a_rows = s->total_rows;
      ga.lda = ldp;
      for (int sp = 0; sp < m->n_species; sp++) {
        if (s->n_rows[sp] == 0) continue;
        GemmGroup &q = ga.group[ga.n_groups++];
        q.b_hi = m->sp[sp].beta_hi.as<__half>();
        q.b_lo = m->sp[sp].beta_lo.as<__half>();
        q.b_rows = nd;
        q.ldb = m->ldb;
        q.row0 = s->row_off[sp];
        q.M = s->n_rows[sp];
        q.out_scale = (float)(1.0 / (8192.0 * m->sp[sp].beta_scale));
      }
      ga.N = nd;
      ga.K = nd;
      ga.V = S.V.as<float>();
      ga.ldv = ldp;
      ga.status = S.status.as<DeviceStatus>();
      const int rc = launch_split_gemm_grouped(ga, st);
      if (rc != 0)
        return fail(FPP_ERR_CUDA,
                    "split-fp16 contraction launch failed (" + std::to_string(rc) + ")");
      g.V32 = S.V.as<float>();
    }
    S.mark(4, st);
    g.phat_hi = S.phat_hi.as<__half>();
    g.phat_lo = S.phat_lo.as<__half>();
    g.pbar = m->pbar32.as<float>();
    g.gvec = m->g32.as<float>();
    for (int k = 0; k < m->n_species; k++) {
      g.c0[k] = m->c0[k];
      g.c0_hi[k] = (float)m->c0[k];
      g.c0_lo[k] = (float)(m->c0[k] - (double)g.c0_hi[k]);
    }
    FPP_TRY(adjoint_buffers(S, sizeof(float), u_row_stride(a)));
    if (launch_b2_adjoint<float>(a, g, neigh_of(S), S.species.as<int>(),
                                 s->row_of_atom.as<int>(), m->pair_tab.as<int>(),
                                 S.c32.as<float>(), S.pn64.as<double>(),
                                 S.atom_e.as<double>(), S.pair_f.as<float>(),
                                 S.forces.as<double>(), S.atom_vir.as<double>(),
                                 S.reduce_out.as<double>(), gather,
                                 S.u.as<float>(), S.n_pairs, S.nbr_i.as<int>(), st) != 0)
      return fail(FPP_ERR_CUDA, "adjoint (mixed) launch failed");
  }
  S.mark(5, st);
  S.ev_pred = S.profile;
  return FPP_OK;
}

}  // namespace fpp

extern "C" {

int fpp_predict_mapped(fpp_model *m, fpp_structure *s, int precision, double *energy,
                       double *forces, double *stress, double *atom_energies,
                       int outputs_on_device, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  FPP_TRY(mapped_core(m, s, precision, st, 0));
  return finish_outputs(s, st, energy, forces, stress, atom_energies, outputs_on_device);
}

int fpp_model_center_on(fpp_model *m, fpp_structure *s, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  FPP_TRY(model_check(m, s));
  if (m->beta_power == 0)
    return fail(FPP_ERR_INVALID, "mapped coefficients not set (fpp_model_compute_beta)");
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  return center_from_structure(m, s, st, true);
}

// Full FP64 kernel matrix on the device: K (n_sparse_total x n_out) row-major.
static int envs_struc_device(fpp_model *m, fpp_structure *s, cudaStream_t st, DevBuf &K) {
  StructureState &S = s->st;
  const int nd = m->n_d, ldp = round_up(nd, 64), noa = S.noa;
  const int n_out = 1 + 3 * noa + 6;
  const double sig2 = m->sigma * m->sigma;
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  B2Args a = m->args;
  a.noa = noa;
  FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), true, st));
  double *phat = S.phat64.as<double>();
  FPP_TRY(K.reserve(sizeof(double) * (size_t)std::max(1, m->n_sparse_total) * n_out));
  FPP_CUDA(cudaMemsetAsync(K.ptr, 0, sizeof(double) * (size_t)m->n_sparse_total * n_out, st));
  // row-ordered atom norms
  DevBuf &rown = m->es_rown;
  FPP_TRY(rown.reserve(sizeof(double) * std::max(1, s->total_rows)));
  FPP_CUDA(cudaMemsetAsync(rown.ptr, 0, sizeof(double) * s->total_rows, st));
  if (launch_gather_rows(noa, s->row_of_atom.as<int>(), S.norm64.as<double>(),
                         rown.as<double>(), st) != 0)
    return fail(FPP_ERR_CUDA, "gather launch failed");
  // per species: the descriptor pairs (central atom of the species, within
  // the pair's cutoff, b2.cpp:277) selected on the device in pair order
  const long long np = S.n_pairs;
  FPP_TRY(m->es_flags.reserve(sizeof(int) * (size_t)(np + 1)));
  FPP_TRY(m->es_pos.reserve(sizeof(int) * (size_t)(np + 1)));
  FPP_TRY(m->es_dmap.reserve(sizeof(int) * (size_t)std::max<long long>(np, 1)));
  size_t scan_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, m->es_flags.as<int>(), m->es_pos.as<int>(),
                                (int)(np + 1), st);
  FPP_TRY(m->es_scan.reserve(std::max<size_t>(scan_bytes, 16)));
  for (int sp = 0; sp < m->n_species; sp++) {
    const int Ss = m->sp[sp].n_sparse, nsa = s->n_rows[sp];
    if (Ss == 0) continue;
    double *Kb = K.as<double>() + (size_t)m->sp[sp].sparse_offset * n_out;
    if (nsa == 0) continue;
    CutRow cut;
    for (int t = 0; t < kSelMaxSpecies; t++)
      cut.c[t] = t < a.n_species ? a.cutoffs[sp * a.n_species + t] : 0.0;
    int nq = 0;
    if (np > 0) {
      if (launch_pair_flags(np, S.nbr_i.as<int>(), S.nbr_s.as<int>(), S.nbr_rel.as<dvec4>(),
                            S.species.as<int>(), sp, cut, m->es_flags.as<int>(), st) != 0)
        return fail(FPP_ERR_CUDA, "pair selection launch failed");
      size_t tb = m->es_scan.bytes;
      FPP_CUDA(cub::DeviceScan::ExclusiveSum(m->es_scan.ptr, tb, m->es_flags.as<int>(),
                                             m->es_pos.as<int>(), (int)(np + 1), st));
      FPP_CUDA(cudaMemcpyAsync(&nq, m->es_pos.as<int>() + np, sizeof(int),
                               cudaMemcpyDeviceToHost, st));
      FPP_CUDA(cudaStreamSynchronize(st));
    }
    DevBuf &d_ndm = m->es_ndm;
    FPP_TRY(d_ndm.reserve(sizeof(double) * (size_t)Ss * nsa));
    const double *Dh = m->sp[sp].d_dhat.as<double>();
    const double *Ph = phat + (size_t)s->row_off[sp] * ldp;
    // ndm[k][i] = dhat_k . phat_i  (row-major S x n_s), tensor cores, FP64-accurate
    FPP_TRY(ozaki_dgemm_nt(Ss, nsa, nd, Dh, nd, Ph, ldp, d_ndm.as<double>(), nsa, m->oz, st));
    const double *anorm = rown.as<double>() + s->row_off[sp];
    if (launch_envs_energy(Ss, nsa, d_ndm.as<double>(), nsa, m->sp[sp].d_norms.as<double>(),
                           anorm, sig2, m->power, Kb, n_out, st) != 0)
      return fail(FPP_ERR_CUDA, "envs energy launch failed");
    if (nq == 0) {
      FPP_CUDA(cudaStreamSynchronize(st));  // ndm is reused by the next species
      continue;
    }
    FPP_TRY(m->es_plist.reserve(sizeof(int) * nq));
    FPP_TRY(m->es_qatom.reserve(sizeof(int) * nq));
    FPP_TRY(m->es_dp.reserve(sizeof(double) * 3 * (size_t)nq * nd));
    FPP_TRY(m->es_sfd.reserve(sizeof(double) * 3 * nq));
    FPP_TRY(m->es_fd.reserve(sizeof(double) * 3 * (size_t)nq * Ss));
    int *d_plist = m->es_plist.as<int>(), *d_qatom = m->es_qatom.as<int>(),
        *d_dmap = m->es_dmap.as<int>();
    double *d_dp = m->es_dp.as<double>(), *d_sfd = m->es_sfd.as<double>(),
           *d_fd = m->es_fd.as<double>();
    if (launch_pair_scatter(np, m->es_flags.as<int>(), m->es_pos.as<int>(), S.nbr_i.as<int>(),
                            s->row_of_atom.as<int>(), s->row_off[sp], d_plist, d_qatom, d_dmap,
                            st) != 0)
      return fail(FPP_ERR_CUDA, "pair selection launch failed");
    if (launch_b2_dp(a, nq, d_plist, S.nbr_i.as<int>(), S.nbr_s.as<int>(),
                     S.nbr_rel.as<dvec4>(), S.species.as<int>(), m->pair_tab.as<int>(),
                     S.c64.as<double>(), S.p64.as<double>(), d_dp, nd, d_sfd, st) != 0)
      return fail(FPP_ERR_CUDA, "stored-derivative kernel launch failed");
    // fd[k][r] = dhat_k . dp_r  (row-major S x 3nq), tensor cores, FP64-accurate
    FPP_TRY(ozaki_dgemm_nt(Ss, 3 * nq, nd, Dh, nd, d_dp, nd, d_fd, 3 * nq, m->oz, st));
    if (launch_envs_fkv(Ss, nq, d_fd, 3 * nq, d_ndm.as<double>(), nsa, d_qatom, d_sfd,
                        m->sp[sp].d_norms.as<double>(), anorm, sig2, m->power, st) != 0 ||
        launch_envs_force(Ss, noa, d_fd, 3 * nq, S.nbr_offset.as<int>(), S.nbr_rev.as<int>(),
                          d_dmap, Kb, n_out, st) != 0 ||
        launch_envs_stress(Ss, nq, d_fd, 3 * nq, d_plist, S.nbr_rel.as<dvec4>(),
                           1.0 / S.ci.volume, noa, Kb, n_out, st) != 0)
      return fail(FPP_ERR_CUDA, "envs assembly launch failed");
    FPP_CUDA(cudaStreamSynchronize(st));  // the workspace is reused by the next species
  }
  return ozaki_check_status(m->oz, st);
}

}  // extern "C"

namespace fpp {
// dst[r][col0 + c] = src[r][cols[c]] for r < rows (row-major, leading dims).
__global__ void k_copy_cols(int rows, int ncols, const double *__restrict__ src, int lds,
                            const int *__restrict__ cols, double *__restrict__ dst,
                            long long ldd) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)rows * ncols) return;
  const int r = (int)(t / ncols), c = (int)(t - (long long)r * ncols);
  dst[(size_t)r * ldd + c] = src[(size_t)r * lds + cols[c]];
}
}  // namespace fpp

// B3 models: envs_struc of each structure through its stored descriptor
// derivatives (the reference's route), copied column by column into Kuf.
static int kuf_stored_derivatives(fpp_model *m, fpp_structure *const *structures,
                                  int32_t n_structures, const int32_t *label_mask,
                                  const int32_t *atom_offsets, const int32_t *atoms,
                                  double *kuf, int64_t n_labels, cudaStream_t st) {
  std::vector<std::vector<int>> cols(n_structures);
  int64_t total = 0;
  for (int k = 0; k < n_structures; k++) {
    fpp_structure *s = structures[k];
    if (!s) return fail(FPP_ERR_INVALID, "null structure");
    const int noa = s->st.noa;
    std::vector<int> &c = cols[k];
    if (label_mask[k] & 1) c.push_back(0);
    if (label_mask[k] & 2) {
      const int b = atom_offsets ? atom_offsets[k] : 0;
      const int e = atom_offsets ? atom_offsets[k + 1] : noa;
      for (int q = b; q < e; q++) {
        const int a = atom_offsets ? atoms[q] : q;
        if (a < 0 || a >= noa) return fail(FPP_ERR_INVALID, "force atom index out of range");
        for (int d = 0; d < 3; d++) c.push_back(1 + 3 * a + d);
      }
    }
    if (label_mask[k] & 4)
      for (int d = 0; d < 6; d++) c.push_back(1 + 3 * noa + d);
    total += (int64_t)c.size();
  }
  if (total != n_labels)
    return fail(FPP_ERR_INVALID, "n_labels (" + std::to_string(n_labels) +
                                     ") differs from the labels of the structures (" +
                                     std::to_string(total) + ")");
  const int nst = m->n_sparse_total;
  DevBuf dK, K, dcols;
  FPP_TRY(dK.reserve(sizeof(double) * std::max<int64_t>(1, (int64_t)nst * n_labels)));
  int64_t col0 = 0;
  for (int k = 0; k < n_structures; k++) {
    fpp_structure *s = structures[k];
    FPP_TRY(model_check(m, s));
    const int n_out = 1 + 3 * s->st.noa + 6;
    const int nc = (int)cols[k].size();
    if (nc == 0 || nst == 0) continue;
    FPP_TRY(envs_struc_device(m, s, st, K));
    FPP_TRY(dcols.reserve(sizeof(int) * nc));
    FPP_CUDA(cudaMemcpyAsync(dcols.ptr, cols[k].data(), sizeof(int) * nc,
                             cudaMemcpyHostToDevice, st));
    const long long t = (long long)nst * nc;
    k_copy_cols<<<(unsigned)((t + 255) / 256), 256, 0, st>>>(
        nst, nc, K.as<double>(), n_out, dcols.as<int>(), dK.as<double>() + col0, n_labels);
    FPP_CUDA(cudaGetLastError());
    FPP_CUDA(cudaStreamSynchronize(st));  // dcols / K are reused by the next structure
    col0 += nc;
  }
  if (nst && n_labels)
    FPP_CUDA(cudaMemcpy(kuf, dK.ptr, sizeof(double) * (size_t)nst * n_labels,
                        cudaMemcpyDeviceToHost));
  return FPP_OK;
}

extern "C" {

int fpp_kuf_batched(fpp_model *m, fpp_structure *const *structures, int32_t n_structures,
                    const int32_t *label_mask, const int32_t *atom_offsets,
                    const int32_t *atoms, double *kuf, int64_t n_labels, void *stream) {
  if (!m || (n_structures > 0 && (!structures || !label_mask)) || !kuf)
    return fail(FPP_ERR_INVALID, "null argument");
  if (n_structures < 0 || n_labels < 0) return fail(FPP_ERR_INVALID, "negative count");
  cudaStream_t st = (cudaStream_t)stream;
  if (m->args.kind != kB2)
    return kuf_stored_derivatives(m, structures, n_structures, label_mask, atom_offsets,
                                  atoms, kuf, n_labels, st);
  // label columns of each structure, stacked: [E] [F of the listed atoms] [S]
  std::vector<KufStruc> hs(n_structures);
  std::vector<int> fcol_off(n_structures + 1, 0);
  for (int k = 0; k < n_structures; k++) {
    if (!structures[k]) return fail(FPP_ERR_INVALID, "null structure");
    fcol_off[k + 1] = fcol_off[k] + structures[k]->st.noa;
  }
  std::vector<int> fcol(std::max(fcol_off[n_structures], 1), -1);
  int64_t col = 0;
  for (int k = 0; k < n_structures; k++) {
    fpp_structure *s = structures[k];
    const int noa = s->st.noa;
    KufStruc &q = hs[k];
    q.col_e = (label_mask[k] & 1) ? col++ : -1;
    if (label_mask[k] & 2) {
      const int b = atom_offsets ? atom_offsets[k] : 0;
      const int e = atom_offsets ? atom_offsets[k + 1] : noa;
      for (int t = b; t < e; t++) {
        const int a = atom_offsets ? atoms[t] : t;
        if (a < 0 || a >= noa) return fail(FPP_ERR_INVALID, "force atom index out of range");
        fcol[fcol_off[k] + a] = (int)col;
        col += 3;
      }
    }
    q.col_s = (label_mask[k] & 4) ? col : -1;
    if (label_mask[k] & 4) col += 6;
  }
  if (col != n_labels)
    return fail(FPP_ERR_INVALID, "n_labels (" + std::to_string(n_labels) +
                                     ") differs from the labels of the structures (" +
                                     std::to_string(col) + ")");
  const int nst = m->n_sparse_total;
  if (nst == 0 || n_labels == 0) {
    std::fill(kuf, kuf + (size_t)nst * n_labels, 0.0);
    return FPP_OK;
  }
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  // FP64 descriptors of every structure, queued without synchronization
  // (each structure keeps its own workspace), and the work list
  DevBuf dK, dfcol, dstruc, ditems;
  FPP_TRY(dK.reserve(sizeof(double) * (size_t)nst * n_labels));
  FPP_CUDA(cudaMemsetAsync(dK.ptr, 0, sizeof(double) * (size_t)nst * n_labels, st));
  FPP_TRY(dfcol.reserve(sizeof(int) * fcol.size()));
  FPP_CUDA(cudaMemcpyAsync(dfcol.ptr, fcol.data(), sizeof(int) * fcol.size(),
                           cudaMemcpyHostToDevice, st));
  std::vector<int2> items;
  for (int k = 0; k < n_structures; k++) {
    fpp_structure *s = structures[k];
    FPP_TRY(model_check(m, s));
    if (!(label_mask[k] & 7)) continue;
    StructureState &S = s->st;
    B2Args a = m->args;
    a.noa = S.noa;
    FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), false, st));
    KufStruc &q = hs[k];
    q.c64 = S.c64.as<double>();
    q.phat64 = S.phat64.as<double>();
    q.norm64 = S.norm64.as<double>();
    q.row_of_atom = s->row_of_atom.as<int>();
    q.species = S.species.as<int>();
    q.offset = S.nbr_offset.as<int>();
    q.nbr_j = S.nbr_j.as<int>();
    q.nbr_s = S.nbr_s.as<int>();
    q.rel = S.nbr_rel.as<dvec4>();
    q.force_col = dfcol.as<int>() + fcol_off[k];
    q.vol_inv = 1.0 / S.ci.volume;
    for (int i = 0; i < S.noa; i++) items.push_back(make_int2(k, i));
  }
  if (items.empty()) {
    FPP_CUDA(cudaMemcpy(kuf, dK.ptr, sizeof(double) * (size_t)nst * n_labels,
                        cudaMemcpyDeviceToHost));
    return FPP_OK;
  }
  FPP_TRY(dstruc.reserve(sizeof(KufStruc) * hs.size()));
  FPP_CUDA(cudaMemcpyAsync(dstruc.ptr, hs.data(), sizeof(KufStruc) * hs.size(),
                           cudaMemcpyHostToDevice, st));
  FPP_TRY(ditems.reserve(sizeof(int2) * items.size()));
  FPP_CUDA(cudaMemcpyAsync(ditems.ptr, items.data(), sizeof(int2) * items.size(),
                           cudaMemcpyHostToDevice, st));
  KufArgs ka;
  std::memset(&ka, 0, sizeof(ka));
  ka.a = m->args;
  ka.strucs = dstruc.as<KufStruc>();
  ka.items = ditems.as<int2>();
  ka.n_items = (int)items.size();
  for (int s = 0; s < m->n_species; s++) {
    ka.sp[s].dhat = m->sp[s].d_dhat.as<double>();
    ka.sp[s].norms = m->sp[s].d_norms.as<double>();
    ka.sp[s].n_sparse = m->sp[s].n_sparse;
    ka.sp[s].row0 = m->sp[s].sparse_offset;
  }
  ka.pair_tab = m->pair_tab.as<int>();
  ka.sig2 = m->sigma * m->sigma;
  ka.power = m->power;
  ka.ldp = round_up(m->n_d, 64);
  ka.kuf = dK.as<double>();
  ka.n_labels = n_labels;
  // tile shape: the cached choice for this device and descriptor, else the
  // autotuner's (timed on a prefix of the work list, then Kuf is cleared)
  int ks = 0, threads = 0;
  FPP_TRY(kuf_tiles(m, ka, (int)items.size(), st, &ks, &threads));
  FPP_CUDA(cudaMemsetAsync(dK.ptr, 0, sizeof(double) * (size_t)nst * n_labels, st));
  struct Events {  // released on every return path
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Events() {
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
  } ev;
  FPP_CUDA(cudaEventCreate(&ev.e0));
  FPP_CUDA(cudaEventCreate(&ev.e1));
  FPP_CUDA(cudaEventRecord(ev.e0, st));
  if (launch_kuf_adjoint(ka, ks, threads, (int)items.size(), 0, st) != 0)
    return fail(FPP_ERR_CUDA, "Kuf (adjoint) launch failed");
  FPP_CUDA(cudaEventRecord(ev.e1, st));
  m->kuf_ks = ks;
  m->kuf_threads = threads;
  m->kuf_items = (long long)items.size();
  FPP_CUDA(cudaMemcpyAsync(kuf, dK.ptr, sizeof(double) * (size_t)nst * n_labels,
                           cudaMemcpyDeviceToHost, st));
  FPP_CUDA(cudaStreamSynchronize(st));
  float ms = 0.f;
  FPP_CUDA(cudaEventElapsedTime(&ms, ev.e0, ev.e1));
  m->kuf_ms = ms;
  return FPP_OK;
}

int fpp_model_kuf_tiles(const fpp_model *m, int32_t *ks, int32_t *threads, float *kernel_ms,
                        int64_t *n_items) {
  if (!m || !ks || !threads) return fail(FPP_ERR_INVALID, "null argument");
  *ks = m->kuf_ks;
  *threads = m->kuf_threads;
  if (kernel_ms) *kernel_ms = m->kuf_ms;
  if (n_items) *n_items = m->kuf_items;
  return FPP_OK;
}

int fpp_envs_envs(fpp_model *m1, fpp_model *m2, double *kernel_mat, void *stream) {
  if (!m1 || !m2 || !kernel_mat) return fail(FPP_ERR_INVALID, "null argument");
  if (m1->n_d != m2->n_d || m1->n_species != m2->n_species)
    return fail(FPP_ERR_INVALID, "models differ in descriptor size or species");
  cudaStream_t st = (cudaStream_t)stream;
  cublasHandle_t h;
  FPP_TRY(get_cublas(m1, st, &h));
  const int n1 = m1->n_sparse_total, n2 = m2->n_sparse_total, nd = m1->n_d;
  DevBuf K, Z, a1, a2;
  FPP_TRY(K.reserve(sizeof(double) * std::max(1, n1) * std::max(1, n2)));
  FPP_CUDA(cudaMemsetAsync(K.ptr, 0, sizeof(double) * (size_t)n1 * n2, st));
  const double one = 1.0, zero = 0.0;
  for (int s = 0; s < m1->n_species; s++) {
    const int S1 = m1->sp[s].n_sparse, S2 = m2->sp[s].n_sparse;
    if (S1 == 0 || S2 == 0) continue;
    FPP_TRY(Z.reserve(sizeof(double) * (size_t)S1 * S2));
    // Z[i][j] = dhat1_i . dhat2_j  (row-major S1 x S2)
    FPP_CUBLAS(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, S2, S1, nd, &one,
                           m2->sp[s].d_dhat.as<double>(), nd, m1->sp[s].d_dhat.as<double>(), nd,
                           &zero, Z.as<double>(), S2));
    if (launch_envs_block(S1, S2, Z.as<double>(), S2, m1->sp[s].d_norms.as<double>(),
                          m2->sp[s].d_norms.as<double>(), m1->sigma * m1->sigma, m1->power,
                          K.as<double>() + (size_t)m1->sp[s].sparse_offset * n2 +
                              m2->sp[s].sparse_offset,
                          n2, st) != 0)
      return fail(FPP_ERR_CUDA, "envs_envs launch failed");
    FPP_CUDA(cudaStreamSynchronize(st));
  }
  FPP_CUDA(cudaStreamSynchronize(st));
  if ((size_t)n1 * n2)
    FPP_CUDA(cudaMemcpy(kernel_mat, K.ptr, sizeof(double) * (size_t)n1 * n2,
                        cudaMemcpyDeviceToHost));
  return FPP_OK;
}

int fpp_local_uncertainties(fpp_model *m, fpp_structure *s, const double *L_inv,
                            int32_t n, double *variances, void *stream) {
  FPP_TRY(model_check(m, s));
  if (!L_inv || !variances) return fail(FPP_ERR_INVALID, "null argument");
  if (n != m->n_sparse_total)
    return fail(FPP_ERR_INVALID, "L_inv size differs from the sparse set");
  cudaStream_t st = (cudaStream_t)stream;
  StructureState &S = s->st;
  const int noa = S.noa, nd = m->n_d, ldp = round_up(nd, 64);
  if (noa == 0) return FPP_OK;
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  B2Args a = m->args;
  a.noa = noa;
  FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), false, st));
  const int R = s->total_rows;
  DevBuf rown, K, Q, Ld, q;
  FPP_TRY(rown.reserve(sizeof(double) * std::max(1, R)));
  FPP_CUDA(cudaMemsetAsync(rown.ptr, 0, sizeof(double) * R, st));
  if (launch_gather_rows(noa, s->row_of_atom.as<int>(), S.norm64.as<double>(),
                         rown.as<double>(), st) != 0)
    return fail(FPP_ERR_CUDA, "gather launch failed");
  FPP_TRY(K.reserve(sizeof(double) * (size_t)std::max(1, R) * std::max(1, n)));
  FPP_CUDA(cudaMemsetAsync(K.ptr, 0, sizeof(double) * (size_t)R * n, st));
  // K[cluster][k] = k(cluster, sparse k): block-diagonal in the species
  for (int sp = 0; sp < m->n_species; sp++) {
    const int Ss = m->sp[sp].n_sparse, nsa = s->n_rows[sp];
    if (Ss == 0 || nsa == 0) continue;
    double *C = K.as<double>() + (size_t)s->row_off[sp] * n + m->sp[sp].sparse_offset;
    const double *Ph = S.phat64.as<double>() + (size_t)s->row_off[sp] * ldp;
    FPP_TRY(ozaki_dgemm_nt(nsa, Ss, nd, Ph, ldp, m->sp[sp].d_dhat.as<double>(), nd, C, n,
                           m->oz, st));
    if (launch_envs_block(nsa, Ss, C, n, rown.as<double>() + s->row_off[sp],
                          m->sp[sp].d_norms.as<double>(), m->sigma * m->sigma, m->power, C,
                          n, st) != 0)
      return fail(FPP_ERR_CUDA, "local kernel launch failed");
  }
  // Q = K L_inv^T; the explained variance of a cluster is |row of Q|^2
  FPP_TRY(Ld.reserve(sizeof(double) * (size_t)n * n));
  FPP_CUDA(cudaMemcpyAsync(Ld.ptr, L_inv, sizeof(double) * (size_t)n * n,
                           cudaMemcpyHostToDevice, st));
  FPP_TRY(Q.reserve(sizeof(double) * (size_t)std::max(1, R) * std::max(1, n)));
  bool lower = true;  // a Cholesky factor's inverse: its zeros are skipped
  for (int i = 0; i < n && lower; i++)
    for (int j = i + 1; j < n; j++)
      if (L_inv[(size_t)i * n + j] != 0.0) {
        lower = false;
        break;
      }
  FPP_TRY(ozaki_dgemm_nt(R, n, n, K.as<double>(), n, Ld.as<double>(), n, Q.as<double>(), n,
                         m->oz, st, lower));
  FPP_TRY(q.reserve(sizeof(double) * std::max(1, R)));
  if (launch_row_sq(R, n, Q.as<double>(), n, q.as<double>(), st) != 0)
    return fail(FPP_ERR_CUDA, "row-norm launch failed");
  std::vector<double> hq(R), hn(R);
  FPP_TRY(ozaki_check_status(m->oz, st));
  FPP_CUDA(cudaMemcpy(hq.data(), q.ptr, sizeof(double) * R, cudaMemcpyDeviceToHost));
  FPP_CUDA(cudaMemcpy(hn.data(), rown.ptr, sizeof(double) * R, cudaMemcpyDeviceToHost));
  // clusters in species order, atoms in structure order within a species
  const double sig2 = m->sigma * m->sigma;
  int out = 0;
  for (int sp = 0; sp < m->n_species; sp++)
    for (int r = 0; r < s->n_rows[sp]; r++) {
      const int row = s->row_off[sp] + r;
      variances[out++] = (hn[row] >= 1e-8 ? sig2 : 0.0) - hq[row];
    }
  return FPP_OK;
}

int fpp_predict_energy_uncertainty(fpp_model *m, fpp_structure *s, double *energy,
                                   double *energy_variance, double *local_variances,
                                   void *stream) {
  FPP_TRY(model_check(m, s));
  if (!energy && !energy_variance && !local_variances)
    return fail(FPP_ERR_INVALID, "no output requested");
  if (energy_variance && !m->has_R_inv)
    return fail(FPP_ERR_INVALID, "R_inv not set (fpp_model_set_R_inv)");
  if (local_variances && !m->has_L_inv)
    return fail(FPP_ERR_INVALID, "L_inv not set (fpp_model_set_L_inv)");
  cudaStream_t st = (cudaStream_t)stream;
  StructureState &S = s->st;
  const int noa = S.noa, nd = m->n_d, ldp = round_up(nd, 64), n = m->n_sparse_total;
  if (noa == 0) {
    if (energy) *energy = 0;
    if (energy_variance) *energy_variance = 0;
    return FPP_OK;
  }
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  B2Args a = m->args;
  a.noa = noa;
  FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), false, st));
  const int R = s->total_rows;
  cublasHandle_t h;
  FPP_TRY(get_cublas(m, st, &h));
  const double one = 1.0, zero = 0.0;
  DevBuf rown, K, kE, ones, al, y, Q, q;
  FPP_TRY(rown.reserve(sizeof(double) * std::max(1, R)));
  FPP_CUDA(cudaMemsetAsync(rown.ptr, 0, sizeof(double) * R, st));
  if (launch_gather_rows(noa, s->row_of_atom.as<int>(), S.norm64.as<double>(),
                         rown.as<double>(), st) != 0)
    return fail(FPP_ERR_CUDA, "gather launch failed");
  // per species block: K_s[c][k] = k(atom c, sparse k) (column-major S_s x
  // n_rows_s, at the block's row offset times S_s); only the energy column of
  // the kernel matrix is needed, so no force or stress columns are formed
  std::vector<size_t> koff(m->n_species + 1, 0);
  for (int sp = 0; sp < m->n_species; sp++)
    koff[sp + 1] = koff[sp] + (size_t)m->sp[sp].n_sparse * std::max(s->n_rows[sp], 0);
  FPP_TRY(K.reserve(sizeof(double) * std::max<size_t>(1, koff[m->n_species])));
  FPP_TRY(kE.reserve(sizeof(double) * std::max(1, n)));
  FPP_CUDA(cudaMemsetAsync(kE.ptr, 0, sizeof(double) * std::max(1, n), st));
  int max_rows = 1;
  for (int sp = 0; sp < m->n_species; sp++) max_rows = std::max(max_rows, s->n_rows[sp]);
  FPP_TRY(ones.reserve(sizeof(double) * max_rows));
  {
    std::vector<double> o(max_rows, 1.0);
    FPP_CUDA(cudaMemcpyAsync(ones.ptr, o.data(), sizeof(double) * max_rows,
                             cudaMemcpyHostToDevice, st));
    FPP_CUDA(cudaStreamSynchronize(st));
  }
  for (int sp = 0; sp < m->n_species; sp++) {
    const int Ss = m->sp[sp].n_sparse, nsa = s->n_rows[sp];
    if (Ss == 0 || nsa == 0) continue;
    double *C = K.as<double>() + koff[sp];
    const double *Ph = S.phat64.as<double>() + (size_t)s->row_off[sp] * ldp;
    // z[c][k] = phat_c . dhat_k on the tensor cores, FP64-accurate
    FPP_TRY(ozaki_dgemm_nt(nsa, Ss, nd, Ph, ldp, m->sp[sp].d_dhat.as<double>(), nd, C, Ss,
                           m->oz, st));
    if (launch_envs_block(nsa, Ss, C, Ss, rown.as<double>() + s->row_off[sp],
                          m->sp[sp].d_norms.as<double>(), m->sigma * m->sigma, m->power, C,
                          Ss, st) != 0)
      return fail(FPP_ERR_CUDA, "kernel block launch failed");
    // k_E = sum over the species' atoms of k(atom, sparse)
    FPP_CUBLAS(cublasDgemv(h, CUBLAS_OP_N, Ss, nsa, &one, C, Ss, ones.as<double>(), 1, &zero,
                           kE.as<double>() + m->sp[sp].sparse_offset, 1));
  }
  FPP_TRY(ozaki_check_status(m->oz, st));
  double e_mean = 0, e_var = 0;
  if (energy) {
    std::vector<double> h_al(std::max(n, 1), 0.0);
    for (auto &x : m->sp)
      for (int k = 0; k < x.n_sparse; k++) h_al[x.sparse_offset + k] = x.alpha[k];
    FPP_TRY(al.reserve(sizeof(double) * h_al.size()));
    FPP_CUDA(cudaMemcpyAsync(al.ptr, h_al.data(), sizeof(double) * h_al.size(),
                             cudaMemcpyHostToDevice, st));
    FPP_CUBLAS(cublasSetPointerMode(h, CUBLAS_POINTER_MODE_HOST));
    FPP_CUBLAS(cublasDdot(h, n, kE.as<double>(), 1, al.as<double>(), 1, &e_mean));
  }
  if (energy_variance) {
    // variance_efs[0] = |R_inv^T k_E|^2 (R_inv row-major: column-major R_inv^T)
    FPP_TRY(y.reserve(sizeof(double) * std::max(1, n)));
    FPP_CUBLAS(cublasDgemv(h, CUBLAS_OP_N, n, n, &one, m->R_inv.as<double>(), n,
                           kE.as<double>(), 1, &zero, y.as<double>(), 1));
    FPP_CUBLAS(cublasDdot(h, n, y.as<double>(), 1, y.as<double>(), 1, &e_var));
  }
  if (local_variances) {
    // q_c = |L_inv k_c|^2, species block by species block when L_inv is
    // block diagonal, else against the whole L_inv
    FPP_TRY(q.reserve(sizeof(double) * std::max(1, R)));
    FPP_CUDA(cudaMemsetAsync(q.ptr, 0, sizeof(double) * std::max(1, R), st));
    if (m->L_inv_species_blocks) {
      FPP_TRY(Q.reserve(sizeof(double) * std::max<size_t>(1, koff[m->n_species])));
      for (int sp = 0; sp < m->n_species; sp++) {
        const int Ss = m->sp[sp].n_sparse, nsa = s->n_rows[sp], off = m->sp[sp].sparse_offset;
        if (Ss == 0 || nsa == 0) continue;
        const double *Lb = m->L_inv.as<double>() + (size_t)off * n + off;
        // Q[c][i] = sum_k K[c][k] L_inv[i][k] on the tensor cores
        FPP_TRY(ozaki_dgemm_nt(nsa, Ss, Ss, K.as<double>() + koff[sp], Ss, Lb, n,
                               Q.as<double>() + koff[sp], Ss, m->oz, st, m->L_inv_lower));
        if (launch_row_sq(nsa, Ss, Q.as<double>() + koff[sp], Ss,
                          q.as<double>() + s->row_off[sp], st) != 0)
          return fail(FPP_ERR_CUDA, "row-norm launch failed");
      }
    } else {
      DevBuf Kf;
      FPP_TRY(Kf.reserve(sizeof(double) * (size_t)std::max(1, R) * std::max(1, n)));
      FPP_CUDA(cudaMemsetAsync(Kf.ptr, 0, sizeof(double) * (size_t)R * n, st));
      for (int sp = 0; sp < m->n_species; sp++) {
        const int Ss = m->sp[sp].n_sparse, nsa = s->n_rows[sp];
        if (Ss == 0 || nsa == 0) continue;
        FPP_CUDA(cudaMemcpy2DAsync(Kf.as<double>() + (size_t)s->row_off[sp] * n +
                                       m->sp[sp].sparse_offset,
                                   sizeof(double) * n, K.as<double>() + koff[sp],
                                   sizeof(double) * Ss, sizeof(double) * Ss, nsa,
                                   cudaMemcpyDeviceToDevice, st));
      }
      FPP_TRY(Q.reserve(sizeof(double) * (size_t)std::max(1, R) * std::max(1, n)));
      FPP_TRY(ozaki_dgemm_nt(R, n, n, Kf.as<double>(), n, m->L_inv.as<double>(), n,
                             Q.as<double>(), n, m->oz, st, m->L_inv_lower));
      if (launch_row_sq(R, n, Q.as<double>(), n, q.as<double>(), st) != 0)
        return fail(FPP_ERR_CUDA, "row-norm launch failed");
    }
    std::vector<double> hq(R), hn(R);
    FPP_TRY(ozaki_check_status(m->oz, st));
    FPP_CUDA(cudaMemcpy(hq.data(), q.ptr, sizeof(double) * R, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(hn.data(), rown.ptr, sizeof(double) * R, cudaMemcpyDeviceToHost));
    const double sig2 = m->sigma * m->sigma;
    std::vector<int> cnt(m->n_species, 0);
    for (int i = 0; i < noa; i++) {
      const int sp = S.species_host[i];
      const int row = s->row_off[sp] + cnt[sp]++;
      local_variances[i] = (hn[row] >= 1e-8 ? sig2 : 0.0) - hq[row];
    }
  }
  FPP_CUDA(cudaStreamSynchronize(st));
  if (energy) *energy = e_mean;
  if (energy_variance) *energy_variance = e_var;
  return FPP_OK;
}

int fpp_envs_struc(fpp_model *m, fpp_structure *s, double *kernel_mat, void *stream) {
  FPP_TRY(model_check(m, s));
  if (!kernel_mat) return fail(FPP_ERR_INVALID, "null output");
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf K;
  FPP_TRY(envs_struc_device(m, s, st, K));
  FPP_CUDA(cudaStreamSynchronize(st));
  const size_t n = (size_t)m->n_sparse_total * (1 + 3 * s->st.noa + 6);
  if (n) FPP_CUDA(cudaMemcpy(kernel_mat, K.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return FPP_OK;
}

int fpp_predict(fpp_model *m, fpp_structure *s, double *mean_efs, double *variance_efs,
                void *stream) {
  FPP_TRY(model_check(m, s));
  if (!mean_efs) return fail(FPP_ERR_INVALID, "null output");
  if (m->power < 2.0 - 1e-12) {
    // the reference's force-force kernel throws for power < 2 with a zero dot
    // product; the mean needs no such term, so only reject what diverges
    if (m->power < 1.0) return fail(FPP_ERR_UNSUPPORTED, "power < 1");
  }
  cudaStream_t st = (cudaStream_t)stream;
  StructureState &S = s->st;
  const int noa = S.noa, nd = m->n_d, ldp = round_up(nd, 64);
  const int n_out = 1 + 3 * noa + 6;
  const int nst = m->n_sparse_total;
  cublasHandle_t h;
  FPP_TRY(get_cublas(m, st, &h));
  const double one = 1.0, zero = 0.0;
  if (variance_efs) {
    if (!m->has_R_inv) return fail(FPP_ERR_INVALID, "R_inv not set (fpp_model_set_R_inv)");
    DevBuf K, alpha, mean, V, var;
    FPP_TRY(envs_struc_device(m, s, st, K));
    std::vector<double> al(std::max(nst, 1), 0.0);
    for (auto &x : m->sp)
      for (int k = 0; k < x.n_sparse; k++) al[x.sparse_offset + k] = x.alpha[k];
    FPP_TRY(alpha.reserve(sizeof(double) * al.size()));
    FPP_TRY(mean.reserve(sizeof(double) * n_out));
    FPP_TRY(V.reserve(sizeof(double) * (size_t)n_out * std::max(nst, 1)));
    FPP_TRY(var.reserve(sizeof(double) * n_out));
    FPP_CUDA(cudaMemcpyAsync(alpha.ptr, al.data(), sizeof(double) * al.size(), cudaMemcpyHostToDevice, st));
    FPP_CUBLAS(cublasDgemv(h, CUBLAS_OP_N, n_out, nst, &one, K.as<double>(), n_out,
                           alpha.as<double>(), 1, &zero, mean.as<double>(), 1));
    // V[o][i] = sum_k K[k][o] R_inv[k][i] (predict_SOR's R_inv^T K, row o per
    // label) on the tensor cores, FP64-accurate: operands K^T and R_inv^T
    DevBuf KT, RT;
    FPP_TRY(KT.reserve(sizeof(double) * (size_t)n_out * std::max(nst, 1)));
    FPP_TRY(RT.reserve(sizeof(double) * (size_t)std::max(nst, 1) * std::max(nst, 1)));
    if (launch_transpose(nst, n_out, K.as<double>(), n_out, KT.as<double>(), nst, st) != 0 ||
        launch_transpose(nst, nst, m->R_inv.as<double>(), nst, RT.as<double>(), nst, st) != 0)
      return fail(FPP_ERR_CUDA, "transpose launch failed");
    FPP_TRY(ozaki_dgemm_nt(n_out, nst, nst, KT.as<double>(), nst, RT.as<double>(), nst,
                           V.as<double>(), nst, m->oz, st, m->R_inv_upper));
    if (launch_row_sq(n_out, nst, V.as<double>(), nst, var.as<double>(), st) != 0)
      return fail(FPP_ERR_CUDA, "variance launch failed");
    FPP_TRY(ozaki_check_status(m->oz, st));
    FPP_CUDA(cudaMemcpy(mean_efs, mean.ptr, sizeof(double) * n_out, cudaMemcpyDeviceToHost));
    FPP_CUDA(cudaMemcpy(variance_efs, var.ptr, sizeof(double) * n_out, cudaMemcpyDeviceToHost));
    return FPP_OK;
  }
  // mean through the adjoint
  FPP_TRY(upload_pair_tab(m->pair_tab, m->pair_tab_host, st));
  B2Args a = m->args;
  a.noa = noa;
  FPP_TRY(forward64(s, a, m->pair_tab.as<int>(), false, st));
  double *phat = S.phat64.as<double>();
  DevBuf rown, E, zc, Z, G, DT;
  FPP_TRY(rown.reserve(sizeof(double) * std::max(1, s->total_rows)));
  FPP_TRY(E.reserve(sizeof(double) * std::max(1, s->total_rows)));
  FPP_TRY(zc.reserve(sizeof(double) * std::max(1, s->total_rows)));
  FPP_CUDA(cudaMemsetAsync(rown.ptr, 0, sizeof(double) * s->total_rows, st));
  FPP_CUDA(cudaMemsetAsync(E.ptr, 0, sizeof(double) * s->total_rows, st));
  FPP_CUDA(cudaMemsetAsync(zc.ptr, 0, sizeof(double) * s->total_rows, st));
  FPP_CUDA(cudaMemsetAsync(S.w64.ptr, 0, sizeof(double) * (size_t)s->total_rows * ldp, st));
  if (launch_gather_rows(noa, s->row_of_atom.as<int>(), S.norm64.as<double>(),
                         rown.as<double>(), st) != 0)
    return fail(FPP_ERR_CUDA, "gather launch failed");
  FPP_TRY(G.reserve(sizeof(double) * (size_t)s->total_rows * ldp));
  for (int sp = 0; sp < m->n_species; sp++) {
    const int Ss = m->sp[sp].n_sparse, nsa = s->n_rows[sp];
    if (Ss == 0 || nsa == 0) continue;
    const size_t r0 = s->row_off[sp];
    FPP_TRY(Z.reserve(sizeof(double) * (size_t)nsa * Ss));
    const double *Dh = m->sp[sp].d_dhat.as<double>();
    // Z[i][k] = phat_i . dhat_k (tensor cores, FP64-accurate)
    FPP_TRY(ozaki_dgemm_nt(nsa, Ss, nd, phat + r0 * ldp, ldp, Dh, nd, Z.as<double>(), Ss,
                           m->oz, st));
    if (launch_kernel_c(nsa, Ss, Z.as<double>(), Ss, m->sp[sp].d_alpha.as<double>(),
                        rown.as<double>() + r0, m->sigma * m->sigma, m->power,
                        E.as<double>() + r0, zc.as<double>() + r0, st) != 0)
      return fail(FPP_ERR_CUDA, "kernel-form launch failed");
    // G[i][d] = sum_k C[i][k] dhat_k[d] = (C Dhat^T^T): B operand Dhat^T (nd x S)
    FPP_TRY(DT.reserve(sizeof(double) * (size_t)nd * Ss));
    if (launch_transpose(Ss, nd, Dh, nd, DT.as<double>(), Ss, st) != 0)
      return fail(FPP_ERR_CUDA, "transpose launch failed");
    FPP_TRY(ozaki_dgemm_nt(nsa, nd, Ss, Z.as<double>(), Ss, DT.as<double>(), Ss,
                           G.as<double>() + r0 * ldp, ldp, m->oz, st));
    if (launch_kernel_w(nsa, nd, G.as<double>() + r0 * ldp, ldp, phat + r0 * ldp, ldp,
                        zc.as<double>() + r0, rown.as<double>() + r0,
                        S.w64.as<double>() + r0 * ldp, ldp, st) != 0)
      return fail(FPP_ERR_CUDA, "kernel-form launch failed");
    FPP_CUDA(cudaStreamSynchronize(st));  // Z is reused by the next species
  }
  FPP_TRY(ozaki_check_status(m->oz, st));
  AdjArgs g;
  std::memset(&g, 0, sizeof(g));
  g.mode = kWGiven;
  g.ldp = ldp;
  g.w_given = S.w64.as<double>();
  g.e_given = E.as<double>();
  FPP_TRY(adjoint_buffers(S, sizeof(double), u_row_stride(a)));
  FPP_CUDA(cudaMemsetAsync(S.status.ptr, 0, sizeof(DeviceStatus), st));
  if (launch_b2_adjoint<double>(a, g, neigh_of(S), S.species.as<int>(),
                                s->row_of_atom.as<int>(), m->pair_tab.as<int>(),
                                S.c64.as<double>(), S.norm64.as<double>(),
                                S.atom_e.as<double>(), S.pair_f.as<double>(),
                                S.forces.as<double>(), S.atom_vir.as<double>(),
                                S.reduce_out.as<double>(), true, S.u.as<double>(),
                                S.n_pairs, S.nbr_i.as<int>(), st) != 0)
    return fail(FPP_ERR_CUDA, "adjoint (FP64) launch failed");
  double e, stress[6];
  std::vector<double> F(3 * (size_t)noa);
  FPP_TRY(finish_outputs(s, st, &e, F.data(), stress, nullptr, 0));
  mean_efs[0] = e;
  for (size_t k = 0; k < F.size(); k++) mean_efs[1 + k] = F[k];
  for (int k = 0; k < 6; k++) mean_efs[1 + 3 * noa + k] = stress[k];
  return FPP_OK;
}

}  // extern "C"
